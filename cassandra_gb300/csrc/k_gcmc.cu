// k_gcmc.cu -- grand-canonical Monte Carlo on the device, boxes in lockstep.
//
// One CTA runs one box's chain for the whole call (gcmc_driver.f90:30-102):
// Translate, Rotate, CBMC Insertion (move_insert.f90), CBMC Deletion
// (move_delete.f90) and CBMC regrowth (Cut_N_Grow, move_regrow.f90).  The
// box is a fixed set of molecule records (the box's molecules and its share of
// free slots, in slot order) with a live flag each; atoms, records and COMs
// live in shared memory.  Thread 0 owns the lfsr258 stream and every serial
// decision, in the reference's order; the trial energies of a CBMC stage and
// the molecule energies are evaluated by the whole block, warps over
// (trial, atom-range) items with a fixed-order sum per trial.  The per-trial
// geometry and intramolecular energies of a stage run one trial per lane of
// warp 0.  FP64 kernel: the reference arithmetic; mixed kernel: FP32 pair
// energies against the box, everything else FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cass_cbmc.cuh"
#include "cass_ctx.h"

namespace cassgpu {

constexpr int kGcThreads = 256;
constexpr int kGcWarps = kGcThreads / 32;
constexpr int kGcMaxSpecies = 8;
constexpr int kGcItems = 256;  // (trial, atom range) items of one batch
constexpr size_t kGcSmemLimit = 200 * 1024;

struct GcSpecies {
  int natoms, linear;
  double mass[kMaxAtoms];
};

struct GcArgs {
  WidomSpecies S;  // growth tables of the exchanged species
  int is_ex, nspecies;
  GcSpecies sp[kGcMaxSpecies];
  long long nsteps;
  double cut_t, cut_r, cut_i, cut_d, cut_g;
  uint64_t seed;
  const double* lib;  // FP64 fragment libraries of the exchanged species
  int nfbond;
  int fb_a[kMaxFrags], fb_b[kMaxFrags];
  double prob_del1[kMaxFrags];
  SpeciesPools P;
};

struct GcBox {
  BoxDev b;
  int natoms, nrec, npool, ibox1;
  double4_32a* xyzq;  // [natoms] x, y, z, q (in / out)
  const int* atype;   // [natoms]
  int4* rec;          // [nrec] slot, species, first atom, live (live written at the end)
  const int* pool;    // [npool] free records, ascending; insertion takes the last
  const double* max_disp;  // [nspecies]
  const double* max_rot;
  double mu, log_lambda3;
  double rcut3, rcut9;    // rcut_vdw^3 and (rcut_vdw^3)^3 of Compute_LR_Correction
  double nb0[kMaxTypes];  // atoms per type at the start
  CassEnergy* energy;
  CassGCMCResult* res;
  int* status;  // 0 ok, 1 overlapping molecule before a move, 2 no free slot
};

// the molecule being built / moved and one stage of trials (shared memory)
struct GrowState {
  double r[3 * kMaxAtoms];
  double com[3];
  unsigned exist;
  int rec, is, na;
  // trial batch
  double trial[kMaxKappa][3 * kMaxAtoms];
  int tids[kMaxAtoms], ntid;
  double e[kMaxKappa];
  int ov[kMaxKappa];
  double part[kGcItems];
  int povl[kGcItems];
  // growth bookkeeping
  double ln_pseq, ln_pbias, e_prev;
  int order[kMaxFrags], norder;
  unsigned placed;
  int flag;  // 1: cbmc overlap
  double draws[3 * kMaxKappa];
  // fragment placement
  double cfg[3 * kMaxAtoms], hg[9];
  int anc_i, anc_c;
  double theta0;
  double dn[kMaxKappa], dd[kMaxKappa];
  int dov[kMaxKappa];
  unsigned newex, combined, idmask;
  // regrowth
  int f_live, f_dead;
};

struct GcView {
  const BoxDev* b;
  const PairTable* T;
  double *sx, *sy, *sz;
  int *stype, *srec;
  int *rlive, *rsp, *roff;
  double* com;
  float4* s32;
  int natoms, nrec;
};

// ---------------------------------------------------------------------------
// block-wide energies of ntr configurations of the atoms gs.tids (taken from
// gs.trial[t]) against every live atom of records other than skip_rec

template <bool MIXED>
__device__ void batch_energies(const GcView& V, GrowState& gs, int ntr, int skip_rec, bool cbmc,
                               const int* ttype) {
  const BoxDev& b = *V.b;
  const int nch = max(1, kGcWarps / ntr);
  const int items = ntr * nch;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = w; it < items; it += kGcWarps) {
    const int t = it / nch, ch = it % nch;
    const int j0 = (int)((long long)V.natoms * ch / nch), j1 = (int)((long long)V.natoms * (ch + 1) / nch);
    double acc = 0.0;
    KahanF kacc;
    int ov = 0;
    for (int j = j0 + lane; j < j1; j += 32) {
      const int rj = V.srec[j];
      if (rj == skip_rec || !V.rlive[rj]) continue;
      const int tj = V.stype[j];
      for (int k = 0; k < gs.ntid; ++k) {
        const int a = gs.tids[k];
        const int ta = ttype[a];
        if (MIXED) {
          const float4 pj = V.s32[j];
          const float dx = fold((float)gs.trial[t][3 * a] - pj.x, b.hLf[0], b.Lf[0]);
          const float dy = fold((float)gs.trial[t][3 * a + 1] - pj.y, b.hLf[1], b.Lf[1]);
          const float dz = fold((float)gs.trial[t][3 * a + 2] - pj.z, b.hLf[2], b.Lf[2]);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          if (r2 < (float)b.rcut_lowsq) {
            ov = 1;
            continue;
          }
          const float rc2 = cbmc ? (float)b.rcut_cbmcsq : (float)b.rcut_vdwsq;
          if (r2 <= rc2 && ta >= 0 && tj >= 0) {
            const int kk = pidx(ta, tj, V.T->ntypes);
            kacc.add(lj_pair_f(V.T->epsf[kk], V.T->sig2f[kk], r2));
          }
        } else {
          const double dx = fold(gs.trial[t][3 * a] - V.sx[j], b.hL[0], b.L[0]);
          const double dy = fold(gs.trial[t][3 * a + 1] - V.sy[j], b.hL[1], b.L[1]);
          const double dz = fold(gs.trial[t][3 * a + 2] - V.sz[j], b.hL[2], b.L[2]);
          const double r2 = dx * dx + dy * dy + dz * dz;
          if (r2 < b.rcut_lowsq) {
            ov = 1;
            continue;
          }
          if (cutoff_mask(b, r2, cbmc) & 1) acc += vdw_pair(*V.T, b, ta, tj, r2, 1.0);
        }
      }
    }
    if (MIXED) acc = kacc.value();
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    ov = __any_sync(0xffffffffu, ov);
    if (lane == 0) {
      gs.part[it] = acc;
      gs.povl[it] = ov;
    }
  }
  __syncthreads();
  if (threadIdx.x < ntr) {
    double e = 0.0;
    int o = 0;
    for (int ch = 0; ch < nch; ++ch) {
      e += gs.part[threadIdx.x * nch + ch];
      o |= gs.povl[threadIdx.x * nch + ch];
    }
    gs.e[threadIdx.x] = o ? 0.0 : e;
    gs.ov[threadIdx.x] = o;
  }
  __syncthreads();
}

// the k-th (1-based) live molecule of species is in record order; all threads
__device__ int nth_live(const GcView& V, int is, int k, int* scratch) {
  const int per = (V.nrec + kGcThreads - 1) / kGcThreads;
  const int r0 = threadIdx.x * per, r1 = min(V.nrec, r0 + per);
  int cnt = 0;
  for (int r = r0; r < r1; ++r) cnt += (V.rlive[r] && V.rsp[r] == is);
  scratch[threadIdx.x] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0, found = -1;
    for (int t = 0; t < kGcThreads && found < 0; ++t) {
      if (acc + scratch[t] >= k) {
        int need = k - acc;
        const int a0 = t * per, a1 = min(V.nrec, a0 + per);
        for (int r = a0; r < a1; ++r)
          if (V.rlive[r] && V.rsp[r] == is && --need == 0) {
            found = r;
            break;
          }
      }
      acc += scratch[t];
    }
    scratch[kGcThreads] = found;
  }
  __syncthreads();
  const int r = scratch[kGcThreads];
  __syncthreads();
  return r;
}

__device__ __forceinline__ bool gc_accept(double ln_pacc, Lfsr& rng) {
  if (ln_pacc <= 0.0) return true;
  if (ln_pacc < kMAX_KBT) return rng.next() <= exp(-ln_pacc);
  return false;
}

// Fragment_Order (fragment_growth.f90:1317-1446) on thread 0
__device__ void gc_fragment_order(const WidomSpecies& S, GrowState& gs, unsigned live, Lfsr& rng) {
  const int f0 = gs.order[0];
  int hang[kMaxFrags];
  int nh = 0;
  for (int k = 0; k < S.frag_nconnect[f0]; ++k) {
    const int f = S.frag_connect[f0][k];
    if (!((live >> f) & 1u)) hang[nh++] = f;
  }
  while (nh > 0) {
    double prob[kMaxFrags], cum[kMaxFrags];
    for (int k = 0; k < nh; ++k) {
      prob[k] = (double)(S.frag_natoms[hang[k]] - 2);
      cum[k] = (k == 0 ? 0.0 : cum[k - 1]) + prob[k];
    }
    const double tot = cum[nh - 1];
    for (int k = 0; k < nh; ++k) {
      prob[k] = prob[k] / tot;
      cum[k] = cum[k] / tot;
    }
    const double u = rng.next();
    int k = 0;
    while (k < nh && !(u < cum[k])) ++k;
    if (k >= nh) k = nh - 1;
    const int f = hang[k];
    gs.ln_pseq = gs.ln_pseq + log(prob[k]);
    gs.order[gs.norder++] = f;
    live |= 1u << f;
    for (int q = k; q + 1 < nh; ++q) hang[q] = hang[q + 1];
    --nh;
    for (int q = 0; q < S.frag_nconnect[f]; ++q) {
      const int g = S.frag_connect[f][q];
      if (!((live >> g) & 1u) && nh < kMaxFrags) hang[nh++] = g;
    }
  }
}

// Cut_Regrow (fragment_growth.f90:1118-1312): the fragments in gs.order are
// removed except the two anchors of the cut bond; thread 0
__device__ void gc_cut(const WidomSpecies& S, GrowState& gs) {
  gs.exist = (1u << S.natoms) - 1u;
  gs.placed = (1u << S.nfrag) - 1u;
  for (int k = 0; k < gs.norder; ++k) {
    const int f = gs.order[k];
    gs.placed &= ~(1u << f);
    for (int j = 0; j < S.frag_natoms[f]; ++j) gs.exist &= ~(1u << S.frag_atoms[f][j]);
  }
  gs.exist |= 1u << S.frag_atoms[gs.f_live][0];
  gs.exist |= 1u << S.frag_atoms[gs.f_dead][0];
  gs.ln_pbias = 0.0;
  gs.flag = 0;
}

// Fragment_Placement (fragment_growth.f90:1449-2132) for gs.order[first..];
// all threads; returns the cbmc overlap flag
template <bool MIXED>
__device__ bool gc_place_fragments(const GcArgs& A, const GcView& V, GrowState& gs, int first, bool del, Lfsr& rng,
                                   const double* lib) {
  const WidomSpecies& S = A.S;
  const SpeciesDevHdr& H = A.P.hdr[S.is0];
  const BoxDev& b = *V.b;
  const int kd = S.kappa_dih;
  for (int oi = first; oi < gs.norder; ++oi) {
    if (threadIdx.x == 0) {
      const int f = gs.order[oi];
      const int nf = S.frag_natoms[f];
      const unsigned grown = gs.exist;
      for (int i = 0; i < 3 * kMaxAtoms; ++i) gs.cfg[i] = 0.0;
      if (del) {
        for (int j = 0; j < nf; ++j) {
          const int a = S.frag_atoms[f][j];
          gs.exist |= 1u << a;
          for (int d = 0; d < 3; ++d) gs.cfg[3 * a + d] = gs.r[3 * a + d];
        }
      } else {
        const int nconf = S.nconfig[f];
        int cf = (int)(rng.next() * nconf);
        cf = (int)(rng.next() * nconf);  // the duplicated draw of fragment_growth.f90:1578,1584
        if (cf >= nconf) cf = nconf - 1;
        const double* L = lib + S.lib_off[f] + (size_t)cf * nf * 3;
        for (int j = 0; j < nf; ++j) {
          const int a = S.frag_atoms[f][j];
          gs.exist |= 1u << a;
          for (int d = 0; d < 3; ++d) gs.cfg[3 * a + d] = L[3 * j + d];
        }
      }
      gs.combined = gs.exist;
      gs.newex = gs.combined & ~grown;
      int fc = -1;
      for (int q = 0; q < S.frag_nconnect[f]; ++q) {
        const int g = S.frag_connect[f][q];
        if ((gs.placed >> g) & 1u) {
          fc = g;
          break;
        }
      }
      gs.flag = fc < 0 ? 1 : 0;
      if (fc >= 0) {
        const int anc_i = S.frag_atoms[f][0], anc_c = S.frag_atoms[fc][0];
        gs.anc_i = anc_i;
        gs.anc_c = anc_c;
        gs.ntid = 0;
        gs.idmask = 0u;
        for (int j = 0; j < nf; ++j) {
          const int a = S.frag_atoms[f][j];
          if (a != anc_i && a != anc_c) {
            gs.tids[gs.ntid++] = a;
            gs.idmask |= 1u << a;
          }
        }
        const int atom_ifrag = gs.ntid > 0 ? gs.tids[0] : S.frag_atoms[f][nf - 1];
        int atom_fc = S.frag_atoms[fc][S.frag_natoms[fc] - 1];
        for (int j = 0; j < S.frag_natoms[fc]; ++j) {
          const int a = S.frag_atoms[fc][j];
          if (a != anc_i && a != anc_c) {
            atom_fc = a;
            break;
          }
        }
        double v1[3], v2[3], al_i[9], hg_i[9], al_c[9], hg_c[9];
        for (int d = 0; d < 3; ++d) {
          v1[d] = gs.cfg[3 * anc_i + d] - gs.cfg[3 * anc_c + d];
          v2[d] = gs.cfg[3 * atom_ifrag + d] - gs.cfg[3 * anc_c + d];
        }
        aligner_hanger(v1, v2, al_i, hg_i);
        if (!del) {
          for (int d = 0; d < 3; ++d) {
            v1[d] = gs.r[3 * anc_i + d] - gs.r[3 * anc_c + d];
            v2[d] = gs.r[3 * atom_fc + d] - gs.r[3 * anc_c + d];
          }
          aligner_hanger(v1, v2, al_c, hg_c);
        }
        const double tx = gs.cfg[3 * anc_c], ty = gs.cfg[3 * anc_c + 1], tz = gs.cfg[3 * anc_c + 2];
        for (int a = 0; a < S.natoms; ++a) {
          gs.cfg[3 * a] -= tx;
          gs.cfg[3 * a + 1] -= ty;
          gs.cfg[3 * a + 2] -= tz;
        }
        for (int j = 0; j < nf; ++j) {
          const int a = S.frag_atoms[f][j];
          const double x = gs.cfg[3 * a], y = gs.cfg[3 * a + 1], z = gs.cfg[3 * a + 2];
          gs.cfg[3 * a] = x * al_i[0] + y * al_i[1] + z * al_i[2];
          gs.cfg[3 * a + 1] = x * al_i[3] + y * al_i[4] + z * al_i[5];
          gs.cfg[3 * a + 2] = x * al_i[6] + y * al_i[7] + z * al_i[8];
        }
        if (del) {
          gs.theta0 = 0.0;
          for (int i = 0; i < 9; ++i) gs.hg[i] = hg_i[i];
        } else {
          gs.theta0 = kTWOPI * rng.next();
          for (int i = 0; i < 9; ++i) gs.hg[i] = hg_c[i];
        }
      }
    }
    __syncthreads();
    if (gs.flag) return true;
    // trial geometry, intramolecular and dihedral energies: trial ii on lane ii of warp 0
    if (threadIdx.x < kd) {
      const int ii = threadIdx.x;
      double theta = gs.theta0;
      for (int k = 0; k < ii; ++k) theta = theta + kTWOPI / (double)kd;
      const double cth = cos(theta), sth = sin(theta);
      double r[3 * kMaxAtoms];
      for (int i = 0; i < 3 * S.natoms; ++i) r[i] = gs.r[i];
      const int f = gs.order[oi];
      for (int j = 0; j < S.frag_natoms[f]; ++j) {
        const int a = S.frag_atoms[f][j];
        if (a == gs.anc_i || a == gs.anc_c) continue;
        const double x = gs.cfg[3 * a], y = gs.cfg[3 * a + 1], z = gs.cfg[3 * a + 2];
        const double yr = cth * y + sth * z, zr = -sth * y + cth * z;
        r[3 * a] = (x * gs.hg[0] + yr * gs.hg[1] + zr * gs.hg[2]) + gs.r[3 * gs.anc_c];
        r[3 * a + 1] = (x * gs.hg[3] + yr * gs.hg[4] + zr * gs.hg[5]) + gs.r[3 * gs.anc_c + 1];
        r[3 * a + 2] = (x * gs.hg[6] + yr * gs.hg[7] + zr * gs.hg[8]) + gs.r[3 * gs.anc_c + 2];
      }
      for (int i = 0; i < 3 * S.natoms; ++i) gs.trial[ii][i] = r[i];
      unsigned ex = gs.combined & ~gs.idmask;
      double niv = 0.0, niq = 0.0, noq = 0.0;
      bool ov = false;
      for (int k = 0; k < gs.ntid && !ov; ++k) {
        ex |= 1u << gs.tids[k];
        double eiv, eiq, eoq;
        ov = atom_intra(H, A.P, b, *V.T, gs.tids[k], r, ex, eiv, eiq, eoq);
        niv += eiv;
        niq += eiq;
        noq += eoq;
      }
      gs.dov[ii] = ov ? 1 : 0;
      gs.dd[ii] = 0.0;
      gs.dn[ii] = niv + niq + noq;  // completed with the inter and dihedral energies below
      if (!ov) gs.dd[ii] = dihedral_masked(H, A.P, r, gs.combined);
    }
    __syncthreads();
    // inter energies of the new atoms (Compute_Molecule_Nonbond_Inter_Energy with new_exist)
    if (threadIdx.x == 0) {
      gs.ntid = 0;
      for (int a = 0; a < S.natoms; ++a)
        if ((gs.newex >> a) & 1u) gs.tids[gs.ntid++] = a;
    }
    __syncthreads();
    batch_energies<MIXED>(V, gs, kd, gs.rec, true, S.type);
    if (threadIdx.x == 0) {
      const double beta = b.beta;
      double w[kMaxKappa];
      bool all_ov = true;
      for (int ii = 0; ii < kd; ++ii) {
        const bool intra_ov = gs.dov[ii] != 0;
        bool ov = intra_ov || gs.ov[ii];
        double wi = 0.0;
        if (!ov) {
          gs.dn[ii] = gs.dd[ii] + gs.dn[ii] + gs.e[ii] - gs.e_prev;
          const double nk = beta * gs.dn[ii];
          if (nk >= kMAX_KBT) ov = true;
          else wi = exp(-nk);
        }
        if (ov) gs.dov[ii] = 1;
        else all_ov = false;
        // an intramolecular overlap keeps the running sum (fragment_growth.f90:1955-1962)
        w[ii] = (intra_ov ? 0.0 : wi) + (ii > 0 ? w[ii - 1] : 0.0);
      }
      int tr = 0;
      if (all_ov) {
        gs.flag = 1;
      } else if (!del) {
        const double pp = rng.next() * w[kd - 1];
        while (tr < kd && !(pp < w[tr])) ++tr;
        if (tr == kd) gs.flag = 1;
      }
      if (!gs.flag) {
        gs.ln_pbias = gs.ln_pbias - beta * gs.dn[tr] - log(w[kd - 1]);
        const int f = gs.order[oi];
        for (int j = 0; j < S.frag_natoms[f]; ++j) {
          const int a = S.frag_atoms[f][j];
          if (a != gs.anc_i && a != gs.anc_c)
            for (int d = 0; d < 3; ++d) gs.r[3 * a + d] = gs.trial[tr][3 * a + d];
        }
        gs.e_prev = gs.dd[tr];
        gs.placed |= 1u << f;
        gs.exist = gs.combined;
      }
    }
    __syncthreads();
    if (gs.flag) return true;
  }
  return false;
}

// Build_Molecule (fragment_growth.f90:72-707) for record gs.rec; all threads
template <bool MIXED>
__device__ bool gc_build(const GcArgs& A, const GcView& V, GrowState& gs, bool del, Lfsr& rng) {
  const WidomSpecies& S = A.S;
  const SpeciesDevHdr& H = A.P.hdr[S.is0];
  const BoxDev& b = *V.b;
  const int ki = S.kappa_ins;
  if (threadIdx.x == 0) {
    gs.ln_pbias = 0.0;
    gs.exist = 0u;
    gs.flag = 0;
    const double u = rng.next();
    int fstart = 0;
    while (fstart < S.nfrag && !(u < S.cum_prob_ins[fstart])) ++fstart;
    if (fstart >= S.nfrag) fstart = S.nfrag - 1;
    gs.ln_pseq = S.ln_prob_ins[fstart];
    gs.order[0] = fstart;
    gs.norder = 1;
    if (S.nfrag > 1) gc_fragment_order(S, gs, 1u << fstart, rng);
    const int nfa = S.frag_natoms[fstart];
    if (!del) {
      const int nconf = S.nconfig[fstart];
      int conf = (int)(rng.next() * nconf);
      if (conf >= nconf) conf = nconf - 1;
      const double* L0 = A.lib + S.lib_off[fstart] + (size_t)conf * nfa * 3;
      for (int i = 0; i < nfa; ++i)
        for (int d = 0; d < 3; ++d) gs.r[3 * S.frag_atoms[fstart][i] + d] = L0[3 * i + d];
    }
    gs.ntid = nfa;
    for (int i = 0; i < nfa; ++i) {
      gs.tids[i] = S.frag_atoms[fstart][i];
      gs.exist |= 1u << gs.tids[i];
    }
    get_com(S, gs.r, gs.exist, gs.com);
    if (!del) {
      const double theta = acos(1.0 - 2.0 * rng.next());
      const double phi = (1.0 - 2.0 * rng.next()) * kPI;
      const double psi = (1.0 - 2.0 * rng.next()) * kPI;
      const double r11 = cos(psi) * cos(phi) - cos(theta) * sin(phi) * sin(psi);
      const double r12 = cos(psi) * sin(phi) + cos(theta) * cos(phi) * sin(psi);
      const double r13 = sin(psi) * sin(theta);
      const double r21 = -sin(psi) * cos(phi) - cos(theta) * sin(phi) * cos(psi);
      const double r22 = -sin(psi) * sin(phi) + cos(theta) * cos(phi) * cos(psi);
      const double r23 = cos(psi) * sin(theta);
      const double r31 = sin(theta) * sin(phi);
      const double r32 = -sin(theta) * cos(phi);
      const double r33 = cos(theta);
      for (int i = 0; i < nfa; ++i) {
        const int a = gs.tids[i];
        const double x = gs.r[3 * a] - gs.com[0], y = gs.r[3 * a + 1] - gs.com[1], z = gs.r[3 * a + 2] - gs.com[2];
        gs.r[3 * a] = (r11 * x + r12 * y + r13 * z) + gs.com[0];
        gs.r[3 * a + 1] = (r21 * x + r22 * y + r23 * z) + gs.com[1];
        gs.r[3 * a + 2] = (r31 * x + r32 * y + r33 * z) + gs.com[2];
      }
    }
    for (int it = 0; it < ki; ++it) {
      if (del && it == 0) {
        gs.draws[0] = gs.com[0];
        gs.draws[1] = gs.com[1];
        gs.draws[2] = gs.com[2];
      } else {
        gs.draws[3 * it] = (0.5 - rng.next()) * b.L[0];
        gs.draws[3 * it + 1] = (0.5 - rng.next()) * b.L[1];
        gs.draws[3 * it + 2] = (0.5 - rng.next()) * b.L[2];
      }
    }
  }
  __syncthreads();
  // trial positions: rtrial(0) - COM + anchor
  for (int it = threadIdx.x; it < ki; it += blockDim.x)
    for (int k = 0; k < gs.ntid; ++k) {
      const int a = gs.tids[k];
      for (int d = 0; d < 3; ++d) gs.trial[it][3 * a + d] = gs.r[3 * a + d] - gs.com[d] + gs.draws[3 * it + d];
    }
  __syncthreads();
  batch_energies<MIXED>(V, gs, ki, gs.rec, true, S.type);
  if (threadIdx.x == 0) {
    const double beta = b.beta;
    double w[kMaxKappa];
    bool all_ov = true;
    for (int it = 0; it < ki; ++it) {
      double wi = 0.0;
      bool ov = gs.ov[it] != 0;
      if (!ov) {
        const double nk = beta * gs.e[it];
        if (nk >= kMAX_KBT) ov = true;
        else wi = exp(-nk);
      }
      gs.ov[it] = ov ? 1 : 0;
      if (!ov) all_ov = false;
      w[it] = wi + (it > 0 ? w[it - 1] : 0.0);
    }
    int sel = 0;
    if (all_ov) {
      gs.flag = 1;
    } else if (!del) {
      const double rn = rng.next() * w[ki - 1];
      while (sel < ki && !(rn < w[sel])) ++sel;
      if (sel == ki) gs.flag = 1;
    }
    if (!gs.flag) {
      gs.ln_pbias = gs.ln_pbias - beta * gs.e[sel] - log(w[ki - 1]);
      for (int k = 0; k < gs.ntid; ++k) {
        const int a = gs.tids[k];
        for (int d = 0; d < 3; ++d) gs.r[3 * a + d] = gs.trial[sel][3 * a + d];
      }
      for (int d = 0; d < 3; ++d) gs.com[d] = gs.draws[3 * sel + d];
      gs.e_prev = dihedral_masked(H, A.P, gs.r, gs.exist);
      gs.placed = 1u << gs.order[0];
    }
  }
  __syncthreads();
  if (gs.flag) return true;
  if (gc_place_fragments<MIXED>(A, V, gs, 1, del, rng, A.lib)) return true;
  if (threadIdx.x == 0 && gs.norder > 1) get_com(S, gs.r, gs.exist, gs.com);
  __syncthreads();
  return false;
}

// energies of the whole molecule gs.r (record gs.rec): inter (full cutoffs,
// block-wide) plus intra and bonded (thread 0); results in out[0..8]:
// ev, eq, eb, ea, ed, ei, eiv, eiq, overlap flags (inter, intra)
template <bool MIXED>
__device__ void gc_mol_energies(const GcArgs& A, const GcView& V, GrowState& gs, const int* ttype, double* out,
                                int* ovs, bool with_intra = true) {
  if (threadIdx.x == 0) {
    gs.ntid = gs.na;
    for (int a = 0; a < gs.na; ++a) {
      gs.tids[a] = a;
      for (int d = 0; d < 3; ++d) gs.trial[0][3 * a + d] = gs.r[3 * a + d];
    }
  }
  __syncthreads();
  batch_energies<MIXED>(V, gs, 1, gs.rec, false, ttype);
  if (threadIdx.x == 0) {
    IntraOut io{0, 0, 0, 0, 0, 0, 0, false};
    if (with_intra) io = molecule_intra(A.P, gs.is, *V.b, *V.T, gs.r);
    out[0] = gs.e[0];
    out[1] = io.pqq;  // the periodic part of the intramolecular Coulomb sum
    out[2] = io.bond;
    out[3] = io.angle;
    out[4] = io.dih;
    out[5] = io.imp;
    out[6] = io.ivdw;
    out[7] = io.iqq;
    ovs[0] = gs.ov[0];
    ovs[1] = io.overlap ? 1 : 0;
  }
  __syncthreads();
}

__device__ double gc_lrc(const BoxDev& b, const PairTable& T, const double* nb, double rcut3, double rcut9) {
  double e = 0.0;
  for (int ia = 0; ia < T.ntypes; ++ia) {
    double eij = 0.0;
    for (int ja = 0; ja < T.ntypes; ++ja) {
      const double eps = T.eps[pidx(ia, ja, T.ntypes)], s2 = T.sig2[pidx(ia, ja, T.ntypes)];
      const double s6 = s2 * s2 * s2, s12 = s6 * s6;
      eij = eij + nb[ja] * 4.0 * eps * (s12 / (9.0 * rcut9) - (s6 / (3.0 * rcut3)));
    }
    e = e + nb[ia] * eij;
  }
  return 2.0 * kPI * e / b.volume;
}

template <bool MIXED>
__global__ void __launch_bounds__(kGcThreads) k_gcmc(GcArgs A, GcBox* boxes, PairTable T) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BoxDev b;
  __shared__ GrowState gs;
  __shared__ int scratch[kGcThreads + 1];
  __shared__ double em[10];
  __shared__ int eov[2];
  __shared__ int mv_kind, mv_rec, mv_skip, mv_acc, mv_stop;
  __shared__ double old_r[3 * kMaxAtoms], old_com[3];
  __shared__ int ttype[kMaxAtoms];
  __shared__ double rg_new[3 * kMaxAtoms], rg_new_com[3], rg_en[8], rg_e_prev, rg_ln_pfor;
  GcBox& G = boxes[blockIdx.x];
  if (threadIdx.x == 0) b = G.b;
  const int N = G.natoms, R = G.nrec;
  double* sx = reinterpret_cast<double*>(smem);
  double* sy = sx + N;
  double* sz = sy + N;
  double* scom = sz + N;  // [R][3]
  int* stype = reinterpret_cast<int*>(scom + 3 * R);
  int* srec = stype + N;
  int* rlive = srec + N;
  int* rsp = rlive + R;
  int* roff = rsp + R;
  int* pool = roff + R;
  float4* s32 = reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(smem) +
                                          ((((size_t)(pool + R) - (size_t)smem) + 15) & ~(size_t)15));
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double4_32a p = G.xyzq[j];
    sx[j] = p.x;
    sy[j] = p.y;
    sz[j] = p.z;
    stype[j] = G.atype[j];
    if (MIXED) {
      int tb = G.atype[j];
      float tf;
      memcpy(&tf, &tb, sizeof(float));
      s32[j] = make_float4((float)p.x, (float)p.y, (float)p.z, tf);
    }
  }
  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    const int4 ri = G.rec[r];
    rlive[r] = ri.w;
    rsp[r] = ri.y;
    roff[r] = ri.z;
    for (int a = 0; a < A.sp[ri.y].natoms; ++a) srec[ri.z + a] = r;
  }
  for (int k = threadIdx.x; k < G.npool; k += blockDim.x) pool[k] = G.pool[k];
  __syncthreads();
  for (int r = threadIdx.x; r < R; r += blockDim.x) {  // Get_COM
    const GcSpecies& s = A.sp[rsp[r]];
    double tm = 0, x = 0, y = 0, z = 0;
    for (int a = 0; a < s.natoms; ++a) {
      const int j = roff[r] + a;
      tm += s.mass[a];
      x += s.mass[a] * sx[j];
      y += s.mass[a] * sy[j];
      z += s.mass[a] * sz[j];
    }
    scom[3 * r] = x / tm;
    scom[3 * r + 1] = y / tm;
    scom[3 * r + 2] = z / tm;
  }
  if (threadIdx.x < kMaxAtoms) ttype[threadIdx.x] = threadIdx.x < A.S.natoms ? A.S.type[threadIdx.x] : -1;
  GcView V;
  V.b = &b;
  V.T = &T;
  V.sx = sx;
  V.sy = sy;
  V.sz = sz;
  V.stype = stype;
  V.srec = srec;
  V.rlive = rlive;
  V.rsp = rsp;
  V.roff = roff;
  V.com = scom;
  V.s32 = s32;
  V.natoms = N;
  V.nrec = R;
  // thread-0 state
  Lfsr rng;
  CassEnergy E;
  CassGCMCResult RS;
  int npool = G.npool, status = 0;
  int nmol[kGcMaxSpecies];
  double nb[kMaxTypes];
  if (threadIdx.x == 0) {
    rng = seed_stream(A.seed, G.ibox1, 0);
    E = *G.energy;
    memset(&RS, 0, sizeof(RS));
    for (int is = 0; is < A.nspecies; ++is) nmol[is] = 0;
    for (int r = 0; r < R; ++r)
      if (rlive[r]) ++nmol[rsp[r]];
    for (int t = 0; t < kMaxTypes; ++t) nb[t] = G.nb0[t];
  }
  const int ise = A.is_ex;
  const WidomSpecies& S = A.S;
  __syncthreads();
  for (long long step = 0; step < A.nsteps; ++step) {
    // ---- move kind (gcmc_driver.f90:30) and the molecule
    if (threadIdx.x == 0) {
      const double u = rng.next();
      mv_kind = u <= A.cut_t ? 0 : (u <= A.cut_r ? 1 : (u <= A.cut_i ? 2 : (u <= A.cut_d ? 3 : (u <= A.cut_g ? 4 : 5))));
      mv_skip = 0;
      mv_stop = 0;
      scratch[kGcThreads] = 0;
      int is = -1, im = 0;
      if (mv_kind == 0 || mv_kind == 1) {  // species choice of Translate / Rotate
        const double* step_sz = mv_kind == 0 ? G.max_disp : G.max_rot;
        int ntot = 0;
        for (int k = 0; k < A.nspecies; ++k)
          if (step_sz[k] > 0.0) ntot += nmol[k];
        if (ntot == 0) {
          mv_skip = 1;
        } else {
          const double v = rng.next();
          double x = 0.0;
          int last = 0;
          for (int k = 0; k < A.nspecies; ++k) {
            x = (step_sz[k] > 0.0 ? (double)nmol[k] / (double)ntot : 0.0) + (k > 0 ? x : 0.0);
            if (step_sz[k] > 0.0 && nmol[k] > 0) last = k;
            if (is < 0 && v <= x) is = k;
          }
          if (is < 0) is = last;
          im = min((int)(rng.next() * nmol[is]) + 1, nmol[is]);
          if (mv_kind == 0) ++RS.n_translate;
          else ++RS.n_rotate;
        }
      } else if (mv_kind == 2) {
        (void)rng.next();  // is_rand
        if (npool == 0) {
          mv_stop = 1;
          status = 2;
        } else {
          ++RS.n_insert;
          is = ise;
        }
      } else if (mv_kind == 3) {
        (void)rng.next();  // is_rand
        if (nmol[ise] == 0) {
          mv_skip = 1;
        } else {
          ++RS.n_delete;
          is = ise;
          im = min((int)(rng.next() * nmol[ise]) + 1, nmol[ise]);
        }
      } else if (mv_kind == 4) {
        if (nmol[ise] == 0) {
          mv_skip = 1;
        } else {
          (void)rng.next();  // the box choice
          (void)rng.next();  // the species choice
          im = min((int)(rng.next() * nmol[ise]) + 1, nmol[ise]);
          is = ise;
          ++RS.n_regrow;
          if (S.nfrag < 2) mv_skip = 1;  // single-fragment regrowth is not on this path
        }
      } else {
        mv_skip = 1;
      }
      scratch[kGcThreads - 1] = is;
      scratch[kGcThreads - 2] = im;
    }
    __syncthreads();
    if (mv_stop) break;
    const int is = scratch[kGcThreads - 1], im = scratch[kGcThreads - 2];
    __syncthreads();
    if (!mv_skip) {
      int rec;
      if (mv_kind == 2) {
        if (threadIdx.x == 0) mv_rec = pool[npool - 1];  // npool > 0: checked when the move was chosen
        __syncthreads();
        rec = mv_rec;
      } else {
        rec = nth_live(V, is, im, scratch);
      }
      if (rec < 0) {  // the live count and the records disagree: stop the chain
        if (threadIdx.x == 0) status = 1;
        break;
      }
      if (threadIdx.x == 0) {
        gs.rec = rec;
        gs.is = is;
        gs.na = A.sp[is].natoms;
        for (int a = 0; a < gs.na; ++a) {
          gs.r[3 * a] = sx[roff[rec] + a];
          gs.r[3 * a + 1] = sy[roff[rec] + a];
          gs.r[3 * a + 2] = sz[roff[rec] + a];
        }
        for (int d = 0; d < 3; ++d) gs.com[d] = scom[3 * rec + d];
      }
      __syncthreads();
      if (mv_kind <= 1) {
        // ---- Translate / Rotate: old and trial energies of the molecule
        if (threadIdx.x == 0) {
          for (int i = 0; i < 3 * gs.na; ++i) old_r[i] = gs.r[i];
          for (int d = 0; d < 3; ++d) old_com[d] = gs.com[d];
        }
        __syncthreads();
        gc_mol_energies<MIXED>(A, V, gs, stype + roff[rec], em, eov, false);
        if (threadIdx.x == 0) {
          if (eov[0]) {
            mv_stop = 1;
            status = 1;
          } else {
            em[8] = em[0];  // old inter vdW
            const double step_sz = mv_kind == 0 ? G.max_disp[is] : G.max_rot[is];
            const GcSpecies& s = A.sp[is];
            if (mv_kind == 0) {
              double d[3];
              for (int k = 0; k < 3; ++k) d[k] = (2.0 * rng.next() - 1.0) * step_sz;
              for (int a = 0; a < gs.na; ++a)
                for (int k = 0; k < 3; ++k) gs.r[3 * a + k] = gs.r[3 * a + k] + d[k];
              for (int k = 0; k < 3; ++k) gs.com[k] = gs.com[k] + d[k];
              for (int k = 0; k < 3; ++k) {  // Fold_Molecule
                double sh = 0.0;
                if (gs.com[k] > b.hL[k]) sh = -b.L[k];
                else if (gs.com[k] < -b.hL[k]) sh = b.L[k];
                if (sh != 0.0) {
                  gs.com[k] = gs.com[k] + sh;
                  for (int a = 0; a < gs.na; ++a) gs.r[3 * a + k] = gs.r[3 * a + k] + sh;
                }
              }
            } else {
              double Rm[9];
              if (s.linear) {
                const double theta = acos(1.0 - 2.0 * rng.next());
                const double phi = (1.0 - 2.0 * rng.next()) * kPI;
                const double psi = (1.0 - 2.0 * rng.next()) * kPI;
                Rm[0] = cos(psi) * cos(phi) - cos(theta) * sin(phi) * sin(psi);
                Rm[1] = cos(psi) * sin(phi) + cos(theta) * cos(phi) * sin(psi);
                Rm[2] = sin(psi) * sin(theta);
                Rm[3] = -sin(psi) * cos(phi) - cos(theta) * sin(phi) * cos(psi);
                Rm[4] = -sin(psi) * sin(phi) + cos(theta) * cos(phi) * cos(psi);
                Rm[5] = cos(psi) * sin(theta);
                Rm[6] = sin(theta) * sin(phi);
                Rm[7] = -sin(theta) * cos(phi);
                Rm[8] = cos(theta);
              } else {
                const int axis = (int)(3.0 * rng.next()) + 1;
                const double ang = (2.0 * rng.next() - 1.0) * step_sz;
                double k1 = 1.0, k2 = 1.0, k3 = 1.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
                if (axis == 1) sincos(ang, &s1, &k1);
                else if (axis == 2) sincos(ang, &s2, &k2);
                else sincos(ang, &s3, &k3);
                Rm[0] = k1 * k3 - s1 * k2 * s3;
                Rm[1] = s1 * k3 + k1 * k2 * s3;
                Rm[2] = s2 * s3;
                Rm[3] = -k1 * s3 - s1 * k2 * k3;
                Rm[4] = -s1 * s3 + k1 * k2 * k3;
                Rm[5] = s2 * k3;
                Rm[6] = s1 * s2;
                Rm[7] = -k1 * s2;
                Rm[8] = k2;
              }
              for (int a = 0; a < gs.na; ++a) {
                const double x = gs.r[3 * a] - gs.com[0], y = gs.r[3 * a + 1] - gs.com[1], z = gs.r[3 * a + 2] - gs.com[2];
                gs.r[3 * a] = (Rm[0] * x + Rm[1] * y + Rm[2] * z) + gs.com[0];
                gs.r[3 * a + 1] = (Rm[3] * x + Rm[4] * y + Rm[5] * z) + gs.com[1];
                gs.r[3 * a + 2] = (Rm[6] * x + Rm[7] * y + Rm[8] * z) + gs.com[2];
              }
            }
          }
        }
        __syncthreads();
        if (mv_stop) break;
        const double ev_old = em[8];
        gc_mol_energies<MIXED>(A, V, gs, stype + roff[rec], em, eov, false);
        if (threadIdx.x == 0) {
          mv_acc = 0;
          if (!eov[0]) {
            const double dv = em[0] - ev_old;
            if (gc_accept(b.beta * dv, rng)) {
              mv_acc = 1;
              E.total = E.total + dv;
              E.inter = E.inter + dv;
              E.inter_vdw = E.inter_vdw + dv;
              if (mv_kind == 0) {
                ++RS.n_translate_accepted;
              } else {
                ++RS.n_rotate_accepted;
                const GcSpecies& s = A.sp[is];  // Get_COM on acceptance
                double tm = 0, x = 0, y = 0, z = 0;
                for (int a = 0; a < gs.na; ++a) {
                  tm += s.mass[a];
                  x += s.mass[a] * gs.r[3 * a];
                  y += s.mass[a] * gs.r[3 * a + 1];
                  z += s.mass[a] * gs.r[3 * a + 2];
                }
                gs.com[0] = x / tm;
                gs.com[1] = y / tm;
                gs.com[2] = z / tm;
              }
            }
          }
          if (!mv_acc) {
            for (int i = 0; i < 3 * gs.na; ++i) gs.r[i] = old_r[i];
            for (int d = 0; d < 3; ++d) gs.com[d] = old_com[d];
          }
        }
      } else if (mv_kind == 2) {
        // ---- Insertion
        const bool ov = gc_build<MIXED>(A, V, gs, false, rng);
        if (threadIdx.x == 0) {
          gs.flag = ov ? 1 : 0;
          gs.ln_pbias = gs.ln_pbias + gs.ln_pseq + S.ln_kappa_ins + S.ln_kappa_dih_term;
          if (!ov) {  // Fold_Molecule, Get_COM
            for (int k = 0; k < 3; ++k) {
              double sh = 0.0;
              if (gs.com[k] > b.hL[k]) sh = -b.L[k];
              else if (gs.com[k] < -b.hL[k]) sh = b.L[k];
              if (sh != 0.0) {
                gs.com[k] = gs.com[k] + sh;
                for (int a = 0; a < gs.na; ++a) gs.r[3 * a + k] = gs.r[3 * a + k] + sh;
              }
            }
            get_com(S, gs.r, (1u << gs.na) - 1u, gs.com);
          }
        }
        if (threadIdx.x == 0) mv_acc = 0;
        __syncthreads();
        if (!gs.flag) {
          gc_mol_energies<MIXED>(A, V, gs, ttype, em, eov);
          if (threadIdx.x == 0 && !eov[0] && !eov[1]) {
            const double ev = em[0], eq = em[1];
            const double eb = em[2], ea = em[3], ed = em[4], ei = em[5], eiv = em[6], eiq = em[7];
            double dE_inter = ev + eq, dE_intra = eiv + eiq + eb + ea + ed + ei;
            double nbn[kMaxTypes];
            for (int t = 0; t < kMaxTypes; ++t) nbn[t] = nb[t];
            for (int a = 0; a < gs.na; ++a)
              if (S.type[a] >= 0) nbn[S.type[a]] += 1.0;
            double e_lrc = E.lrc;
            const bool tail = b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL;
            if (tail) {
              e_lrc = gc_lrc(b, T, nbn, G.rcut3, G.rcut9);
              dE_inter = dE_inter + e_lrc - E.lrc;
            }
            const double dE = dE_intra + dE_inter;
            double ln_pacc = b.beta * (dE - ea);
            ln_pacc = ln_pacc - G.mu * b.beta;
            ln_pacc = ln_pacc + gs.ln_pbias;
            ln_pacc = ln_pacc + log((double)(nmol[ise] + 1)) + G.log_lambda3;
            ln_pacc = ln_pacc - log(b.volume);
            if (gc_accept(ln_pacc, rng)) {
              mv_acc = 1;
              E.total += dE;
              E.intra += dE_intra;
              E.inter += dE_inter;
              E.bond += eb;
              E.angle += ea;
              E.dihedral += ed;
              E.improper += ei;
              E.intra_vdw += eiv;
              E.intra_q += eiq;
              E.inter_vdw += ev;
              E.inter_q += eq;
              if (tail) E.lrc = e_lrc;
              for (int t = 0; t < kMaxTypes; ++t) nb[t] = nbn[t];
              ++RS.n_insert_accepted;
              ++nmol[ise];
              --npool;
            }
          }
        }
        if (threadIdx.x == 0 && mv_acc) rlive[gs.rec] = 1;
      } else if (mv_kind == 3) {
        // ---- Deletion
        const bool ov = gc_build<MIXED>(A, V, gs, true, rng);
        if (threadIdx.x == 0) {
          gs.flag = ov ? 1 : 0;
          if (ov) {
            mv_stop = 1;
            status = 1;
          }
          gs.ln_pbias = gs.ln_pbias + gs.ln_pseq + S.ln_kappa_ins + S.ln_kappa_dih_term;
          get_com(S, gs.r, (1u << gs.na) - 1u, gs.com);
        }
        __syncthreads();
        if (mv_stop) break;
        gc_mol_energies<MIXED>(A, V, gs, ttype, em, eov);
        if (threadIdx.x == 0) {
          mv_acc = 0;
          const double ev = em[0], eq = em[1];
          const double eb = em[2], ea = em[3], ed = em[4], ei = em[5], eiv = em[6], eiq = em[7];
          double dE_inter = -ev;
          double dE_intra = -eb - ea - ed - ei;
          dE_intra = dE_intra - eiv - eiq;
          dE_inter = dE_inter - eq;
          double nbn[kMaxTypes];
          for (int t = 0; t < kMaxTypes; ++t) nbn[t] = nb[t];
          for (int a = 0; a < gs.na; ++a)
            if (S.type[a] >= 0) nbn[S.type[a]] -= 1.0;
          double e_lrc = E.lrc;
          const bool tail = b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL;
          if (tail) {
            e_lrc = gc_lrc(b, T, nbn, G.rcut3, G.rcut9);
            dE_inter = dE_inter + (e_lrc - E.lrc);
          }
          const double dE = dE_intra + dE_inter;
          double ln_pacc = b.beta * (dE + ea);
          ln_pacc = ln_pacc + b.beta * G.mu;
          ln_pacc = ln_pacc - gs.ln_pbias;
          ln_pacc = ln_pacc - log((double)nmol[ise]) - G.log_lambda3;
          ln_pacc = ln_pacc + log(b.volume);
          if (gc_accept(ln_pacc, rng)) {
            mv_acc = 1;
            E.total += dE;
            E.intra += dE_intra;
            E.inter += dE_inter;
            E.bond -= eb;
            E.angle -= ea;
            E.dihedral -= ed;
            E.improper -= ei;
            E.intra_vdw -= eiv;
            E.intra_q -= eiq;
            E.inter_vdw -= ev;
            E.inter_q -= eq;
            if (tail) E.lrc = e_lrc;
            for (int t = 0; t < kMaxTypes; ++t) nb[t] = nbn[t];
            ++RS.n_delete_accepted;
            --nmol[ise];
            rlive[gs.rec] = 0;
            pool[npool++] = gs.rec;
          }
          // a rejected deletion keeps the coordinates its Rosenbluth pass left
        }
      } else {
        // ---- Cut_N_Grow: Cut_Regrow for the new configuration, then for the old one
        if (threadIdx.x == 0) {
          mv_acc = 0;
          for (int i = 0; i < 3 * gs.na; ++i) old_r[i] = gs.r[i];
          for (int d = 0; d < 3; ++d) old_com[d] = gs.com[d];
          const int fb = min((int)(rng.next() * A.nfbond), A.nfbond - 1);
          if (rng.next() < A.prob_del1[fb]) {
            gs.f_dead = A.fb_a[fb];
            gs.f_live = A.fb_b[fb];
          } else {
            gs.f_dead = A.fb_b[fb];
            gs.f_live = A.fb_a[fb];
          }
          gs.order[0] = gs.f_dead;
          gs.norder = 1;
          gs.ln_pseq = 0.0;
          gc_fragment_order(S, gs, (1u << gs.f_live) | (1u << gs.f_dead), rng);
          gc_cut(S, gs);
          rg_e_prev = dihedral_masked(A.P.hdr[S.is0], A.P, gs.r, gs.exist);
          gs.e_prev = rg_e_prev;
        }
        __syncthreads();
        bool ov = gc_place_fragments<MIXED>(A, V, gs, 0, false, rng, A.lib);
        if (threadIdx.x == 0) {
          if (ov) {  // Revert_Old_Cartesian_Coordinates
            for (int i = 0; i < 3 * gs.na; ++i) gs.r[i] = old_r[i];
            for (int d = 0; d < 3; ++d) gs.com[d] = old_com[d];
          } else {  // Get_COM, Fold_Molecule
            rg_ln_pfor = gs.ln_pbias;
            get_com(S, gs.r, (1u << gs.na) - 1u, gs.com);
            for (int k = 0; k < 3; ++k) {
              double sh = 0.0;
              if (gs.com[k] > b.hL[k]) sh = -b.L[k];
              else if (gs.com[k] < -b.hL[k]) sh = b.L[k];
              if (sh != 0.0) {
                gs.com[k] = gs.com[k] + sh;
                for (int a = 0; a < gs.na; ++a) gs.r[3 * a + k] = gs.r[3 * a + k] + sh;
              }
            }
          }
        }
        __syncthreads();
        if (!ov) {
          gc_mol_energies<MIXED>(A, V, gs, ttype, em, eov);
          if (threadIdx.x == 0) {
            if (eov[0]) {
              ov = true;
              for (int i = 0; i < 3 * gs.na; ++i) gs.r[i] = old_r[i];
              for (int d = 0; d < 3; ++d) gs.com[d] = old_com[d];
            } else {
              for (int k = 0; k < 8; ++k) rg_en[k] = em[k];
              for (int i = 0; i < 3 * gs.na; ++i) {
                rg_new[i] = gs.r[i];
                gs.r[i] = old_r[i];
              }
              for (int d = 0; d < 3; ++d) {
                rg_new_com[d] = gs.com[d];
                gs.com[d] = old_com[d];
              }
              gc_cut(S, gs);
              gs.e_prev = rg_e_prev;
              gs.ln_pbias = 0.0;
            }
            gs.flag = ov ? 1 : 0;
          }
          __syncthreads();
          if (!gs.flag) {
            const bool ov_old = gc_place_fragments<MIXED>(A, V, gs, 0, true, rng, A.lib);
            if (threadIdx.x == 0) {
              if (ov_old) {
                mv_stop = 1;
                status = 1;
              } else {
                get_com(S, gs.r, (1u << gs.na) - 1u, gs.com);
              }
            }
            __syncthreads();
            if (mv_stop) break;
            gc_mol_energies<MIXED>(A, V, gs, ttype, em, eov);
            if (threadIdx.x == 0) {
              const double* en = rg_en;  // ev, eq, eb, ea, ed, ei, eiv, eiq of the new configuration
              double dE_intra = en[2] + en[3] + en[4] + en[5] + en[7] + en[6];
              double dE_inter = en[1] + en[0];
              dE_intra = dE_intra - em[2] - em[3] - em[4] - em[5] - em[7] - em[6];
              dE_inter = dE_inter - em[1] - em[0];
              const double dE = dE_intra + dE_inter;
              const double dE_frag = en[3] - em[3];
              const double ln_pacc = b.beta * (dE - dE_frag) + rg_ln_pfor - gs.ln_pbias;
              if (gc_accept(ln_pacc, rng)) {
                mv_acc = 1;
                for (int i = 0; i < 3 * gs.na; ++i) gs.r[i] = rg_new[i];
                for (int d = 0; d < 3; ++d) gs.com[d] = rg_new_com[d];
                E.total += dE;
                E.intra += dE_intra;
                E.inter += dE_inter;
                E.bond += en[2] - em[2];
                E.angle += en[3] - em[3];
                E.dihedral += en[4] - em[4];
                E.improper += en[5] - em[5];
                E.intra_vdw += en[6] - em[6];
                E.intra_q += en[7] - em[7];
                E.inter_vdw += en[0] - em[0];
                E.inter_q += en[1] - em[1];
                ++RS.n_regrow_accepted;
              }
            }
          }
        }
      }
      __syncthreads();
      // commit the molecule's coordinates (rejected deletions and regrowths keep
      // the coordinates of their Rosenbluth pass, as the reference does)
      if (threadIdx.x == 0) {
        if (mv_kind != 2 || mv_acc) {
          for (int a = 0; a < gs.na; ++a) {
            const int j = roff[gs.rec] + a;
            sx[j] = gs.r[3 * a];
            sy[j] = gs.r[3 * a + 1];
            sz[j] = gs.r[3 * a + 2];
            if (MIXED) s32[j] = make_float4((float)gs.r[3 * a], (float)gs.r[3 * a + 1], (float)gs.r[3 * a + 2], s32[j].w);
          }
          for (int d = 0; d < 3; ++d) scom[3 * gs.rec + d] = gs.com[d];
        }
      }
    }
    if (threadIdx.x == 0) RS.sum_n_molecules += (double)nmol[ise];
    __syncthreads();
  }
  __syncthreads();
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    double4_32a p = G.xyzq[j];
    p.x = sx[j];
    p.y = sy[j];
    p.z = sz[j];
    G.xyzq[j] = p;
  }
  for (int r = threadIdx.x; r < R; r += blockDim.x) G.rec[r].w = rlive[r];
  if (threadIdx.x == 0) {
    RS.energy = E;
    RS.n_molecules = nmol[ise];
    *G.res = RS;
    *G.energy = E;
    *G.status = status;
  }
}

}  // namespace cassgpu

namespace cassgpu {
int pack_box_ext(cass_ctx* c, int ibox);
const std::vector<int>& members_ext(cass_ctx* c, int ibox);
int ensure_pools(cass_ctx* c);
void fill_growth_species(const SpeciesH& s, int is0, int kappa_ins, int kappa_dih, WidomSpecies& S);
void invalidate_ext(cass_ctx* c, int ibox);
void set_mol_box_ext(cass_ctx* c, int slot, int ibox);

size_t gc_smem_bytes(int natoms, int nrec, bool mixed) {
  size_t s = (size_t)natoms * (3 * sizeof(double) + 2 * sizeof(int)) + (size_t)nrec * (3 * sizeof(double) + 4 * sizeof(int));
  s = (s + 15) & ~(size_t)15;
  if (mixed) s += (size_t)natoms * sizeof(float4);
  return s;
}
}  // namespace cassgpu

using namespace cassgpu;

extern "C" int cass_gcmc(cass_ctx* c, int32_t nboxes, const int32_t* iboxes, const CassGCMCParams* p,
                         const double* mu, const double* max_disp, const double* max_rot, uint64_t seed,
                         CassGCMCResult* out) {
  if (!c || nboxes < 1 || !iboxes || !p || !mu || !max_disp || !max_rot || !out || p->nsteps < 0 ||
      p->is_exchange < 1 || p->is_exchange > c->nspecies || p->kappa_ins < 1 || p->kappa_ins > kMaxKappa)
    return set_error(CASS_EINVAL, "bad gcmc arguments");
  if (c->nspecies > kGcMaxSpecies) return set_error(CASS_ECAPACITY, "gcmc supports at most 8 species");
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  const int is = p->is_exchange - 1;
  const SpeciesH& s = c->sp[is];
  if (!s.defined || s.nfrag < 1) return set_error(CASS_ESTATE, "exchanged species not defined or without fragments");
  if (s.nfrag > 1 && (p->kappa_dih < 1 || p->kappa_dih > kMaxKappa)) return set_error(CASS_EINVAL, "kappa_dih must be in 1..32");
  if (s.nfrag > kMaxFrags) return set_error(CASS_ECAPACITY, "exchanged species has more than 8 fragments");
  for (int k = 0; k < c->nspecies; ++k)
    if (c->sp[k].defined && c->sp[k].natoms > kMaxAtoms) return set_error(CASS_ECAPACITY, "gcmc moves molecules of at most 16 atoms");
  for (int f = 0; f < s.nfrag; ++f)
    if (s.frag_nconfig[f] < 1) return set_error(CASS_EINVAL, "fragment library is empty");
  bool mixed = c->precision == CASS_PREC_MIXED;
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    if (ib < 0 || ib >= c->nboxes) return set_error(CASS_EINVAL, "box index out of range");
    for (int j = 0; j < k; ++j)
      if (iboxes[j] == iboxes[k]) return set_error(CASS_EINVAL, "box listed twice");
    const BoxH& B = c->box[ib];
    if (!B.energy_valid) return set_error(CASS_ESTATE, "system energy of box not computed");
    if (B.desc.charge_style != CASS_CHARGE_NONE) return set_error(CASS_EUNSUPPORTED, "gcmc boxes hold no charges");
    if (B.desc.vdw_style != CASS_VDW_LJ) return set_error(CASS_EUNSUPPORTED, "gcmc needs LJ boxes");
    mixed = mixed && (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT || B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL);
  }
  int rc;
  CASS_CUDA(cudaSetDevice(c->device));
  if ((rc = ensure_pools(c))) return rc;
  GcArgs A;
  memset(&A, 0, sizeof(A));
  fill_growth_species(s, is, p->kappa_ins, p->kappa_dih, A.S);
  A.is_ex = is;
  A.nspecies = c->nspecies;
  for (int k = 0; k < c->nspecies; ++k) {
    const SpeciesH& t = c->sp[k];
    A.sp[k].natoms = t.natoms;
    bool lin = true;
    for (size_t q = 0; q < t.angle_kind.size(); ++q)
      if (t.angle_kind[q] != CASS_BONDED_FIXED || t.angle_param[2 * q] != 180.0) lin = false;
    A.sp[k].linear = lin ? 1 : 0;
    for (int a = 0; a < t.natoms && a < kMaxAtoms; ++a) A.sp[k].mass[a] = t.mass[a];
  }
  A.nsteps = p->nsteps;
  A.cut_t = p->cut_translate;
  A.cut_r = p->cut_rotate;
  A.cut_i = p->cut_insert;
  A.cut_d = p->cut_delete;
  A.cut_g = p->cut_regrow;
  A.seed = seed;
  A.lib = s.d_library.as<double>();
  A.P = c->pools;
  // fragment bonds (f, g), f < g, and the probability of deleting f when the bond is cut
  // (input_routines.f90:3035-3120): atoms beyond the bond on g's side over both sides
  for (int f = 0; f < s.nfrag; ++f)
    for (int g : s.frag_connect[f]) {
      if (g <= f || A.nfbond >= kMaxFrags) continue;
      int ndel[2];
      for (int side = 0; side < 2; ++side) {
        const int f1 = side ? g : f, f2 = side ? f : g;
        std::vector<int> live(s.nfrag, 0), order{f1};
        live[f1] = live[f2] = 1;
        for (size_t q = 0; q < order.size(); ++q)
          for (int h : s.frag_connect[order[q]])
            if (!live[h]) {
              live[h] = 1;
              order.push_back(h);
            }
        ndel[side] = 0;
        for (int h : order) ndel[side] += (int)s.frag_atoms[h].size() - 2;
      }
      A.fb_a[A.nfbond] = f;
      A.fb_b[A.nfbond] = g;
      A.prob_del1[A.nfbond] = (double)ndel[1] / (double)(ndel[0] + ndel[1]);
      ++A.nfbond;
    }
  double mw = 0.0;
  for (double m : s.mass) mw += m;
  // free slots of the exchanged species, dealt to the boxes in turn
  std::vector<std::vector<int>> pools(nboxes);
  {
    int nfree = 0;
    for (int im = 0; im < c->max_mol[is]; ++im) {
      const int slot = c->mol_base[is] + im;
      if (c->mol_box[slot] >= 0) continue;
      pools[nfree % nboxes].push_back(slot);
      ++nfree;
    }
  }
  // per-box records: the live molecules and the box's free slots, in slot order
  struct HostBox {
    std::vector<int> slots;
    std::vector<int4> rec;
    std::vector<double4_32a> xyzq;
    std::vector<int> atype, pool;
  };
  std::vector<HostBox> hb(nboxes);
  std::vector<GcBox> gb(nboxes);
  size_t smem = 0, tot_atoms = 0, tot_rec = 0;
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    BoxH& B = c->box[ib];
    HostBox& h = hb[k];
    const std::vector<int>& mem = members_ext(c, ib);
    h.slots.assign(mem.begin(), mem.end());
    h.slots.insert(h.slots.end(), pools[k].begin(), pools[k].end());
    std::sort(h.slots.begin(), h.slots.end());
    int off = 0;
    double nb0[kMaxTypes] = {0};
    for (size_t r = 0; r < h.slots.size(); ++r) {
      const int slot = h.slots[r], sp = c->slot_sp[slot];
      const SpeciesH& t = c->sp[sp];
      const bool live = c->mol_box[slot] == ib;
      h.rec.push_back(make_int4(slot, sp, off, live ? 1 : 0));
      const double* x = &t.pos[(size_t)(slot - c->mol_base[sp]) * 3 * t.natoms];
      for (int a = 0; a < t.natoms; ++a) {
        h.xyzq.push_back(make_double4_32a(live ? x[3 * a] : 0.0, live ? x[3 * a + 1] : 0.0, live ? x[3 * a + 2] : 0.0, t.q[a]));
        h.atype.push_back(t.type[a]);
        if (live && t.type[a] >= 0) nb0[t.type[a]] += 1.0;
      }
      off += t.natoms;
    }
    for (int slot : pools[k]) h.pool.push_back((int)(std::lower_bound(h.slots.begin(), h.slots.end(), slot) - h.slots.begin()));
    GcBox& g = gb[k];
    memset(&g, 0, sizeof(g));
    g.b = B.dev;
    g.natoms = off;
    g.nrec = (int)h.slots.size();
    g.npool = (int)h.pool.size();
    g.ibox1 = iboxes[k];
    g.mu = mu[k] / 0.01;  // kJ/mol to internal units (atomic_to_kJmol)
    g.log_lambda3 = 3.0 * std::log(39.9031268605 * std::sqrt(B.dev.beta / (kTWOPI * mw)));  // de Broglie
    g.rcut3 = B.rcut3;
    g.rcut9 = B.rcut9;
    for (int t = 0; t < kMaxTypes; ++t) g.nb0[t] = nb0[t];
    smem = std::max(smem, gc_smem_bytes(g.natoms, g.nrec, mixed));
    tot_atoms += (size_t)off;
    tot_rec += h.slots.size();
  }
  if (smem > kGcSmemLimit)
    return set_error(CASS_ECAPACITY, "gcmc holds a box's molecules and free slots in shared memory: too many atoms");
  const size_t nsp = (size_t)c->nspecies;
  const size_t bytes = nboxes * sizeof(GcBox) + tot_atoms * (sizeof(double4_32a) + sizeof(int)) +
                       tot_rec * (sizeof(int4) + sizeof(int)) + 2 * nboxes * nsp * sizeof(double) +
                       nboxes * (sizeof(CassEnergy) + sizeof(CassGCMCResult) + sizeof(int)) + 1024;
  if ((rc = c->d_gc.reserve(bytes))) return rc;
  char* base = static_cast<char*>(c->d_gc.p);
  auto carve = [&](size_t n, size_t align) {
    size_t o = ((size_t)(base - static_cast<char*>(c->d_gc.p)) + align - 1) & ~(align - 1);
    char* q = static_cast<char*>(c->d_gc.p) + o;
    base = q + n;
    return q;
  };
  GcBox* d_box = reinterpret_cast<GcBox*>(carve(nboxes * sizeof(GcBox), 64));
  CassEnergy* d_E = reinterpret_cast<CassEnergy*>(carve(nboxes * sizeof(CassEnergy), 16));
  CassGCMCResult* d_res = reinterpret_cast<CassGCMCResult*>(carve(nboxes * sizeof(CassGCMCResult), 16));
  int* d_status = reinterpret_cast<int*>(carve(nboxes * sizeof(int), 16));
  double* d_md = reinterpret_cast<double*>(carve(nboxes * nsp * sizeof(double), 16));
  double* d_mr = reinterpret_cast<double*>(carve(nboxes * nsp * sizeof(double), 16));
  std::vector<CassEnergy> hE(nboxes);
  std::vector<double4_32a*> d_xyz(nboxes);
  std::vector<int4*> d_rec(nboxes);
  for (int k = 0; k < nboxes; ++k) {
    HostBox& h = hb[k];
    GcBox& g = gb[k];
    d_xyz[k] = reinterpret_cast<double4_32a*>(carve(std::max<size_t>(1, h.xyzq.size()) * sizeof(double4_32a), 32));
    int* d_at = reinterpret_cast<int*>(carve(std::max<size_t>(1, h.atype.size()) * sizeof(int), 16));
    d_rec[k] = reinterpret_cast<int4*>(carve(std::max<size_t>(1, h.rec.size()) * sizeof(int4), 16));
    int* d_pool = reinterpret_cast<int*>(carve(std::max<size_t>(1, h.pool.size()) * sizeof(int), 16));
    if (!h.xyzq.empty()) {
      CASS_CUDA(h2d(c, d_xyz[k], h.xyzq.data(), h.xyzq.size() * sizeof(double4_32a)));
      CASS_CUDA(h2d(c, d_at, h.atype.data(), h.atype.size() * sizeof(int)));
      CASS_CUDA(h2d(c, d_rec[k], h.rec.data(), h.rec.size() * sizeof(int4)));
    }
    if (!h.pool.empty()) CASS_CUDA(h2d(c, d_pool, h.pool.data(), h.pool.size() * sizeof(int)));
    g.xyzq = d_xyz[k];
    g.atype = d_at;
    g.rec = d_rec[k];
    g.pool = d_pool;
    g.max_disp = d_md + k * nsp;
    g.max_rot = d_mr + k * nsp;
    g.energy = d_E + k;
    g.res = d_res + k;
    g.status = d_status + k;
    hE[k] = c->box[iboxes[k] - 1].energy;
  }
  CASS_CUDA(h2d(c, d_box, gb.data(), nboxes * sizeof(GcBox)));
  CASS_CUDA(h2d(c, d_E, hE.data(), nboxes * sizeof(CassEnergy)));
  CASS_CUDA(h2d(c, d_md, max_disp, nboxes * nsp * sizeof(double)));
  CASS_CUDA(h2d(c, d_mr, max_rot, nboxes * nsp * sizeof(double)));
  auto kern = mixed ? k_gcmc<true> : k_gcmc<false>;
  CASS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  CASS_CUDA(cudaEventRecord(c->ev[0], c->stream));
  kern<<<nboxes, kGcThreads, smem, c->stream>>>(A, d_box, c->pt);
  CASS_CUDA(cudaGetLastError());
  CASS_CUDA(cudaEventRecord(c->ev[1], c->stream));
  count_launch(c);
  std::vector<CassGCMCResult> hr(nboxes);
  std::vector<int> hs(nboxes);
  CASS_CUDA(d2h(c, hr.data(), d_res, nboxes * sizeof(CassGCMCResult)));
  CASS_CUDA(d2h(c, hs.data(), d_status, nboxes * sizeof(int)));
  for (int k = 0; k < nboxes; ++k) {
    HostBox& h = hb[k];
    if (h.xyzq.empty()) continue;
    CASS_CUDA(d2h(c, h.xyzq.data(), d_xyz[k], h.xyzq.size() * sizeof(double4_32a)));
    CASS_CUDA(d2h(c, h.rec.data(), d_rec[k], h.rec.size() * sizeof(int4)));
  }
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  float ms = 0.0f;
  CASS_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->stats.mc_ms = ms;
  c->stats.mc_moves = p->nsteps * nboxes;
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    HostBox& h = hb[k];
    for (size_t r = 0; r < h.rec.size(); ++r) {
      const int4 ri = h.rec[r];
      const int slot = ri.x, sp = ri.y;
      SpeciesH& t = c->sp[sp];
      set_mol_box_ext(c, slot, ri.w ? ib : -1);
      if (!ri.w) continue;
      double* x = &t.pos[(size_t)(slot - c->mol_base[sp]) * 3 * t.natoms];
      for (int a = 0; a < t.natoms; ++a) {
        const double4_32a& v = h.xyzq[ri.z + a];
        x[3 * a] = v.x;
        x[3 * a + 1] = v.y;
        x[3 * a + 2] = v.z;
      }
    }
    invalidate_ext(c, ib);  // repack on next use; the running energy stays valid
    c->box[ib].energy = hr[k].energy;
    c->box[ib].energy_valid = true;
    out[k] = hr[k];
  }
  for (int k = 0; k < nboxes; ++k) {
    if (hs[k] == 1) return set_error(CASS_ESTATE, "a molecule overlapped another before its move (energy too high)");
    if (hs[k] == 2) return set_error(CASS_ECAPACITY, "no free molecule slot left for an insertion");
  }
  return CASS_OK;
}
