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
//
// A box may be run by a thread-block cluster of C CTAs (C = 1, 2, 4 or 8,
// chosen so that all boxes run at once).  Every CTA of the cluster holds the
// whole box and runs the same serial steps from the same lfsr258 stream, so
// all make the same decisions; the pair loops of a batch are split over the
// CTAs, whose per-trial partial sums are exchanged through distributed shared
// memory and added in rank order after one cluster barrier per batch (two
// partial buffers alternate, so a buffer is rewritten only after every CTA
// has read it).
//
// Charged boxes (Coulomb with the Ewald sum) run the FP64 kernel on one CTA
// per box: the pair batches add the real-space terms, and each move that
// changes a charged molecule computes the box's new reciprocal energy from
// the running structure factors (thread k mod blockDim.x owns k-vector k),
// which are committed, with the molecule's row, only on acceptance.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cass_cbmc.cuh"
#include "cass_cbmc_f.cuh"
#include "cass_ctx.h"

namespace cassgpu {

constexpr int kGcThreads = 512;
constexpr int kGcWarps = kGcThreads / 32;
constexpr int kGcMaxSpecies = 8;
constexpr size_t kGcSmemLimit = 190 * 1024;  // dynamic; the static part is about 35 KB of the 227 KB

struct GcSpecies {
  int natoms, linear, has_charge;
  int l_coul_cbmc;  // species_list%L_Coul_CBMC: CBMC trial energies include the intermolecular charges
  double mass[kMaxAtoms];
  double q[kMaxAtoms];
  int type[kMaxAtoms];  // nonbond type per atom, -1: none
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
  // FP32 copies for the mixed kernel
  SpeciesF SF;
  const float* libf;
  float prob_del1f[kMaxFrags];
  float cutf[5];
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
  double lrc_c[kMaxTypes * kMaxTypes];  // 4 eps (sigma^12 / (9 rc^9) - sigma^6 / (3 rc^3)) per type pair
  double lrc_pref;        // 2 pi / V
  double log_vol;         // ln V
  const double* logn;     // ln k, k = 0 .. nrec + 1 (mixed kernel)
  double nb0[kMaxTypes];  // atoms per type at the start
  CassEnergy* energy;
  CassGCMCResult* res;
  int* status;  // 0 ok, 1 overlapping molecule before a move, 2 no free slot
  int comcut;    // LJ CHARMM: molecule pairs selected by Check_MoleculePair_Cutoff (FP64 kernel)
  double rmax;   // rcut_max of that test
  // charged boxes (Coulomb with the Ewald sum; FP64 kernel, one CTA per box):
  // the k-vectors (hx, hy, hz, Cn), the box's running structure factors, the
  // per-molecule rows (slot-major, row stride `stride`) and a scratch row for
  // the moved molecule's new factors
  int qon, nvecs, stride;
  const double4_32a* kvec;
  double *cos_sum, *sin_sum, *cos_mol, *sin_mol, *new_cos, *new_sin;
};

// the molecule being built / moved and one stage of trials (shared memory)
struct GrowState {
  double r[3 * kMaxAtoms];
  double com[3];
  unsigned exist;
  int rec, is, na;
  // trial batch
  double trial[kMaxKappa][3 * kMaxAtoms];
  float trialf[kMaxKappa][3 * kMaxAtoms];  // FP32 copy of the atoms a batch evaluates (mixed kernel)
  int tids[kMaxAtoms], ntid;
  double e[kMaxKappa];
  float ef[kMaxKappa];
  int ov[kMaxKappa];
  double tcom[kMaxKappa][4];  // COM and max_dcom of each trial's atoms (molecule-pair cutoff boxes)
  double cpart[2][kMaxKappa];  // per-CTA trial sums read by the cluster (alternating buffers)
  float cpartf[2][kMaxKappa];
  int covl[2][kMaxKappa];
  int cbuf;
  double part[kGcWarps * kMaxKappa];  // per-warp trial sums
  float partf[kGcWarps * kMaxKappa];  // the same in FP32 (mixed CBMC batches)
  int povl[kGcWarps];                 // per-warp overlap masks
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

// The box as a kernel sees it.  Atoms of every record (live molecules and the
// box's free slots) sit at fixed offsets (roff) in sx/sy/sz; the atoms of the
// live molecules are also listed compactly in lv (atom index), with apos the
// inverse map (-1: not listed) and per entry the type (lvt) or, in the mixed
// kernel, an FP32 copy x, y, z, type bits (lv32).  Pair loops run over lv.
// lrec holds, per species s from rs0[s], the live records in ascending order.
// FP32 state of the molecule a mixed-kernel CBMC move grows (shared memory);
// GrowState holds the integer bookkeeping and the trial batch
struct GrowF {
  float r[3 * kMaxAtoms];
  float com[3];
  float cfg[3 * kMaxAtoms], hg[9];
  float theta0;
  float draws[3 * kMaxKappa];
  float dn[kMaxKappa], dd[kMaxKappa];
  float ln_pseq, ln_pbias, e_prev;
};

struct GcView {
  const BoxDev* b;
  const PairTable* T;
  const float* epsf;  // FP32 pair table copied to shared memory
  const float* sig2f;
  const BoxF* bf;     // FP32 box constants (mixed kernel)
  const float2* ljp;  // (eps, sigma^2) with row stride kMaxTypes (mixed kernel)
  double *sx, *sy, *sz;
  int *lv, *apos, *lvt;
  float4* lv32;
  int *rlive, *rsp, *roff, *lrec;
  const int* nlv;
  double* com;
  double* rdcom;  // per record max_dcom (molecule-pair cutoff boxes)
  int* arec;      // record of each atom
  const double* sq;  // charge of each atom (charged boxes), else nullptr
  int comcut;
  double rmax;
  int natoms, nrec;
  int crank, csize;  // rank of this CTA in the box's cluster, cluster size
};

// ---------------------------------------------------------------------------
// Sums TG per-lane values over a warp.  The values are halved at each step of
// a butterfly (the lane keeps one half and adds its partner's copy of it), so
// TG sums take TG - 1 + log2(32 / TG) shuffles instead of 5 TG.  Returns the
// warp total of value `which`; every lane gets one, lanes l and l ^ m (m <
// 32 / TG) the same one.  Fixed order, so the result is deterministic.
template <int TG, class R>
__device__ __forceinline__ R warp_multi_sum(R (&v)[TG], int lane, int& which) {
  which = 0;
  int off = 16;
#pragma unroll
  for (int n = TG; n > 1; n >>= 1) {
    const bool hi = (lane & off) != 0;
#pragma unroll
    for (int u = 0; u < n / 2; ++u) {
      const R send = hi ? v[u] : v[u + n / 2];
      const R keep = hi ? v[u + n / 2] : v[u];
      v[u] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
    which = 2 * which + (hi ? 1 : 0);
    off >>= 1;
  }
  R s = v[0];
  for (; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}

// Block-wide energies of ntr configurations of the atoms gs.tids (taken from
// gs.trial[t]) against every listed atom outside the atom range of record
// skip_rec.  Each lane takes box atoms and evaluates all trials of a group of
// TG against them, with the sums in registers; the per-warp sums are added
// in warp order.  gs.e[t] (0 on overlap) and gs.ov[t] on return.  In the
// mixed kernel a lane's sum and the sum over a warp are FP32 (the FP64 pipe
// of GB300 issues at 1/64 of the FP32 rate); CBMC trial batches (TG > 2) stay
// FP32 to the end and fill gs.ef only, molecule energies (TG = 2) add the
// per-warp sums in FP64 and fill both gs.e and gs.ef.
// In a molecule-pair cutoff box (FP64 kernel) a box atom counts for trial t
// only when its molecule passes Check_MoleculePair_Cutoff (energy_routines.f90:
// 3027-3088) against the trial's atoms gs.tids (their COM and max_dcom, masses
// tmass), overlap test included, as in the reference's molecule loops.
// In a charged box (FP64 kernel; V.sq and the trial atoms' charges tq set)
// the real-space Ewald term of each pair within the charge cutoff (rcut_cbmc
// in CBMC batches) is added as well (Compute_AtomPair_Energy, energy_routines.
// f90:2014-2049): to the trial's sum, or with SPLITQ (ntr <= TG / 2) to entry
// t + TG / 2, so that gs.e[t] holds the vdW and gs.e[t + TG / 2] the Coulomb
// sum of trial t.
template <bool MIXED, int TG, bool SPLITQ = false>
__device__ void batch_energies(const GcView& V, GrowState& gs, int ntr, int skip_rec, bool cbmc,
                               const int* ttype, bool convert = true, const double* tmass = nullptr,
                               const double* tq = nullptr) {
  const BoxDev& b = *V.b;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntid = gs.ntid;
  const bool mp = !MIXED && V.comcut && tmass != nullptr;
  const bool qon = !MIXED && V.sq != nullptr && tq != nullptr;
  const int nout = SPLITQ ? TG : ntr;  // sums written per trial group
  if (mp) {
    for (int t = threadIdx.x; t < ntr; t += blockDim.x) {  // Get_COM, Compute_Max_COM_Distance
      double tm = 0.0, x = 0.0, y = 0.0, z = 0.0;
      for (int k = 0; k < ntid; ++k) {
        const int a = gs.tids[k];
        const double* tr = gs.trial[t] + 3 * a;
        tm += tmass[a];
        x += tmass[a] * tr[0];
        y += tmass[a] * tr[1];
        z += tmass[a] * tr[2];
      }
      const double cx = x / tm, cy = y / tm, cz = z / tm;
      double dmax = 0.0;
      for (int k = 0; k < ntid; ++k) {
        const double* tr = gs.trial[t] + 3 * gs.tids[k];
        const double dx = tr[0] - cx, dy = tr[1] - cy, dz = tr[2] - cz;
        dmax = fmax(dmax, dx * dx + dy * dy + dz * dz);
      }
      gs.tcom[t][0] = cx;
      gs.tcom[t][1] = cy;
      gs.tcom[t][2] = cz;
      gs.tcom[t][3] = sqrt(dmax);
    }
    __syncthreads();
  }
  const double rint0 = cbmc ? sqrt(b.rcut_cbmcsq) : V.rmax;
  if (MIXED && convert) {  // else the caller wrote gs.trialf
    for (int q = threadIdx.x; q < ntr * ntid * 3; q += blockDim.x) {
      const int t = q / (3 * ntid), r = q % (3 * ntid), a = gs.tids[r / 3];
      gs.trialf[t][3 * a + r % 3] = (float)gs.trial[t][3 * a + r % 3];
    }
    __syncthreads();
  }
  int s0 = -1, s1 = -1;
  if (skip_rec >= 0) {
    s0 = V.roff[skip_rec];
    s1 = s0 + gs.na;
  }
  const int nlv = *V.nlv;
  const float rlow2 = (float)b.rcut_lowsq, rc2 = cbmc ? (float)b.rcut_cbmcsq : (float)b.rcut_vdwsq;
  const bool tab = cbmc && b.tab_res > 0;
  const int ntypes = V.T->ntypes;
  const BoxF& bf = *V.bf;
  unsigned ovall = 0u;
  for (int t0 = 0; t0 < ntr; t0 += TG) {
    double accd[TG];
    float accf[TG];
#pragma unroll
    for (int u = 0; u < TG; ++u) {
      accd[u] = 0.0;
      accf[u] = 0.0f;
    }
    unsigned ovm = 0u;
    for (int i = threadIdx.x + V.crank * blockDim.x; i < nlv; i += blockDim.x * V.csize) {
      const int j = V.lv[i];
      if (j >= s0 && j < s1) continue;
      if (MIXED) {
        const float4 pj = V.lv32[i];
        const int tj = __float_as_int(pj.w);
        for (int k = 0; k < ntid; ++k) {
          const int a = gs.tids[k], ta = ttype[a];
          const bool has = ta >= 0 && tj >= 0;
          const int kk = has ? pidx(ta, tj, V.T->ntypes) : 0;
          const float eps = V.epsf[kk], s2 = V.sig2f[kk];
#pragma unroll
          for (int u = 0; u < TG; ++u) {
            if (t0 + u < ntr) {
              const float* tr = gs.trialf[t0 + u] + 3 * a;
              const float dx = fold(tr[0] - pj.x, b.hLf[0], b.Lf[0]);
              const float dy = fold(tr[1] - pj.y, b.hLf[1], b.Lf[1]);
              const float dz = fold(tr[2] - pj.z, b.hLf[2], b.Lf[2]);
              const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
              if (tab) {  // Estimate_MoleculePair_Energy from the FP32 table
                float et;
                const int kt = table_pair_f(bf.tab_v, bf.tab_f2, bf.tab_res, bf.tab_shift, bf.tab_rcs, bf.tab_step,
                                            bf.tab_inv_step, ntypes, r2, ta, tj, 0.0f, 0.0f, et);
                if (kt == 2) ovm |= 1u << u;
                else if (kt == 1) accf[u] += et;
              } else if (r2 < rlow2) {
                ovm |= 1u << u;
              } else if (r2 <= rc2 && has) {
                accf[u] += lj_pair_f(eps, s2, r2);
              }
            }
          }
        }
      } else {
        const double xj = V.sx[j], yj = V.sy[j], zj = V.sz[j];
        const double qj = qon ? V.sq[j] : 0.0;
        const int tj = V.lvt[i];
        unsigned inm = 0xffffffffu;  // trials whose molecule pair with j's molecule interacts
        if (mp) {
          const int rj = V.arec[j];
          const double mx = V.com[3 * rj], my = V.com[3 * rj + 1], mz = V.com[3 * rj + 2], md = V.rdcom[rj];
#pragma unroll
          for (int u = 0; u < TG; ++u) {
            if (t0 + u < ntr) {
              const double* c = gs.tcom[t0 + u];
              const double dx = fold(c[0] - mx, b.hL[0], b.L[0]);
              const double dy = fold(c[1] - my, b.hL[1], b.L[1]);
              const double dz = fold(c[2] - mz, b.hL[2], b.L[2]);
              if (sqrt(dx * dx + dy * dy + dz * dz) > rint0 + c[3] + md) inm &= ~(1u << u);
            }
          }
        }
        for (int k = 0; k < ntid; ++k) {
          const int a = gs.tids[k], ta = ttype[a];
          const double qa = qon ? tq[a] : 0.0;
#pragma unroll
          for (int u = 0; u < TG; ++u) {
            if (t0 + u < ntr && ((inm >> u) & 1u)) {
              const double* tr = gs.trial[t0 + u] + 3 * a;
              const double dx = fold(tr[0] - xj, b.hL[0], b.L[0]);
              const double dy = fold(tr[1] - yj, b.hL[1], b.L[1]);
              const double dz = fold(tr[2] - zj, b.hL[2], b.L[2]);
              const double r2 = dx * dx + dy * dy + dz * dz;
              if (tab) {  // Estimate_MoleculePair_Energy
                if (table_pair(b, ntypes, r2, ta, tj, qa, qj, accd[u]) == 2) ovm |= 1u << u;
              } else if (r2 < b.rcut_lowsq) {
                ovm |= 1u << u;
              } else {
                const int m = cutoff_mask(b, r2, cbmc);
                if (m & 1) accd[u] += vdw_pair(*V.T, b, ta, tj, r2, 1.0);
                if (qon && (m & 2)) accd[SPLITQ ? (u + TG / 2) % TG : u] += qq_pair_inter(b, qa * qj, r2);
              }
            }
          }
        }
      }
    }
    int which;
    if (MIXED) {
      const float tot = warp_multi_sum<TG>(accf, lane, which);
      if ((lane & (32 / TG - 1)) == 0 && t0 + which < ntr) {
        if (TG > 2) gs.partf[w * kMaxKappa + t0 + which] = tot;
        else gs.part[w * kMaxKappa + t0 + which] = (double)tot;
      }
    } else {
      const double tot = warp_multi_sum<TG>(accd, lane, which);
      if ((lane & (32 / TG - 1)) == 0 && t0 + which < nout) gs.part[w * kMaxKappa + t0 + which] = tot;
    }
    ovall |= __reduce_or_sync(0xffffffffu, ovm) << t0;
  }
  if (lane == 0) gs.povl[w] = (int)ovall;
  __syncthreads();
  constexpr bool kF = MIXED && TG > 2;  // FP32 to the end
  const int t = threadIdx.x;
  if (V.csize == 1) {
    if (t < nout) {
      int o = 0;
      for (int ww = 0; ww < kGcWarps; ++ww) o |= (gs.povl[ww] >> t) & 1;
      if (kF) {
        float e = 0.0f;
        for (int ww = 0; ww < kGcWarps; ++ww) e += gs.partf[ww * kMaxKappa + t];
        gs.ef[t] = o ? 0.0f : e;
      } else {
        double e = 0.0;
        for (int ww = 0; ww < kGcWarps; ++ww) e += gs.part[ww * kMaxKappa + t];
        gs.e[t] = o ? 0.0 : e;
        if (MIXED) gs.ef[t] = o ? 0.0f : (float)e;
      }
      gs.ov[t] = o;
    }
  } else {
    // this CTA's sums, then the cluster's in rank order
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    const int buf = gs.cbuf;
    if (t < nout) {
      int o = 0;
      for (int ww = 0; ww < kGcWarps; ++ww) o |= (gs.povl[ww] >> t) & 1;
      if (kF) {
        float e = 0.0f;
        for (int ww = 0; ww < kGcWarps; ++ww) e += gs.partf[ww * kMaxKappa + t];
        gs.cpartf[buf][t] = e;
      } else {
        double e = 0.0;
        for (int ww = 0; ww < kGcWarps; ++ww) e += gs.part[ww * kMaxKappa + t];
        gs.cpart[buf][t] = e;
      }
      gs.covl[buf][t] = o;
    }
    cl.sync();
    if (t < nout) {
      int o = 0;
      for (int r = 0; r < V.csize; ++r) o |= *cl.map_shared_rank(&gs.covl[buf][t], r);
      if (kF) {
        float e = 0.0f;
        for (int r = 0; r < V.csize; ++r) e += *cl.map_shared_rank(&gs.cpartf[buf][t], r);
        gs.ef[t] = o ? 0.0f : e;
      } else {
        double e = 0.0;
        for (int r = 0; r < V.csize; ++r) e += *cl.map_shared_rank(&gs.cpart[buf][t], r);
        gs.e[t] = o ? 0.0 : e;
        if (MIXED) gs.ef[t] = o ? 0.0f : (float)e;
      }
      gs.ov[t] = o;
    }
  }
  __syncthreads();
  if (t == 0) gs.cbuf ^= 1;
}

// charges of the intermolecular CBMC trial terms of species is: only with
// L_Coul_CBMC (Compute_MoleculePair_Energy, energy_routines.f90:1684-1686)
__device__ __forceinline__ const double* gc_cbmc_q(const GcArgs& A, int is) {
  return A.sp[is].l_coul_cbmc ? A.sp[is].q : nullptr;
}

// the live-atom list and the sorted live records (thread 0)
template <bool MIXED>
__device__ void list_add(const GcView& V, int* nlv, int r, int na, const int* types) {
  for (int a = 0; a < na; ++a) {
    const int j = V.roff[r] + a, i = (*nlv)++;
    V.apos[j] = i;
    V.lv[i] = j;
    if (MIXED) V.lv32[i] = make_float4((float)V.sx[j], (float)V.sy[j], (float)V.sz[j], __int_as_float(types[a]));
    else V.lvt[i] = types[a];
  }
}

template <bool MIXED>
__device__ void list_remove(const GcView& V, int* nlv, int r, int na) {
  for (int a = 0; a < na; ++a) {
    const int j = V.roff[r] + a, i = V.apos[j], last = --(*nlv);
    if (i != last) {
      const int jl = V.lv[last];
      V.lv[i] = jl;
      V.apos[jl] = i;
      if (MIXED) V.lv32[i] = V.lv32[last];
      else V.lvt[i] = V.lvt[last];
    }
    V.apos[j] = -1;
  }
}

// n: live records of the species before the change
__device__ void lrec_insert(int* lrec, int base, int n, int r) {
  int p = n;
  while (p > 0 && lrec[base + p - 1] > r) {
    lrec[base + p] = lrec[base + p - 1];
    --p;
  }
  lrec[base + p] = r;
}

__device__ void lrec_remove(int* lrec, int base, int n, int r) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (lrec[base + mid] < r) lo = mid + 1;
    else hi = mid;
  }
  for (int p = lo; p + 1 < n; ++p) lrec[base + p] = lrec[base + p + 1];
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
    batch_energies<MIXED, 16>(V, gs, kd, gs.rec, true, S.type, true, S.mass, gc_cbmc_q(A, gs.is));
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
  batch_energies<MIXED, 16>(V, gs, ki, gs.rec, true, S.type, true, S.mass, gc_cbmc_q(A, gs.is));
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
// block-wide) plus intra and bonded (thread 0); results in out[0..9]: ev, eq,
// eb, ea, ed, ei, eiv, eiq, then the two parts of eq (the intermolecular
// real-space sum and the periodic part of the intramolecular one); overlap
// flags (inter, intra) in ovs
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
  const bool qon = !MIXED && V.sq != nullptr;
  if constexpr (!MIXED) {
    if (qon) batch_energies<false, 2, true>(V, gs, 1, gs.rec, false, ttype, true, A.sp[gs.is].mass, A.sp[gs.is].q);
    else batch_energies<false, 2>(V, gs, 1, gs.rec, false, ttype, true, A.sp[gs.is].mass);
  } else {
    batch_energies<true, 2>(V, gs, 1, gs.rec, false, ttype, true, A.sp[gs.is].mass);
  }
  if (threadIdx.x == 0) {
    IntraOut io{0, 0, 0, 0, 0, 0, 0, false};
    if (with_intra) io = molecule_intra(A.P, gs.is, *V.b, *V.T, gs.r);
    const double eqx = qon ? gs.e[1] : 0.0;
    out[0] = gs.e[0];
    out[1] = qon ? eqx + io.pqq : io.pqq;  // with the periodic part of the intramolecular Coulomb sum
    out[8] = eqx;
    out[9] = io.pqq;
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

// Reciprocal-space energy of a charged box after a move of the molecule in
// slot `slot` (Update_System_Ewald_Reciprocal_Energy, energy_routines.f90:
// 2384-2431): mode 0 adds the structure factors of the new molecule r
// (int_insertion), 1 takes the molecule's stored factors out (int_deletion),
// 2 replaces them by those of r (int_translation, int_rotation, int_intra).
// All threads; k-vector k stays with thread k mod blockDim.x, which writes the
// molecule's new factors to G.new_cos / G.new_sin.  Returns CHARGE_FACTOR
// sum_k Cn (S_c^2 + S_s^2) on every thread (red: one double per warp).
__device__ double gc_recip(const GcBox& G, const GcSpecies& s, const double* r, int slot, int mode, double* red) {
  const double* cm = G.cos_mol + (size_t)slot * G.stride;
  const double* smv = G.sin_mol + (size_t)slot * G.stride;
  double part = 0.0;
  for (int k = threadIdx.x; k < G.nvecs; k += blockDim.x) {
    const double4_32a h = G.kvec[k];
    double cn = 0.0, sn = 0.0;
    if (mode != 1)
      for (int a = 0; a < s.natoms; ++a) {
        const double hdotr = h.x * r[3 * a] + h.y * r[3 * a + 1] + h.z * r[3 * a + 2];
        double sv, cv;
        sincos(hdotr, &sv, &cv);
        cn = cn + s.q[a] * cv;
        sn = sn + s.q[a] * sv;
      }
    double c, sm;
    if (mode == 0) {
      c = G.cos_sum[k] + cn;
      sm = G.sin_sum[k] + sn;
    } else if (mode == 1) {
      c = G.cos_sum[k] - cm[k];
      sm = G.sin_sum[k] - smv[k];
    } else {
      c = G.cos_sum[k] + (cn - cm[k]);
      sm = G.sin_sum[k] + (sn - smv[k]);
    }
    part += h.w * (c * c + sm * sm);
    if (mode != 1) {
      G.new_cos[k] = cn;
      G.new_sin[k] = sn;
    }
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  double e = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) e += red[w];
  __syncthreads();  // red is free again
  return e * kCHARGE_FACTOR;
}

// the accepted move of gc_recip: the box's sums and the molecule's row
__device__ void gc_recip_commit(const GcBox& G, int slot, int mode) {
  double* cm = G.cos_mol + (size_t)slot * G.stride;
  double* smv = G.sin_mol + (size_t)slot * G.stride;
  for (int k = threadIdx.x; k < G.nvecs; k += blockDim.x) {
    if (mode == 0) {
      G.cos_sum[k] = G.cos_sum[k] + G.new_cos[k];
      G.sin_sum[k] = G.sin_sum[k] + G.new_sin[k];
    } else if (mode == 1) {
      G.cos_sum[k] = G.cos_sum[k] - cm[k];
      G.sin_sum[k] = G.sin_sum[k] - smv[k];
    } else {
      G.cos_sum[k] = G.cos_sum[k] + (G.new_cos[k] - cm[k]);
      G.sin_sum[k] = G.sin_sum[k] + (G.new_sin[k] - smv[k]);
    }
    if (mode != 1) {
      cm[k] = G.new_cos[k];
      smv[k] = G.new_sin[k];
    }
  }
}

// Compute_Molecule_Self_Energy (energy_routines.f90:2606-2645), Ewald sum
__device__ __forceinline__ double gc_self(const GcSpecies& s, const BoxDev& b) {
  double qq = 0.0;
  for (int a = 0; a < s.natoms; ++a) qq += s.q[a] * s.q[a];
  return -qq * kCHARGE_FACTOR * b.alpha / kROOTPI;
}

// Compute_LR_Correction (energy_routines.f90:2956-3023) for type counts nb,
// with the per-pair coefficients computed on the host
__device__ double gc_lrc(const GcBox& G, int ntypes, const double* nb) {
  double e = 0.0;
  for (int ia = 0; ia < ntypes; ++ia) {
    double eij = 0.0;
    for (int ja = 0; ja < ntypes; ++ja) eij = eij + nb[ja] * G.lrc_c[ia * ntypes + ja];
    e = e + nb[ia] * eij;
  }
  return G.lrc_pref * e;
}


// ---------------------------------------------------------------------------
// FP32 CBMC growth of the mixed kernel: the steps of gc_fragment_order,
// gc_place_fragments and gc_build with FP32 geometry, draws (top 23 bits of
// the same lfsr258 numbers), trial intramolecular energies and Boltzmann
// weights (shifted by the lowest trial energy).  ln P_bias is accumulated in
// FP32; the acceptance exponent it enters is formed in FP64.

// weights of k trials with energies u (ovm: overlapping trials), the rule
// "rand * sum < cumulative sum" with pick = rand (pick < 0: no draw, trial 0)
// and ln of the weight sum shifted by the lowest energy: returns the trial,
// -1 if all overlap; *dlnw = beta (U_sel - U_min) + ln sum exp(-beta (U - U_min))
__device__ __forceinline__ int gc_select_f(int k, const float* u, unsigned ovm, float beta, Lfsr& rng, bool del,
                                           float* dlnw) {
  float umin = 3.0e38f;
  for (int t = 0; t < k; ++t)
    if (!((ovm >> t) & 1u)) umin = fminf(umin, u[t]);
  if (umin == 3.0e38f) return -1;
  float w[kMaxKappa];
  float cum = 0.0f;
  for (int t = 0; t < k; ++t) {
    cum += ((ovm >> t) & 1u) ? 0.0f : __expf(-beta * (u[t] - umin));
    w[t] = cum;
  }
  int sel = 0;
  if (!del) {
    const float x = draw_f(rng) * cum;
    while (sel < k && !(x < w[sel])) ++sel;
    if (sel == k) return -1;
  }
  *dlnw = beta * (u[sel] - umin) + __logf(cum);
  return sel;
}

// Fragment_Order (fragment_growth.f90:1317-1446), FP32; thread 0
__device__ void gc_fragment_order_f(const WidomSpecies& S, GrowState& gs, GrowF& g, unsigned live, Lfsr& rng) {
  const int f0 = gs.order[0];
  int hang[kMaxFrags];
  int nh = 0;
  for (int k = 0; k < S.frag_nconnect[f0]; ++k) {
    const int f = S.frag_connect[f0][k];
    if (!((live >> f) & 1u)) hang[nh++] = f;
  }
  while (nh > 0) {
    float tot = 0.0f;
    for (int k = 0; k < nh; ++k) tot += (float)(S.frag_natoms[hang[k]] - 2);
    const float u = draw_f(rng);
    int k = 0;
    float cum = 0.0f;
    for (; k < nh; ++k) {
      cum += (float)(S.frag_natoms[hang[k]] - 2) / tot;
      if (u < cum) break;
    }
    if (k >= nh) k = nh - 1;
    const int f = hang[k];
    if (nh > 1) g.ln_pseq += __logf((float)(S.frag_natoms[f] - 2) / tot);
    gs.order[gs.norder++] = f;
    live |= 1u << f;
    for (int q = k; q + 1 < nh; ++q) hang[q] = hang[q + 1];
    --nh;
    for (int q = 0; q < S.frag_nconnect[f]; ++q) {
      const int h = S.frag_connect[f][q];
      if (!((live >> h) & 1u) && nh < kMaxFrags) hang[nh++] = h;
    }
  }
}

// Cut_Regrow (fragment_growth.f90:1118-1312) masks; thread 0
__device__ void gc_cut_f(const WidomSpecies& S, GrowState& gs, GrowF& g) {
  gs.exist = (1u << S.natoms) - 1u;
  gs.placed = (1u << S.nfrag) - 1u;
  for (int k = 0; k < gs.norder; ++k) {
    const int f = gs.order[k];
    gs.placed &= ~(1u << f);
    for (int j = 0; j < S.frag_natoms[f]; ++j) gs.exist &= ~(1u << S.frag_atoms[f][j]);
  }
  gs.exist |= 1u << S.frag_atoms[gs.f_live][0];
  gs.exist |= 1u << S.frag_atoms[gs.f_dead][0];
  g.ln_pbias = 0.0f;
  gs.flag = 0;
}

// Fragment_Placement (fragment_growth.f90:1449-2132) for gs.order[first..], FP32; all threads
__device__ bool gc_place_fragments_f(const GcArgs& A, const GcView& V, GrowState& gs, GrowF& g, int first, bool del,
                                     Lfsr& rng) {
  const WidomSpecies& S = A.S;
  const SpeciesF& F = A.SF;
  const BoxF& bf = *V.bf;
  const int kd = S.kappa_dih;
  for (int oi = first; oi < gs.norder; ++oi) {
    if (threadIdx.x == 0) {
      const int f = gs.order[oi];
      const int nf = S.frag_natoms[f];
      const unsigned grown = gs.exist;
      for (int i = 0; i < 3 * kMaxAtoms; ++i) g.cfg[i] = 0.0f;
      if (del) {
        for (int j = 0; j < nf; ++j) {
          const int a = S.frag_atoms[f][j];
          gs.exist |= 1u << a;
          for (int d = 0; d < 3; ++d) g.cfg[3 * a + d] = g.r[3 * a + d];
        }
      } else {
        const int nconf = S.nconfig[f];
        int cf = (int)(draw_f(rng) * (float)nconf);
        cf = (int)(draw_f(rng) * (float)nconf);  // the duplicated draw of fragment_growth.f90:1578,1584
        if (cf >= nconf) cf = nconf - 1;
        const float* L = A.libf + S.lib_off[f] + (size_t)cf * nf * 3;
        for (int j = 0; j < nf; ++j) {
          const int a = S.frag_atoms[f][j];
          gs.exist |= 1u << a;
          for (int d = 0; d < 3; ++d) g.cfg[3 * a + d] = L[3 * j + d];
        }
      }
      gs.combined = gs.exist;
      gs.newex = gs.combined & ~grown;
      int fc = -1;
      for (int q = 0; q < S.frag_nconnect[f]; ++q) {
        const int h = S.frag_connect[f][q];
        if ((gs.placed >> h) & 1u) {
          fc = h;
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
        float v1[3], v2[3], al_i[9], hg_i[9], al_c[9], hg_c[9];
        for (int d = 0; d < 3; ++d) {
          v1[d] = g.cfg[3 * anc_i + d] - g.cfg[3 * anc_c + d];
          v2[d] = g.cfg[3 * atom_ifrag + d] - g.cfg[3 * anc_c + d];
        }
        aligner_hanger_f(v1, v2, al_i, hg_i);
        if (!del) {
          for (int d = 0; d < 3; ++d) {
            v1[d] = g.r[3 * anc_i + d] - g.r[3 * anc_c + d];
            v2[d] = g.r[3 * atom_fc + d] - g.r[3 * anc_c + d];
          }
          aligner_hanger_f(v1, v2, al_c, hg_c);
        }
        const float tx = g.cfg[3 * anc_c], ty = g.cfg[3 * anc_c + 1], tz = g.cfg[3 * anc_c + 2];
        for (int j = 0; j < nf; ++j) {
          const int a = S.frag_atoms[f][j];
          const float x = g.cfg[3 * a] - tx, y = g.cfg[3 * a + 1] - ty, z = g.cfg[3 * a + 2] - tz;
          g.cfg[3 * a] = x * al_i[0] + y * al_i[1] + z * al_i[2];
          g.cfg[3 * a + 1] = x * al_i[3] + y * al_i[4] + z * al_i[5];
          g.cfg[3 * a + 2] = x * al_i[6] + y * al_i[7] + z * al_i[8];
        }
        if (del) {
          g.theta0 = 0.0f;
          for (int i = 0; i < 9; ++i) g.hg[i] = hg_i[i];
        } else {
          g.theta0 = (float)kTWOPI * draw_f(rng);
          for (int i = 0; i < 9; ++i) g.hg[i] = hg_c[i];
        }
      }
    }
    __syncthreads();
    if (gs.flag) return true;
    // trial geometry, intramolecular and dihedral energies: trial ii on lane ii of warp 0
    if (threadIdx.x < kd) {
      const int ii = threadIdx.x;
      const float theta = g.theta0 + (float)ii * ((float)kTWOPI / (float)kd);
      float sth, cth;
      sincosf(theta, &sth, &cth);
      float r[3 * kMaxAtoms];
      for (int i = 0; i < 3 * S.natoms; ++i) r[i] = g.r[i];
      const int f = gs.order[oi];
      const float ax = g.r[3 * gs.anc_c], ay = g.r[3 * gs.anc_c + 1], az = g.r[3 * gs.anc_c + 2];
      for (int j = 0; j < S.frag_natoms[f]; ++j) {
        const int a = S.frag_atoms[f][j];
        if (a == gs.anc_i || a == gs.anc_c) continue;
        const float x = g.cfg[3 * a], y = g.cfg[3 * a + 1], z = g.cfg[3 * a + 2];
        const float yr = cth * y + sth * z, zr = -sth * y + cth * z;
        r[3 * a] = (x * g.hg[0] + yr * g.hg[1] + zr * g.hg[2]) + ax;
        r[3 * a + 1] = (x * g.hg[3] + yr * g.hg[4] + zr * g.hg[5]) + ay;
        r[3 * a + 2] = (x * g.hg[6] + yr * g.hg[7] + zr * g.hg[8]) + az;
      }
      for (int i = 0; i < 3 * S.natoms; ++i) gs.trialf[ii][i] = r[i];
      unsigned ex = gs.combined & ~gs.idmask;
      float niv = 0.0f, niq = 0.0f, noq = 0.0f;
      bool ov = false;
      for (int k = 0; k < gs.ntid && !ov; ++k) {
        ex |= 1u << gs.tids[k];
        float eiv, eiq, eoq;
        ov = atom_intra_f(F, bf, V.ljp, gs.tids[k], r, ex, eiv, eiq, eoq);
        niv += eiv;
        niq += eiq;
        noq += eoq;
      }
      gs.dov[ii] = ov ? 1 : 0;
      g.dd[ii] = ov ? 0.0f : dihedral_f(F, r, gs.combined);
      g.dn[ii] = niv + niq + noq;  // completed with the inter and dihedral energies below
    }
    __syncthreads();
    // inter energies of the new atoms (Compute_Molecule_Nonbond_Inter_Energy with new_exist)
    if (threadIdx.x == 0) {
      gs.ntid = 0;
      for (int a = 0; a < S.natoms; ++a)
        if ((gs.newex >> a) & 1u) gs.tids[gs.ntid++] = a;
    }
    __syncthreads();
    batch_energies<true, 16>(V, gs, kd, gs.rec, true, S.type, false);
    if (threadIdx.x == 0) {
      unsigned ovm = 0u;
      float u[kMaxKappa];
      for (int ii = 0; ii < kd; ++ii) {
        u[ii] = 0.0f;
        bool ov = gs.dov[ii] || gs.ov[ii];
        if (!ov) {
          u[ii] = g.dd[ii] + g.dn[ii] + gs.ef[ii] - g.e_prev;
          if (u[ii] >= bf.kmaxE) ov = true;
        }
        if (ov) {
          ovm |= 1u << ii;
          gs.dov[ii] = 1;
        }
      }
      float dlnw = 0.0f;
      const int tr = gc_select_f(kd, u, ovm, bf.beta, rng, del, &dlnw);
      if (tr < 0) {
        gs.flag = 1;
      } else {
        g.ln_pbias = g.ln_pbias - dlnw;
        const int f = gs.order[oi];
        for (int j = 0; j < S.frag_natoms[f]; ++j) {
          const int a = S.frag_atoms[f][j];
          if (a != gs.anc_i && a != gs.anc_c)
            for (int d = 0; d < 3; ++d) g.r[3 * a + d] = gs.trialf[tr][3 * a + d];
        }
        g.e_prev = g.dd[tr];
        gs.placed |= 1u << f;
        gs.exist = gs.combined;
      }
    }
    __syncthreads();
    if (gs.flag) return true;
  }
  return false;
}

// Build_Molecule (fragment_growth.f90:72-707) for record gs.rec, FP32; all threads
__device__ bool gc_build_f(const GcArgs& A, const GcView& V, GrowState& gs, GrowF& g, bool del, Lfsr& rng) {
  const WidomSpecies& S = A.S;
  const SpeciesF& F = A.SF;
  const BoxF& bf = *V.bf;
  const int ki = S.kappa_ins;
  if (threadIdx.x == 0) {
    g.ln_pbias = 0.0f;
    gs.exist = 0u;
    gs.flag = 0;
    const float u = draw_f(rng);
    int fstart = 0;
    while (fstart < S.nfrag && !(u < F.cum_prob_ins[fstart])) ++fstart;
    if (fstart >= S.nfrag) fstart = S.nfrag - 1;
    g.ln_pseq = (float)S.ln_prob_ins[fstart];
    gs.order[0] = fstart;
    gs.norder = 1;
    if (S.nfrag > 1) gc_fragment_order_f(S, gs, g, 1u << fstart, rng);
    const int nfa = S.frag_natoms[fstart];
    if (!del) {
      const int nconf = S.nconfig[fstart];
      int conf = (int)(draw_f(rng) * (float)nconf);
      if (conf >= nconf) conf = nconf - 1;
      const float* L0 = A.libf + S.lib_off[fstart] + (size_t)conf * nfa * 3;
      for (int i = 0; i < nfa; ++i)
        for (int d = 0; d < 3; ++d) g.r[3 * S.frag_atoms[fstart][i] + d] = L0[3 * i + d];
    }
    gs.ntid = nfa;
    for (int i = 0; i < nfa; ++i) {
      gs.tids[i] = S.frag_atoms[fstart][i];
      gs.exist |= 1u << gs.tids[i];
    }
    get_com_f(F, g.r, gs.exist, g.com);
    if (!del) {  // Rotate_Molecule_Eulerian
      const float theta = acosf(1.0f - 2.0f * draw_f(rng));
      const float phi = (1.0f - 2.0f * draw_f(rng)) * (float)kPI;
      const float psi = (1.0f - 2.0f * draw_f(rng)) * (float)kPI;
      float st, ct, sp, cp, ss, cs;
      sincosf(theta, &st, &ct);
      sincosf(phi, &sp, &cp);
      sincosf(psi, &ss, &cs);
      const float r11 = cs * cp - ct * sp * ss, r12 = cs * sp + ct * cp * ss, r13 = ss * st;
      const float r21 = -ss * cp - ct * sp * cs, r22 = -ss * sp + ct * cp * cs, r23 = cs * st;
      const float r31 = st * sp, r32 = -st * cp, r33 = ct;
      for (int i = 0; i < nfa; ++i) {
        const int a = gs.tids[i];
        const float x = g.r[3 * a] - g.com[0], y = g.r[3 * a + 1] - g.com[1], z = g.r[3 * a + 2] - g.com[2];
        g.r[3 * a] = (r11 * x + r12 * y + r13 * z) + g.com[0];
        g.r[3 * a + 1] = (r21 * x + r22 * y + r23 * z) + g.com[1];
        g.r[3 * a + 2] = (r31 * x + r32 * y + r33 * z) + g.com[2];
      }
    }
    for (int it = 0; it < ki; ++it) {
      if (del && it == 0) {
        g.draws[0] = g.com[0];
        g.draws[1] = g.com[1];
        g.draws[2] = g.com[2];
      } else {
        g.draws[3 * it] = (0.5f - draw_f(rng)) * bf.L[0];
        g.draws[3 * it + 1] = (0.5f - draw_f(rng)) * bf.L[1];
        g.draws[3 * it + 2] = (0.5f - draw_f(rng)) * bf.L[2];
      }
    }
  }
  __syncthreads();
  // trial positions: rtrial(0) - COM + anchor
  for (int q = threadIdx.x; q < ki * gs.ntid; q += blockDim.x) {
    const int it = q / gs.ntid, a = gs.tids[q % gs.ntid];
    for (int d = 0; d < 3; ++d) gs.trialf[it][3 * a + d] = g.r[3 * a + d] - g.com[d] + g.draws[3 * it + d];
  }
  __syncthreads();
  batch_energies<true, 16>(V, gs, ki, gs.rec, true, S.type, false);
  if (threadIdx.x == 0) {
    unsigned ovm = 0u;
    float u[kMaxKappa];
    for (int it = 0; it < ki; ++it) {
      u[it] = gs.ef[it];
      if (gs.ov[it] || u[it] >= bf.kmaxE) ovm |= 1u << it;
    }
    float dlnw = 0.0f;
    const int sel = gc_select_f(ki, u, ovm, bf.beta, rng, del, &dlnw);
    if (sel < 0) {
      gs.flag = 1;
    } else {
      g.ln_pbias = g.ln_pbias - dlnw;
      for (int k = 0; k < gs.ntid; ++k) {
        const int a = gs.tids[k];
        for (int d = 0; d < 3; ++d) g.r[3 * a + d] = gs.trialf[sel][3 * a + d];
      }
      for (int d = 0; d < 3; ++d) g.com[d] = g.draws[3 * sel + d];
      g.e_prev = dihedral_f(F, g.r, gs.exist);
      gs.placed = 1u << gs.order[0];
    }
  }
  __syncthreads();
  if (gs.flag) return true;
  if (gc_place_fragments_f(A, V, gs, g, 1, del, rng)) return true;
  if (threadIdx.x == 0 && gs.norder > 1) get_com_f(F, g.r, gs.exist, g.com);
  __syncthreads();
  return false;
}

// energies of the whole molecule g.r (record gs.rec), FP32 geometry: inter
// (full cutoffs, block-wide) plus intra and bonded (thread 0); out[0..7] as
// gc_mol_energies
__device__ void gc_mol_energies_f(const GcArgs& A, const GcView& V, GrowState& gs, GrowF& g, const int* ttype,
                                  double* out, int* ovs) {
  if (threadIdx.x == 0) {
    gs.ntid = gs.na;
    for (int a = 0; a < gs.na; ++a) {
      gs.tids[a] = a;
      for (int d = 0; d < 3; ++d) gs.trialf[0][3 * a + d] = g.r[3 * a + d];
    }
  }
  __syncthreads();
  batch_energies<true, 2>(V, gs, 1, gs.rec, false, ttype, false);
  if (threadIdx.x == 0) {
    const IntraF io = molecule_intra_f(A.SF, *V.bf, V.ljp, g.r);
    out[0] = gs.e[0];
    out[1] = io.pqq;
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

// Fold_Molecule of g (FP32); thread 0
__device__ __forceinline__ void gc_fold_f(const BoxF& bf, GrowF& g, int na) {
  for (int k = 0; k < 3; ++k) {
    float sh = 0.0f;
    if (g.com[k] > bf.hL[k]) sh = -bf.L[k];
    else if (g.com[k] < -bf.hL[k]) sh = bf.L[k];
    if (sh != 0.0f) {
      g.com[k] += sh;
      for (int a = 0; a < na; ++a) g.r[3 * a + k] += sh;
    }
  }
}

// min((int)(u n) + 1, n) for a uniform draw u (the molecule pick of the
// move routines); the mixed kernel takes u from the top 23 bits
template <bool MIXED>
__device__ __forceinline__ int gc_pick(Lfsr& rng, int n) {
  if constexpr (MIXED) return min((int)(draw_f(rng) * (float)n) + 1, n);
  else return min((int)(rng.next() * n) + 1, n);
}

// a draw whose value is not used (the box and species choices of the reference)
template <bool MIXED>
__device__ __forceinline__ void gc_skip_draw(Lfsr& rng) {
  if constexpr (MIXED) rng.next_bits();
  else (void)rng.next();
}

// The box view of a grand-canonical kernel (one box per CTA, or per cluster):
// the box constants, the pair table and the FP32 tables in shared memory, the
// records' atoms and COMs, the live-atom list and the sorted live records in
// dynamic shared memory `smem` (gc_smem_bytes).  All threads; ends with a barrier.
template <bool MIXED>
__device__ void gc_setup(const GcArgs& A, const GcBox& G, const PairTable& T, int csize, int crank,
                         unsigned char* smem, BoxDev& b, BoxF& bf, PairTable& sT, float2* s_ljp, float* s_epsf,
                         float* s_sig2f, int* rs0, int& s_nlv, int* ttype, GcView& V) {
  if (threadIdx.x == 0) {
    b = G.b;
    if (MIXED) {  // FP32 box constants
      for (int d = 0; d < 3; ++d) {
        bf.L[d] = (float)G.b.L[d];
        bf.hL[d] = (float)G.b.hL[d];
        bf.cinv[d] = 0.0f;
        bf.nc[d] = 1;
      }
      bf.rcb2 = (float)G.b.rcut_cbmcsq;
      bf.rv2 = (float)G.b.rcut_vdwsq;
      bf.rq2 = (float)G.b.rcut_coulsq;
      bf.low2 = (float)G.b.rcut_lowsq;
      bf.rc_cbmc = (float)sqrt(G.b.rcut_cbmcsq);
      bf.rc_full = (float)sqrt(G.b.rcut_vdwsq);
      bf.beta = (float)G.b.beta;
      bf.kmaxE = (float)(kMAX_KBT / G.b.beta);
      bf.alpha = (float)G.b.alpha;
      bf.charge_on = 0;
    }
  }
  {
    const int* src = reinterpret_cast<const int*>(&T);
    int* dst = reinterpret_cast<int*>(&sT);
    for (int i = threadIdx.x; i < (int)(sizeof(PairTable) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  }
  if (MIXED) boxf_options(bf, G.b, T.ntypes);
  for (int i = threadIdx.x; i < kMaxTypes * kMaxTypes; i += blockDim.x) {
    const int ta = i / kMaxTypes, tb = i % kMaxTypes;
    const bool ok = ta < T.ntypes && tb < T.ntypes;
    s_ljp[i] = ok ? make_float2(T.epsf[ta * T.ntypes + tb], T.sig2f[ta * T.ntypes + tb]) : make_float2(0.f, 0.f);
  }
  const int N = G.natoms, R = G.nrec;
  double* sx = reinterpret_cast<double*>(smem);
  double* sy = sx + N;
  double* sz = sy + N;
  double* scom = sz + N;  // [R][3]
  int* lv = reinterpret_cast<int*>(scom + 3 * R);
  int* apos = lv + N;
  int* lvt = apos + N;  // FP64 kernel only
  int* rlive = lvt + (MIXED ? 0 : N);
  int* rsp = rlive + R;
  int* roff = rsp + R;
  int* pool = roff + R;
  int* lrec = pool + R;
  float4* lv32 = reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(smem) +
                                           ((((size_t)(lrec + R) - (size_t)smem) + 15) & ~(size_t)15));
  // molecule-pair cutoff boxes only: per record max_dcom, the record of each atom
  double* rdcom = nullptr;
  int* arec = nullptr;
  if (G.comcut) {
    rdcom = reinterpret_cast<double*>(lv32 + (MIXED ? N : 0));
    arec = reinterpret_cast<int*>(rdcom + R);
  }
  // charged boxes only: the charge of each atom (after the optional arrays)
  double* sq = nullptr;
  if (!MIXED && G.qon) {
    const size_t o = (size_t)(G.comcut ? reinterpret_cast<unsigned char*>(arec + N)
                                       : reinterpret_cast<unsigned char*>(lv32)) - (size_t)smem;
    sq = reinterpret_cast<double*>(smem + ((o + 15) & ~(size_t)15));
  }
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double4_32a p = G.xyzq[j];
    sx[j] = p.x;
    sy[j] = p.y;
    sz[j] = p.z;
    if (sq) sq[j] = p.w;
    apos[j] = -1;
  }
  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    const int4 ri = G.rec[r];
    rlive[r] = ri.w;
    rsp[r] = ri.y;
    roff[r] = ri.z;
  }
  for (int k = threadIdx.x; k < G.npool; k += blockDim.x) pool[k] = G.pool[k];
  for (int k = threadIdx.x; k < kMaxTypes * kMaxTypes; k += blockDim.x) {
    s_epsf[k] = T.epsf[k];
    s_sig2f[k] = T.sig2f[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // the list of live atoms (record order) and the sorted live records per
    // species (records are in slot order, so each species is one range)
    int n = 0;
    for (int k = 0; k < kGcMaxSpecies; ++k) rs0[k] = 0;
    for (int r = R - 1; r >= 0; --r) rs0[rsp[r]] = r;
    int cnt[kGcMaxSpecies] = {0};
    for (int r = 0; r < R; ++r) {
      if (!rlive[r]) continue;
      const int sp = rsp[r];
      lrec[rs0[sp] + cnt[sp]++] = r;
      for (int a = 0; a < A.sp[sp].natoms; ++a) {
        const int j = roff[r] + a;
        apos[j] = n;
        lv[n++] = j;
      }
    }
    s_nlv = n;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < s_nlv; i += blockDim.x) {
    const int j = lv[i];
    const int tj = G.atype[j];
    if (MIXED) lv32[i] = make_float4((float)sx[j], (float)sy[j], (float)sz[j], __int_as_float(tj));
    else lvt[i] = tj;
  }
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
    if (G.comcut) {
      double dmax = 0.0;  // Compute_Max_COM_Distance
      for (int a = 0; a < s.natoms; ++a) {
        const int j = roff[r] + a;
        arec[j] = r;
        const double dx = sx[j] - scom[3 * r], dy = sy[j] - scom[3 * r + 1], dz = sz[j] - scom[3 * r + 2];
        dmax = fmax(dmax, dx * dx + dy * dy + dz * dz);
      }
      rdcom[r] = sqrt(dmax);
    }
  }
  if (threadIdx.x < kMaxAtoms) ttype[threadIdx.x] = threadIdx.x < A.S.natoms ? A.S.type[threadIdx.x] : -1;
  V.b = &b;
  V.T = &sT;
  V.epsf = s_epsf;
  V.sig2f = s_sig2f;
  V.bf = &bf;
  V.ljp = s_ljp;
  V.sx = sx;
  V.sy = sy;
  V.sz = sz;
  V.lv = lv;
  V.apos = apos;
  V.lvt = lvt;
  V.lv32 = lv32;
  V.rlive = rlive;
  V.rsp = rsp;
  V.roff = roff;
  V.lrec = lrec;
  V.nlv = &s_nlv;
  V.com = scom;
  V.rdcom = rdcom;
  V.arec = arec;
  V.sq = sq;
  V.comcut = G.comcut;
  V.rmax = G.rmax;
  V.natoms = N;
  V.nrec = R;
  V.crank = crank;
  V.csize = csize;
  __syncthreads();
}

template <bool MIXED>
__global__ void __launch_bounds__(kGcThreads, 1) k_gcmc(GcArgs A, GcBox* boxes, PairTable T, int csize) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BoxDev b;
  __shared__ GrowState gs;
  __shared__ double em[10];
  __shared__ int eov[2];
  __shared__ int mv_kind, mv_rec, mv_is, mv_skip, mv_acc, mv_stop, s_nlv;
  __shared__ int mv_slot, mv_ew;  // the molecule's slot; the accepted structure-factor update (-1: none)
  __shared__ double s_red[kGcWarps];
  __shared__ int rs0[kGcMaxSpecies];
  __shared__ double old_r[3 * kMaxAtoms], old_com[3];
  __shared__ int ttype[kMaxAtoms];
  __shared__ float s_epsf[kMaxTypes * kMaxTypes], s_sig2f[kMaxTypes * kMaxTypes];
  __shared__ double rg_new[3 * kMaxAtoms], rg_new_com[3], rg_en[8], rg_e_prev, rg_ln_pfor;
  __shared__ GrowF gf;
  __shared__ BoxF bf;
  __shared__ float2 s_ljp[kMaxTypes * kMaxTypes];
  __shared__ PairTable sT;  // the pair table in shared memory (its address is passed to device functions)
  __shared__ float rgf_new[3 * kMaxAtoms], rgf_new_com[3], rgf_e_prev, rgf_ln_pfor;
  const int crank = (int)(blockIdx.x % (unsigned)csize);
  GcBox& G = boxes[blockIdx.x / csize];
  if (threadIdx.x == 0) gs.cbuf = 0;
  GcView V;
  gc_setup<MIXED>(A, G, T, csize, crank, smem, b, bf, sT, s_ljp, s_epsf, s_sig2f, rs0, s_nlv, ttype, V);
  const int N = G.natoms, R = G.nrec;
  double* sx = V.sx;
  double* sy = V.sy;
  double* sz = V.sz;
  double* scom = V.com;
  double* rdcom = V.rdcom;
  int* lv = V.lv;
  int* apos = V.apos;
  int* rlive = V.rlive;
  int* rsp = V.rsp;
  int* roff = V.roff;
  int* pool = V.roff + R;
  int* lrec = V.lrec;
  float4* lv32 = V.lv32;
  // thread-0 state
  Lfsr rng;
  CassEnergy E;
  CassGCMCResult RS;
  int npool = G.npool, status = 0;
  long long sum_n = 0;
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
      if constexpr (MIXED) {
        const float u = draw_f(rng);
        mv_kind = u <= A.cutf[0] ? 0 : (u <= A.cutf[1] ? 1 : (u <= A.cutf[2] ? 2 : (u <= A.cutf[3] ? 3 : (u <= A.cutf[4] ? 4 : 5))));
      } else {
        const double u = rng.next();
        mv_kind = u <= A.cut_t ? 0 : (u <= A.cut_r ? 1 : (u <= A.cut_i ? 2 : (u <= A.cut_d ? 3 : (u <= A.cut_g ? 4 : 5))));
      }
      mv_skip = 0;
      mv_stop = 0;
      mv_ew = -1;
      int is = -1, im = 0;
      if (mv_kind == 0 || mv_kind == 1) {  // species choice of Translate / Rotate
        const double* step_sz = mv_kind == 0 ? G.max_disp : G.max_rot;
        int ntot = 0;
        for (int k = 0; k < A.nspecies; ++k)
          if (step_sz[k] > 0.0) ntot += nmol[k];
        if (ntot == 0) {
          mv_skip = 1;
        } else {
          int last = 0;
          if constexpr (MIXED) {
            const float v = draw_f(rng) * (float)ntot;
            int cum = 0;
            for (int k = 0; k < A.nspecies; ++k) {
              if (!(step_sz[k] > 0.0)) continue;
              cum += nmol[k];
              if (nmol[k] > 0) last = k;
              if (is < 0 && v <= (float)cum) is = k;
            }
          } else {
            const double v = rng.next();
            double x = 0.0;
            for (int k = 0; k < A.nspecies; ++k) {
              x = (step_sz[k] > 0.0 ? (double)nmol[k] / (double)ntot : 0.0) + (k > 0 ? x : 0.0);
              if (step_sz[k] > 0.0 && nmol[k] > 0) last = k;
              if (is < 0 && v <= x) is = k;
            }
          }
          if (is < 0) is = last;
          im = gc_pick<MIXED>(rng, nmol[is]);
          if (mv_kind == 0) ++RS.n_translate;
          else ++RS.n_rotate;
        }
      } else if (mv_kind == 2) {
        gc_skip_draw<MIXED>(rng);  // is_rand
        if (npool == 0) {
          mv_stop = 1;
          status = 2;
        } else {
          ++RS.n_insert;
          is = ise;
        }
      } else if (mv_kind == 3) {
        gc_skip_draw<MIXED>(rng);  // is_rand
        if (nmol[ise] == 0) {
          mv_skip = 1;
        } else {
          ++RS.n_delete;
          is = ise;
          im = gc_pick<MIXED>(rng, nmol[ise]);
        }
      } else if (mv_kind == 4) {
        if (nmol[ise] == 0) {
          mv_skip = 1;
        } else {
          gc_skip_draw<MIXED>(rng);  // the box choice
          gc_skip_draw<MIXED>(rng);  // the species choice
          im = gc_pick<MIXED>(rng, nmol[ise]);
          is = ise;
          ++RS.n_regrow;
          if (S.nfrag < 2) mv_skip = 1;  // single-fragment regrowth is not on this path
        }
      } else {
        mv_skip = 1;
      }
      // the molecule: a free record for an insertion, else the im-th live
      // molecule of species is in slot order
      if (!mv_skip && !mv_stop) {
        const int rec = mv_kind == 2 ? pool[npool - 1] : lrec[rs0[is] + im - 1];
        mv_rec = rec;
        mv_is = is;
        mv_slot = G.rec[rec].x;
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
    }
    __syncthreads();
    if (mv_stop) break;
    if (!mv_skip) {
      const int is = mv_is;
      if (mv_kind <= 1) {
        // ---- Translate / Rotate: the trial position first (no draw depends on
        // the old energy), then old and trial energies in one pass
        if (threadIdx.x == 0) {
          for (int i = 0; i < 3 * gs.na; ++i) old_r[i] = gs.r[i];
          for (int d = 0; d < 3; ++d) old_com[d] = gs.com[d];
          {
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
          gs.ntid = gs.na;
          for (int a = 0; a < gs.na; ++a) {
            gs.tids[a] = a;
            for (int d = 0; d < 3; ++d) {
              gs.trial[0][3 * a + d] = old_r[3 * a + d];
              gs.trial[1][3 * a + d] = gs.r[3 * a + d];
            }
          }
        }
        __syncthreads();
        // charged boxes: vdW in gs.e[0..1], Coulomb in gs.e[2..3], and the
        // reciprocal energy after the move (move_translate.f90:250-290)
        const bool qon = !MIXED && G.qon;
        const bool ew = qon && A.sp[is].has_charge;
        if constexpr (!MIXED) {
          if (qon) batch_energies<false, 4, true>(V, gs, 2, gs.rec, false, A.sp[is].type, true, A.sp[is].mass, A.sp[is].q);
          else batch_energies<false, 2>(V, gs, 2, gs.rec, false, A.sp[is].type, true, A.sp[is].mass);
        } else {
          batch_energies<true, 2>(V, gs, 2, gs.rec, false, A.sp[is].type, true, A.sp[is].mass);
        }
        double e_recip = 0.0;
        if (ew && !gs.ov[0] && !gs.ov[1]) e_recip = gc_recip(G, A.sp[is], gs.r, mv_slot, 2, s_red);
        if (threadIdx.x == 0) {
          mv_acc = 0;
          if (gs.ov[0]) {  // the molecule overlapped before the move
            mv_stop = 1;
            status = 1;
          } else if (!gs.ov[1]) {
            const double dv = gs.e[1] - gs.e[0];
            const double dq = qon ? gs.e[3] - gs.e[2] : 0.0;
            double dE = dv;
            if (qon) {
              dE = ew ? e_recip - E.reciprocal : 0.0;
              dE = dE + dv + dq;
            }
            if (gc_accept(b.beta * dE, rng)) {
              mv_acc = 1;
              E.total = E.total + dE;
              E.inter = E.inter + dE;
              E.inter_vdw = E.inter_vdw + dv;
              if (qon) E.inter_q = E.inter_q + dq;
              if (ew) {
                E.reciprocal = e_recip;
                mv_ew = 2;
              }
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
        __syncthreads();
        if (mv_stop) break;
      } else if (mv_kind == 2) {
        if constexpr (MIXED) {
          // ---- Insertion (FP32 growth)
          if (threadIdx.x == 0) mv_acc = 0;
          const bool ov = gc_build_f(A, V, gs, gf, false, rng);
          if (threadIdx.x == 0) {
            gs.flag = ov ? 1 : 0;
            if (!ov) {
              gc_fold_f(bf, gf, gs.na);
              get_com_f(A.SF, gf.r, (1u << gs.na) - 1u, gf.com);
            }
          }
          __syncthreads();
          if (!gs.flag) {
            gc_mol_energies_f(A, V, gs, gf, ttype, em, eov);
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
                e_lrc = gc_lrc(G, T.ntypes, nbn);
                dE_inter = dE_inter + e_lrc - E.lrc;
              }
              const double dE = dE_intra + dE_inter;
              const double ln_pbias = (double)(gf.ln_pbias + gf.ln_pseq) + (S.ln_kappa_ins + S.ln_kappa_dih_term);
              const double ln_pacc = b.beta * (dE - ea - G.mu) + ln_pbias + G.logn[nmol[ise] + 1] + G.log_lambda3 -
                                     G.log_vol;
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
                // the new molecule: coordinates, live lists
                const int rec = gs.rec;
                rlive[rec] = 1;
                for (int a = 0; a < gs.na; ++a) {
                  const int j = roff[rec] + a;
                  sx[j] = (double)gf.r[3 * a];
                  sy[j] = (double)gf.r[3 * a + 1];
                  sz[j] = (double)gf.r[3 * a + 2];
                }
                for (int d = 0; d < 3; ++d) scom[3 * rec + d] = (double)gf.com[d];
                lrec_insert(lrec, rs0[ise], nmol[ise] - 1, rec);
                for (int a = 0; a < gs.na; ++a) {
                  const int j = roff[rec] + a, i = s_nlv++;
                  apos[j] = i;
                  lv[i] = j;
                  lv32[i] = make_float4(gf.r[3 * a], gf.r[3 * a + 1], gf.r[3 * a + 2], __int_as_float(S.type[a]));
                }
              }
            }
          }
        } else {
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
            // charged boxes (move_insert.f90:274-291): the reciprocal energy with
            // the molecule's structure factors added, and its self energy
            const bool qon = G.qon != 0;
            const bool ew = qon && A.sp[ise].has_charge;
            double e_recip = 0.0;
            if (ew && !eov[0] && !eov[1]) e_recip = gc_recip(G, A.sp[ise], gs.r, mv_slot, 0, s_red);
            if (threadIdx.x == 0 && !eov[0] && !eov[1]) {
              const double ev = em[0], eq = em[1];
              const double eb = em[2], ea = em[3], ed = em[4], ei = em[5], eiv = em[6], eiq = em[7];
              double dE_inter = ev + eq, dE_intra = eiv + eiq + eb + ea + ed + ei;
              double e_self = 0.0;
              if (qon) {
                if (ew) dE_inter = dE_inter + (e_recip - E.reciprocal);
                e_self = gc_self(A.sp[ise], b);
                dE_inter = dE_inter + e_self;
              }
              double nbn[kMaxTypes];
              for (int t = 0; t < kMaxTypes; ++t) nbn[t] = nb[t];
              for (int a = 0; a < gs.na; ++a)
                if (S.type[a] >= 0) nbn[S.type[a]] += 1.0;
              double e_lrc = E.lrc;
              const bool tail = b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL;
              if (tail) {
                e_lrc = gc_lrc(G, T.ntypes, nbn);
                dE_inter = dE_inter + e_lrc - E.lrc;
              }
              const double dE = dE_intra + dE_inter;
              double ln_pacc = b.beta * (dE - ea);
              ln_pacc = ln_pacc - G.mu * b.beta;
              ln_pacc = ln_pacc + gs.ln_pbias;
              ln_pacc = ln_pacc + log((double)(nmol[ise] + 1)) + G.log_lambda3;
              ln_pacc = ln_pacc - G.log_vol;
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
                if (ew) {
                  E.reciprocal = e_recip;
                  mv_ew = 0;
                }
                E.self += e_self;
                for (int t = 0; t < kMaxTypes; ++t) nb[t] = nbn[t];
                ++RS.n_insert_accepted;
                ++nmol[ise];
                --npool;
              }
            }
          }
          if (threadIdx.x == 0 && mv_acc) {
            rlive[gs.rec] = 1;
            lrec_insert(lrec, rs0[ise], nmol[ise] - 1, gs.rec);
            list_add<MIXED>(V, &s_nlv, gs.rec, gs.na, S.type);  // coordinates follow in the commit below
          }
        }
      } else if (mv_kind == 3) {
        if constexpr (MIXED) {
          // ---- Deletion (FP32 old-weight pass from the stored coordinates)
          if (threadIdx.x == 0) {
            mv_acc = 0;
            for (int i = 0; i < 3 * gs.na; ++i) gf.r[i] = (float)gs.r[i];
            for (int d = 0; d < 3; ++d) gf.com[d] = (float)gs.com[d];
          }
          __syncthreads();
          const bool ov = gc_build_f(A, V, gs, gf, true, rng);
          if (threadIdx.x == 0) {
            gs.flag = ov ? 1 : 0;
            if (ov) {
              mv_stop = 1;
              status = 1;
            }
            get_com_f(A.SF, gf.r, (1u << gs.na) - 1u, gf.com);
          }
          __syncthreads();
          if (mv_stop) break;
          gc_mol_energies_f(A, V, gs, gf, ttype, em, eov);
          if (threadIdx.x == 0) {
            const double ev = em[0], eq = em[1];
            const double eb = em[2], ea = em[3], ed = em[4], ei = em[5], eiv = em[6], eiq = em[7];
            double dE_inter = -ev - eq;
            double dE_intra = -eb - ea - ed - ei - eiv - eiq;
            double nbn[kMaxTypes];
            for (int t = 0; t < kMaxTypes; ++t) nbn[t] = nb[t];
            for (int a = 0; a < gs.na; ++a)
              if (S.type[a] >= 0) nbn[S.type[a]] -= 1.0;
            double e_lrc = E.lrc;
            const bool tail = b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL;
            if (tail) {
              e_lrc = gc_lrc(G, T.ntypes, nbn);
              dE_inter = dE_inter + (e_lrc - E.lrc);
            }
            const double dE = dE_intra + dE_inter;
            const double ln_pbias = (double)(gf.ln_pbias + gf.ln_pseq) + (S.ln_kappa_ins + S.ln_kappa_dih_term);
            const double ln_pacc = b.beta * (dE + ea + G.mu) - ln_pbias - G.logn[nmol[ise]] - G.log_lambda3 +
                                   G.log_vol;
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
              lrec_remove(lrec, rs0[ise], nmol[ise] + 1, gs.rec);
              list_remove<MIXED>(V, &s_nlv, gs.rec, gs.na);
            }
            // a rejected deletion leaves the stored coordinates as they were
          }
        } else {
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
          // charged boxes (move_delete.f90:261-277): the reciprocal energy with
          // the molecule's structure factors taken out, and its self energy
          const bool qon = G.qon != 0;
          const bool ew = qon && A.sp[ise].has_charge;
          double e_recip = 0.0;
          if (ew) e_recip = gc_recip(G, A.sp[ise], nullptr, mv_slot, 1, s_red);
          if (threadIdx.x == 0) {
            mv_acc = 0;
            const double ev = em[0], eq = em[1];
            const double eb = em[2], ea = em[3], ed = em[4], ei = em[5], eiv = em[6], eiq = em[7];
            double dE_inter = -ev - em[8];
            double dE_intra = -eb - ea - ed - ei;
            dE_intra = dE_intra - eiv - eiq;
            dE_inter = dE_inter - em[9];
            double e_self = 0.0;
            if (qon) {
              if (ew) dE_inter = dE_inter + (e_recip - E.reciprocal);
              e_self = gc_self(A.sp[ise], b);
              dE_inter = dE_inter - e_self;
            }
            double nbn[kMaxTypes];
            for (int t = 0; t < kMaxTypes; ++t) nbn[t] = nb[t];
            for (int a = 0; a < gs.na; ++a)
              if (S.type[a] >= 0) nbn[S.type[a]] -= 1.0;
            double e_lrc = E.lrc;
            const bool tail = b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL;
            if (tail) {
              e_lrc = gc_lrc(G, T.ntypes, nbn);
              dE_inter = dE_inter + (e_lrc - E.lrc);
            }
            const double dE = dE_intra + dE_inter;
            double ln_pacc = b.beta * (dE + ea);
            ln_pacc = ln_pacc + b.beta * G.mu;
            ln_pacc = ln_pacc - gs.ln_pbias;
            ln_pacc = ln_pacc - log((double)nmol[ise]) - G.log_lambda3;
            ln_pacc = ln_pacc + G.log_vol;
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
              if (ew) {
                E.reciprocal = e_recip;
                mv_ew = 1;
              }
              E.self -= e_self;
              for (int t = 0; t < kMaxTypes; ++t) nb[t] = nbn[t];
              ++RS.n_delete_accepted;
              --nmol[ise];
              rlive[gs.rec] = 0;
              pool[npool++] = gs.rec;
              lrec_remove(lrec, rs0[ise], nmol[ise] + 1, gs.rec);
              list_remove<MIXED>(V, &s_nlv, gs.rec, gs.na);
            }
            // a rejected deletion keeps the coordinates its Rosenbluth pass left
          }
        }
      } else {
        if constexpr (MIXED) {
          // ---- Cut_N_Grow (FP32 growth): new configuration, then the old one
          if (threadIdx.x == 0) {
            mv_acc = 0;
            for (int i = 0; i < 3 * gs.na; ++i) gf.r[i] = (float)gs.r[i];
            for (int d = 0; d < 3; ++d) gf.com[d] = (float)gs.com[d];
            const int fb = min((int)(draw_f(rng) * (float)A.nfbond), A.nfbond - 1);
            if (draw_f(rng) < A.prob_del1f[fb]) {
              gs.f_dead = A.fb_a[fb];
              gs.f_live = A.fb_b[fb];
            } else {
              gs.f_dead = A.fb_b[fb];
              gs.f_live = A.fb_a[fb];
            }
            gs.order[0] = gs.f_dead;
            gs.norder = 1;
            gf.ln_pseq = 0.0f;
            gc_fragment_order_f(S, gs, gf, (1u << gs.f_live) | (1u << gs.f_dead), rng);
            gc_cut_f(S, gs, gf);
            rgf_e_prev = dihedral_f(A.SF, gf.r, gs.exist);
            gf.e_prev = rgf_e_prev;
          }
          __syncthreads();
          bool ov = gc_place_fragments_f(A, V, gs, gf, 0, false, rng);
          if (threadIdx.x == 0 && !ov) {
            rgf_ln_pfor = gf.ln_pbias;
            get_com_f(A.SF, gf.r, (1u << gs.na) - 1u, gf.com);
            gc_fold_f(bf, gf, gs.na);
          }
          __syncthreads();
          if (!ov) {
            gc_mol_energies_f(A, V, gs, gf, ttype, em, eov);
            if (threadIdx.x == 0) {
              if (eov[0]) {
                ov = true;
              } else {
                for (int k = 0; k < 8; ++k) rg_en[k] = em[k];
                for (int i = 0; i < 3 * gs.na; ++i) {
                  rgf_new[i] = gf.r[i];
                  gf.r[i] = (float)gs.r[i];
                }
                for (int d = 0; d < 3; ++d) {
                  rgf_new_com[d] = gf.com[d];
                  gf.com[d] = (float)gs.com[d];
                }
                gc_cut_f(S, gs, gf);
                gf.e_prev = rgf_e_prev;
              }
              gs.flag = ov ? 1 : 0;
            }
            __syncthreads();
            if (!gs.flag) {
              const bool ov_old = gc_place_fragments_f(A, V, gs, gf, 0, true, rng);
              if (threadIdx.x == 0) {
                if (ov_old) {
                  mv_stop = 1;
                  status = 1;
                } else {
                  get_com_f(A.SF, gf.r, (1u << gs.na) - 1u, gf.com);
                }
              }
              __syncthreads();
              if (mv_stop) break;
              gc_mol_energies_f(A, V, gs, gf, ttype, em, eov);
              if (threadIdx.x == 0) {
                const double* en = rg_en;  // ev, eq, eb, ea, ed, ei, eiv, eiq of the new configuration
                double dE_intra = en[2] + en[3] + en[4] + en[5] + en[7] + en[6];
                double dE_inter = en[1] + en[0];
                dE_intra = dE_intra - em[2] - em[3] - em[4] - em[5] - em[7] - em[6];
                dE_inter = dE_inter - em[1] - em[0];
                const double dE = dE_intra + dE_inter;
                const double dE_frag = en[3] - em[3];
                const double ln_pacc = b.beta * (dE - dE_frag) + (double)(rgf_ln_pfor - gf.ln_pbias);
                if (gc_accept(ln_pacc, rng)) {
                  mv_acc = 1;
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
                  const int rec = gs.rec;
                  for (int a = 0; a < gs.na; ++a) {
                    const int j = roff[rec] + a;
                    sx[j] = (double)rgf_new[3 * a];
                    sy[j] = (double)rgf_new[3 * a + 1];
                    sz[j] = (double)rgf_new[3 * a + 2];
                    const int i = apos[j];
                    lv32[i] = make_float4(rgf_new[3 * a], rgf_new[3 * a + 1], rgf_new[3 * a + 2], lv32[i].w);
                  }
                  for (int d = 0; d < 3; ++d) scom[3 * rec + d] = (double)rgf_new_com[d];
                }
              }
            }
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
              // charged boxes: the reciprocal energy of the new configuration
              // (move_regrow.f90:338-354, int_intra)
              const bool ew = G.qon && A.sp[ise].has_charge;
              double e_recip = 0.0;
              if (ew) e_recip = gc_recip(G, A.sp[ise], rg_new, mv_slot, 2, s_red);
              if (threadIdx.x == 0) {
                const double* en = rg_en;  // ev, eq, eb, ea, ed, ei, eiv, eiq of the new configuration
                double dE_intra = en[2] + en[3] + en[4] + en[5] + en[7] + en[6];
                double dE_inter = en[1] + en[0];
                if (ew) dE_inter = dE_inter + (e_recip - E.reciprocal);
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
                  if (ew) {
                    E.reciprocal = e_recip;
                    mv_ew = 2;
                  }
                  ++RS.n_regrow_accepted;
                }
              }
            }
          }
        }
      }
      __syncthreads();
      if (!MIXED && mv_ew >= 0) gc_recip_commit(G, mv_slot, mv_ew);  // accepted moves of charged molecules
      // commit the molecule's coordinates (rejected deletions and regrowths keep
      // the coordinates of their Rosenbluth pass, as the reference does)
      if (threadIdx.x == 0) {
        if (MIXED ? (mv_kind <= 1 && mv_acc) : (mv_kind != 2 || mv_acc)) {
          for (int a = 0; a < gs.na; ++a) {
            const int j = roff[gs.rec] + a;
            sx[j] = gs.r[3 * a];
            sy[j] = gs.r[3 * a + 1];
            sz[j] = gs.r[3 * a + 2];
            const int i = apos[j];
            if (MIXED && i >= 0) lv32[i] = make_float4((float)gs.r[3 * a], (float)gs.r[3 * a + 1], (float)gs.r[3 * a + 2], lv32[i].w);
          }
          for (int d = 0; d < 3; ++d) scom[3 * gs.rec + d] = gs.com[d];
          if (!MIXED && V.comcut) {  // max_dcom of the molecule as placed (insertion, regrowth; rigid moves keep it)
            double dmax = 0.0;
            for (int a = 0; a < gs.na; ++a) {
              const double dx = gs.r[3 * a] - gs.com[0], dy = gs.r[3 * a + 1] - gs.com[1],
                           dz = gs.r[3 * a + 2] - gs.com[2];
              dmax = fmax(dmax, dx * dx + dy * dy + dz * dz);
            }
            rdcom[gs.rec] = sqrt(dmax);
          }
        }
      }
    }
    if (threadIdx.x == 0) sum_n += nmol[ise];
    __syncthreads();
  }
  __syncthreads();
  if (csize > 1) cooperative_groups::this_cluster().sync();  // no CTA leaves while its shared memory may be read
  if (crank != 0) return;
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
    RS.sum_n_molecules = (double)sum_n;
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

// the dynamic shared memory layout of k_gcmc: sx, sy, sz, scom, lv, apos,
// [lvt], rlive, rsp, roff, pool, lrec, [lv32]
// Build_Molecule (fragment_growth.f90:72-707) of one molecule, record `rec` of
// the box view, as a host's own insertion or deletion move calls it: the
// whole CTA grows it (gc_build in FP64, gc_build_f in the mixed kernel) from
// the caller's lfsr258 state.  Outputs: iout = cbmc overlap, number of
// fragments placed, the growth order; out = ln_pseq, ln_pbias, coordinates.
template <bool MIXED>
__global__ void __launch_bounds__(kGcThreads, 1)
    k_build_mol(GcArgs A, const GcBox* box, PairTable T, int rec, int del, unsigned long long* state, double* out,
                int* iout) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BoxDev b;
  __shared__ GrowState gs;
  __shared__ GrowF gf;
  __shared__ BoxF bf;
  __shared__ PairTable sT;
  __shared__ float2 s_ljp[kMaxTypes * kMaxTypes];
  __shared__ float s_epsf[kMaxTypes * kMaxTypes], s_sig2f[kMaxTypes * kMaxTypes];
  __shared__ int rs0[kGcMaxSpecies];
  __shared__ int ttype[kMaxAtoms];
  __shared__ int s_nlv;
  if (threadIdx.x == 0) gs.cbuf = 0;
  GcView V;
  gc_setup<MIXED>(A, *box, T, 1, 0, smem, b, bf, sT, s_ljp, s_epsf, s_sig2f, rs0, s_nlv, ttype, V);
  Lfsr rng;
  if (threadIdx.x == 0) {
    rng.s1 = state[0];
    rng.s2 = state[1];
    rng.s3 = state[2];
    rng.s4 = state[3];
    rng.s5 = state[4];
    gs.rec = rec;
    gs.is = A.is_ex;
    gs.na = A.sp[A.is_ex].natoms;
    for (int a = 0; a < gs.na; ++a) {
      gs.r[3 * a] = V.sx[V.roff[rec] + a];
      gs.r[3 * a + 1] = V.sy[V.roff[rec] + a];
      gs.r[3 * a + 2] = V.sz[V.roff[rec] + a];
    }
    for (int d = 0; d < 3; ++d) gs.com[d] = V.com[3 * rec + d];
    if (MIXED) {
      for (int i = 0; i < 3 * gs.na; ++i) gf.r[i] = (float)gs.r[i];
      for (int d = 0; d < 3; ++d) gf.com[d] = (float)gs.com[d];
    }
  }
  __syncthreads();
  bool ov;
  if constexpr (MIXED) ov = gc_build_f(A, V, gs, gf, del != 0, rng);
  else ov = gc_build<false>(A, V, gs, del != 0, rng);
  if (threadIdx.x == 0) {
    state[0] = rng.s1;
    state[1] = rng.s2;
    state[2] = rng.s3;
    state[3] = rng.s4;
    state[4] = rng.s5;
    iout[0] = ov ? 1 : 0;
    iout[1] = gs.norder;
    for (int k = 0; k < gs.norder && k < kMaxFrags; ++k) iout[2 + k] = gs.order[k];
    out[0] = MIXED ? (double)gf.ln_pseq : gs.ln_pseq;
    out[1] = MIXED ? (double)gf.ln_pbias : gs.ln_pbias;
    for (int a = 0; a < gs.na; ++a)
      for (int d = 0; d < 3; ++d) {
        const double v = d == 0 ? V.sx[V.roff[rec] + a] : (d == 1 ? V.sy[V.roff[rec] + a] : V.sz[V.roff[rec] + a]);
        out[2 + 3 * a + d] = del ? v : (MIXED ? (double)gf.r[3 * a + d] : gs.r[3 * a + d]);
      }
  }
}

size_t gc_smem_bytes(int natoms, int nrec, bool mixed, bool comcut, bool charged) {
  size_t s = (size_t)natoms * (3 * sizeof(double) + (mixed ? 2 : 3) * sizeof(int)) +
             (size_t)nrec * (3 * sizeof(double) + 5 * sizeof(int));
  s = (s + 15) & ~(size_t)15;
  if (mixed) s += (size_t)natoms * sizeof(float4);
  if (comcut) s += (size_t)nrec * sizeof(double) + (size_t)natoms * sizeof(int);
  if (charged && !mixed) s = ((s + 15) & ~(size_t)15) + (size_t)natoms * sizeof(double);
  return s;
}
}  // namespace cassgpu

using namespace cassgpu;

// A box as a grand-canonical kernel holds it: records of its live molecules and
// of the free slots `free_slots`, in slot order, with their atoms (free slots at
// the origin), the free records' indices, and the box constants of g (mu and
// the de Broglie term are the caller's).
struct HostBox {
  std::vector<int> slots;
  std::vector<int4> rec;
  std::vector<double4_32a> xyzq;
  std::vector<int> atype, pool;
};

static void gc_host_box(cass_ctx* c, int ib, const std::vector<int>& free_slots, HostBox& h, GcBox& g) {
  BoxH& B = c->box[ib];
  const std::vector<int>& mem = members_ext(c, ib);
  h.slots.assign(mem.begin(), mem.end());
  h.slots.insert(h.slots.end(), free_slots.begin(), free_slots.end());
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
  for (int slot : free_slots) h.pool.push_back((int)(std::lower_bound(h.slots.begin(), h.slots.end(), slot) - h.slots.begin()));
  memset(&g, 0, sizeof(g));
  g.b = B.dev;
  g.natoms = off;
  g.nrec = (int)h.slots.size();
  g.npool = (int)h.pool.size();
  g.ibox1 = ib + 1;
  g.rcut3 = B.rcut3;
  g.rcut9 = B.rcut9;
  g.comcut = B.comcut ? 1 : 0;
  g.rmax = B.rcut_max;
  // charged boxes: the Ewald state of the box and the per-molecule structure
  // factors (scratch rows new_cos / new_sin are the caller's)
  g.qon = B.desc.charge_style == CASS_CHARGE_COUL ? 1 : 0;
  if (g.qon && B.nvecs > 0) {
    g.nvecs = B.nvecs;
    g.kvec = B.d_kvec.as<double4_32a>();
    g.cos_sum = B.d_cos_sum.as<double>();
    g.sin_sum = B.d_sin_sum.as<double>();
    g.cos_mol = c->d_cos_mol.as<double>();
    g.sin_mol = c->d_sin_mol.as<double>();
    g.stride = c->cos_mol_stride;
  }
  const int nt = c->pt.ntypes;
  for (int ia = 0; ia < nt; ++ia)
    for (int ja = 0; ja < nt; ++ja) {
      const double eps = c->pt.eps[ia * nt + ja], s2 = c->pt.sig2[ia * nt + ja];
      const double s6 = s2 * s2 * s2, s12 = s6 * s6;
      g.lrc_c[ia * nt + ja] = 4.0 * eps * (s12 / (9.0 * B.rcut9) - (s6 / (3.0 * B.rcut3)));
    }
  g.lrc_pref = 2.0 * kPI / B.dev.volume;
  g.log_vol = std::log(B.dev.volume);
  for (int t = 0; t < kMaxTypes; ++t) g.nb0[t] = nb0[t];
}

// The growth tables and species tables of a grand-canonical kernel for the
// exchanged species is (0-based); mixed is cleared when the species does not fit
// the FP32 tables.  Move probabilities, steps and seed are the caller's.
static void gc_fill_args(cass_ctx* c, int is, int kappa_ins, int kappa_dih, bool& mixed, GcArgs& A) {
  const SpeciesH& s = c->sp[is];
  memset(&A, 0, sizeof(A));
  fill_growth_species(s, is, kappa_ins, kappa_dih, A.S);
  A.is_ex = is;
  A.nspecies = c->nspecies;
  for (int k = 0; k < c->nspecies; ++k) {
    const SpeciesH& t = c->sp[k];
    A.sp[k].natoms = t.natoms;
    A.sp[k].has_charge = t.has_charge ? 1 : 0;
    A.sp[k].l_coul_cbmc = t.l_coul_cbmc ? 1 : 0;
    bool lin = true;
    for (size_t q = 0; q < t.angle_kind.size(); ++q)
      if (t.angle_kind[q] != CASS_BONDED_FIXED || t.angle_param[2 * q] != 180.0) lin = false;
    A.sp[k].linear = lin ? 1 : 0;
    for (int a = 0; a < kMaxAtoms; ++a) A.sp[k].type[a] = -1;
    for (int a = 0; a < t.natoms && a < kMaxAtoms; ++a) {
      A.sp[k].mass[a] = t.mass[a];
      A.sp[k].q[a] = t.q[a];
      A.sp[k].type[a] = t.type[a];
    }
  }
  A.lib = s.d_library.as<double>();
  A.P = c->pools;
  // the mixed kernel grows molecules in FP32 from FP32 copies of the species and library
  mixed = mixed && species_f(s, A.SF) && s.d_library_f.p != nullptr;
  A.libf = s.d_library_f.as<float>();
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
      A.prob_del1f[A.nfbond] = (float)A.prob_del1[A.nfbond];
      ++A.nfbond;
    }
}

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
  bool any_q = false;
  int max_nv = 0;
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    if (ib < 0 || ib >= c->nboxes) return set_error(CASS_EINVAL, "box index out of range");
    for (int j = 0; j < k; ++j)
      if (iboxes[j] == iboxes[k]) return set_error(CASS_EINVAL, "box listed twice");
    const BoxH& B = c->box[ib];
    if (!B.energy_valid) return set_error(CASS_ESTATE, "system energy of box not computed");
    if (B.desc.charge_style != CASS_CHARGE_NONE && B.desc.charge_sum_style != CASS_QQ_EWALD)
      return set_error(CASS_EUNSUPPORTED, "gcmc: charges need the Ewald sum");
    if (B.desc.vdw_style != CASS_VDW_LJ) return set_error(CASS_EUNSUPPORTED, "gcmc needs LJ boxes");
    if (B.desc.charge_style != CASS_CHARGE_NONE) {
      if (B.nvecs > 0 && !c->d_cos_mol.p) return set_error(CASS_ESTATE, "structure factors not computed");
      any_q = true;
      max_nv = std::max(max_nv, B.nvecs);
    }
    mixed = mixed && (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT || B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL);
  }
  // charged boxes run the FP64 kernel, one CTA per box
  if (any_q) mixed = false;
  int rc;
  CASS_CUDA(cudaSetDevice(c->device));
  if ((rc = ensure_pools(c))) return rc;
  if ((rc = ensure_cbmc(c))) return rc;
  GcArgs A;
  gc_fill_args(c, is, p->kappa_ins, p->kappa_dih, mixed, A);
  A.nsteps = p->nsteps;
  A.cut_t = p->cut_translate;
  A.cut_r = p->cut_rotate;
  A.cut_i = p->cut_insert;
  A.cut_d = p->cut_delete;
  A.cut_g = p->cut_regrow;
  A.seed = seed;
  A.cutf[0] = (float)p->cut_translate;
  A.cutf[1] = (float)p->cut_rotate;
  A.cutf[2] = (float)p->cut_insert;
  A.cutf[3] = (float)p->cut_delete;
  A.cutf[4] = (float)p->cut_regrow;
  double mw = 0.0;
  for (double m : s.mass) mw += m;
  // free slots of the exchanged species, in ascending order, each to the box
  // holding the fewest atoms so far (live molecules of every species plus the
  // slots dealt; ties to the first listed box): the boxes' shares even out
  std::vector<std::vector<int>> pools(nboxes);
  {
    std::vector<long long> load(nboxes, 0);
    for (int k = 0; k < nboxes; ++k)
      for (int slot : members_ext(c, iboxes[k] - 1)) load[k] += c->sp[c->slot_sp[slot]].natoms;
    for (int im = 0; im < c->max_mol[is]; ++im) {
      const int slot = c->mol_base[is] + im;
      if (c->mol_box[slot] >= 0) continue;
      int kmin = 0;
      for (int k = 1; k < nboxes; ++k)
        if (load[k] < load[kmin]) kmin = k;
      pools[kmin].push_back(slot);
      load[kmin] += s.natoms;
    }
  }
  std::vector<HostBox> hb(nboxes);
  std::vector<GcBox> gb(nboxes);
  size_t smem = 0, tot_atoms = 0, tot_rec = 0;
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    BoxH& B = c->box[ib];
    HostBox& h = hb[k];
    GcBox& g = gb[k];
    gc_host_box(c, ib, pools[k], h, g);
    g.mu = mu[k] / 0.01;  // kJ/mol to internal units (atomic_to_kJmol)
    g.log_lambda3 = 3.0 * std::log(39.9031268605 * std::sqrt(B.dev.beta / (kTWOPI * mw)));  // de Broglie
    smem = std::max(smem, gc_smem_bytes(g.natoms, g.nrec, mixed, g.comcut != 0, g.qon != 0));
    tot_atoms += (size_t)g.natoms;
    tot_rec += h.slots.size();
  }
  if (smem > kGcSmemLimit)
    return set_error(CASS_ECAPACITY, "gcmc holds a box's molecules and free slots in shared memory: too many atoms");
  const size_t nsp = (size_t)c->nspecies;
  size_t max_rec = 0;
  for (const HostBox& h : hb) max_rec = std::max(max_rec, h.slots.size());
  const size_t nlog = max_rec + 2;
  const size_t bytes = nboxes * sizeof(GcBox) + nlog * sizeof(double) + tot_atoms * (sizeof(double4_32a) + sizeof(int)) +
                       tot_rec * (sizeof(int4) + sizeof(int)) + 2 * nboxes * nsp * sizeof(double) +
                       nboxes * (sizeof(CassEnergy) + sizeof(CassGCMCResult) + sizeof(int)) +
                       2 * (size_t)nboxes * max_nv * sizeof(double) + 1024;
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
  double* d_logn = reinterpret_cast<double*>(carve(nlog * sizeof(double), 16));
  {
    std::vector<double> logn(nlog);
    logn[0] = 0.0;  // never read: ln N is taken for N >= 1
    for (size_t k = 1; k < nlog; ++k) logn[k] = std::log((double)k);
    CASS_CUDA(h2d(c, d_logn, logn.data(), nlog * sizeof(double)));
  }
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
    g.logn = d_logn;
    g.max_disp = d_md + k * nsp;
    g.max_rot = d_mr + k * nsp;
    g.energy = d_E + k;
    g.res = d_res + k;
    g.status = d_status + k;
    if (g.nvecs > 0) {
      g.new_cos = reinterpret_cast<double*>(carve(2 * (size_t)g.nvecs * sizeof(double), 16));
      g.new_sin = g.new_cos + g.nvecs;
    }
    hE[k] = c->box[iboxes[k] - 1].energy;
  }
  CASS_CUDA(h2d(c, d_box, gb.data(), nboxes * sizeof(GcBox)));
  CASS_CUDA(h2d(c, d_E, hE.data(), nboxes * sizeof(CassEnergy)));
  CASS_CUDA(h2d(c, d_md, max_disp, nboxes * nsp * sizeof(double)));
  CASS_CUDA(h2d(c, d_mr, max_rot, nboxes * nsp * sizeof(double)));
  auto kern = mixed ? k_gcmc<true> : k_gcmc<false>;
  CASS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // cluster size: the largest of 8, 4, 2 for which every box's cluster can be
  // resident at once; else one CTA per box (always for charged boxes, whose
  // reciprocal-space pass runs on one CTA)
  int csize = 1;
  for (int cs = any_q ? 1 : 8; cs >= 2; cs >>= 1) {
    cudaLaunchConfig_t q = {};
    cudaLaunchAttribute qa[1];
    qa[0].id = cudaLaunchAttributeClusterDimension;
    qa[0].val.clusterDim.x = cs;
    qa[0].val.clusterDim.y = 1;
    qa[0].val.clusterDim.z = 1;
    q.gridDim = dim3(nboxes * cs);
    q.blockDim = dim3(kGcThreads);
    q.dynamicSmemBytes = smem;
    q.attrs = qa;
    q.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &q) == cudaSuccess && nclusters >= nboxes) {
      csize = cs;
      break;
    }
    (void)cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(nboxes * csize);
  cfg.blockDim = dim3(kGcThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = c->stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  c->stats.gcmc_cluster = csize;
  CASS_CUDA(cudaEventRecord(c->ev[0], c->stream));
  CASS_CUDA(cudaLaunchKernelEx(&cfg, kern, A, d_box, c->pt, csize));
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

// Build_Molecule for one molecule (the per-call growth a host's own CBMC moves
// use): the box view of cass_gcmc with the molecule's slot as a record (live
// for del_flag, else a free record), one CTA, the caller's lfsr258 state
extern "C" int cass_build_molecule(cass_ctx* c, int32_t im, int32_t is1, int32_t ibox, int32_t del_flag,
                                   int32_t kappa_ins, int32_t kappa_dih, uint64_t* rng_state, int32_t* frag_order,
                                   double* ln_pseq, double* ln_pbias, double* xyz, int32_t* cbmc_overlap) {
  if (!c || is1 < 1 || is1 > c->nspecies || ibox < 1 || ibox > c->nboxes || !rng_state || !ln_pseq || !ln_pbias ||
      !cbmc_overlap || kappa_ins < 1 || kappa_ins > kMaxKappa)
    return set_error(CASS_EINVAL, "bad build_molecule arguments");
  if (c->nspecies > kGcMaxSpecies) return set_error(CASS_ECAPACITY, "build_molecule supports at most 8 species");
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  const int is = is1 - 1, ib = ibox - 1;
  const SpeciesH& s = c->sp[is];
  if (!s.defined || s.nfrag < 1) return set_error(CASS_ESTATE, "species not defined or without fragments");
  if (im < 1 || im > c->max_mol[is]) return set_error(CASS_EINVAL, "molecule index out of range");
  if (s.nfrag > 1 && (kappa_dih < 1 || kappa_dih > kMaxKappa)) return set_error(CASS_EINVAL, "kappa_dih must be in 1..32");
  if (s.nfrag > kMaxFrags) return set_error(CASS_ECAPACITY, "species has more than 8 fragments");
  for (int k = 0; k < c->nspecies; ++k)
    if (c->sp[k].defined && c->sp[k].natoms > kMaxAtoms) return set_error(CASS_ECAPACITY, "molecules of at most 16 atoms");
  for (int f = 0; f < s.nfrag; ++f)
    if (s.frag_nconfig[f] < 1) return set_error(CASS_EINVAL, "fragment library is empty");
  const BoxH& B = c->box[ib];
  if (!B.defined) return set_error(CASS_ESTATE, "box not defined");
  if (B.desc.charge_style != CASS_CHARGE_NONE && B.desc.charge_sum_style != CASS_QQ_EWALD)
    return set_error(CASS_EUNSUPPORTED, "build_molecule: charges need the Ewald sum");
  if (B.desc.vdw_style != CASS_VDW_LJ) return set_error(CASS_EUNSUPPORTED, "build_molecule needs LJ boxes");
  const int slot = c->mol_base[is] + im - 1;
  if (del_flag && c->mol_box[slot] != ib) return set_error(CASS_ESTATE, "del_flag: the molecule is not live in the box");
  if (!del_flag && c->mol_box[slot] >= 0) return set_error(CASS_ESTATE, "the molecule to grow is live");
  bool mixed = c->precision == CASS_PREC_MIXED && B.desc.charge_style == CASS_CHARGE_NONE &&
               (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT || B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL);
  int rc;
  CASS_CUDA(cudaSetDevice(c->device));
  if ((rc = ensure_pools(c))) return rc;
  if ((rc = ensure_cbmc(c))) return rc;
  GcArgs A;
  gc_fill_args(c, is, kappa_ins, kappa_dih, mixed, A);
  HostBox h;
  GcBox g;
  gc_host_box(c, ib, del_flag ? std::vector<int>() : std::vector<int>{slot}, h, g);
  const int rec = (int)(std::lower_bound(h.slots.begin(), h.slots.end(), slot) - h.slots.begin());
  const size_t smem = gc_smem_bytes(g.natoms, g.nrec, mixed, g.comcut != 0, g.qon != 0);
  if (smem > kGcSmemLimit)
    return set_error(CASS_ECAPACITY, "build_molecule holds the box in shared memory: too many atoms");
  const size_t nout = 2 + 3 * (size_t)s.natoms, niout = 2 + kMaxFrags;
  const size_t bytes = sizeof(GcBox) + h.xyzq.size() * sizeof(double4_32a) + h.atype.size() * sizeof(int) +
                       h.rec.size() * sizeof(int4) + 8 * sizeof(double) + nout * sizeof(double) +
                       niout * sizeof(int) + 256;
  if ((rc = c->d_gc.reserve(bytes))) return rc;
  char* base = static_cast<char*>(c->d_gc.p);
  auto carve = [&](size_t n, size_t align) {
    size_t o = ((size_t)(base - static_cast<char*>(c->d_gc.p)) + align - 1) & ~(align - 1);
    char* q = static_cast<char*>(c->d_gc.p) + o;
    base = q + n;
    return q;
  };
  GcBox* d_box = reinterpret_cast<GcBox*>(carve(sizeof(GcBox), 64));
  double4_32a* d_xyz = reinterpret_cast<double4_32a*>(carve(std::max<size_t>(1, h.xyzq.size()) * sizeof(double4_32a), 32));
  int* d_at = reinterpret_cast<int*>(carve(std::max<size_t>(1, h.atype.size()) * sizeof(int), 16));
  int4* d_rec = reinterpret_cast<int4*>(carve(std::max<size_t>(1, h.rec.size()) * sizeof(int4), 16));
  unsigned long long* d_state = reinterpret_cast<unsigned long long*>(carve(8 * sizeof(double), 16));
  double* d_out = reinterpret_cast<double*>(carve(nout * sizeof(double), 16));
  int* d_iout = reinterpret_cast<int*>(carve(niout * sizeof(int), 16));
  CASS_CUDA(h2d(c, d_xyz, h.xyzq.data(), h.xyzq.size() * sizeof(double4_32a)));
  CASS_CUDA(h2d(c, d_at, h.atype.data(), h.atype.size() * sizeof(int)));
  CASS_CUDA(h2d(c, d_rec, h.rec.data(), h.rec.size() * sizeof(int4)));
  CASS_CUDA(h2d(c, d_state, rng_state, 5 * sizeof(uint64_t)));
  g.xyzq = d_xyz;
  g.atype = d_at;
  g.rec = d_rec;
  g.pool = nullptr;
  g.npool = 0;
  CASS_CUDA(h2d(c, d_box, &g, sizeof(GcBox)));
  auto kern = mixed ? k_build_mol<true> : k_build_mol<false>;
  CASS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<1, kGcThreads, smem, c->stream>>>(A, d_box, c->pt, rec, del_flag ? 1 : 0, d_state, d_out, d_iout);
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  std::vector<double> hout(nout);
  int hiout[2 + kMaxFrags];
  CASS_CUDA(d2h(c, rng_state, d_state, 5 * sizeof(uint64_t)));
  CASS_CUDA(d2h(c, hout.data(), d_out, nout * sizeof(double)));
  CASS_CUDA(d2h(c, hiout, d_iout, niout * sizeof(int)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  *cbmc_overlap = hiout[0];
  *ln_pseq = hout[0];
  *ln_pbias = hout[1];
  if (frag_order)
    for (int k = 0; k < s.nfrag; ++k) frag_order[k] = k < hiout[1] ? hiout[2 + k] + 1 : 0;
  if (xyz)
    for (int k = 0; k < 3 * s.natoms; ++k) xyz[k] = hout[2 + k];
  return CASS_OK;
}
