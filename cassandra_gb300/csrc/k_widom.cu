// k_widom.cu -- batched CBMC Widom insertion on the GPU.
//
//   k_cell_count / k_cell_scan / k_cell_scatter / k_cell_sort
//       per-box cell lists (counting sort, deterministic order inside a cell);
//       the GPU counterpart of Sector_Setup / CBMC_Cell_List_Setup
//       (sector_routines.f90:39-374).  Cells only accelerate the search:
//       every pair with r <= cutoff is visited exactly once, whatever the cell
//       count, so the energies are those of the molecule loop of
//       Compute_Molecule_Nonbond_Inter_Energy_Widom (energy_routines.f90:1266-1297).
//   k_widom
//       one thread per Widom insertion: Build_Molecule with kappa_ins first-
//       fragment trials and Fragment_Placement with kappa_dih dihedral trials
//       (fragment_growth.f90:72-707, 1449-2132), then the full-cutoff energy,
//       intramolecular and bonded energies of the grown molecule
//       (widom_insert.f90:320-447).  The CTA's box (cell-sorted atoms and cell
//       offsets) is staged in shared memory when it fits.
//   k_widom_recip
//       Update_System_Ewald_Reciprocal_Energy_Widom (energy_routines.f90:2500-2550)
//       for the insertions that survived, when the box carries an Ewald sum.
//   k_widom_finalize
//       widom_var = exp(-beta (dE - dE_frag) - ln_pbias) and the per-box sums
//       (widom_insert.f90:445-447, 538), in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cass_ctx.h"
#include "cass_cbmc.cuh"
#include "cass_cbmc_f.cuh"

namespace cassgpu {


struct BoxSrc {
  const double4_32a* p64;
  const float4* p32;
  const int4* meta;
};

// Per-insertion record: dE_intra, dE_inter (without reciprocal), dE_frag, ln_pbias.
using WRec = double4_32a;

// Widom cell edge rcut_cbmc / cells-per-cutoff, measured on the 64-box butane
// batch: with row-trimmed stencils, cells of a third of the cutoff visit 2.4x
// fewer candidates and the FP64 kernel runs 22 % faster than with cells of the
// cutoff; the FP32 kernel is fastest with cells of the cutoff (its time goes
// to set-up and divergence more than to candidates: 22.5 ms at 1, 26.0 ms at 2).
constexpr double kCellsPerCutoffFP64 = 3.0;
constexpr double kCellsPerCutoffMixed = 1.0;

__device__ __forceinline__ int wrapc(int c, int n) {
  c %= n;
  return c < 0 ? c + n : c;
}

// Periodic image of unwrapped cell c: the shift s (in box lengths) with
// c + s * n in [0, n); the division only runs outside one image either side
__device__ __forceinline__ int cell_image(int c, int n) {
  if (c >= 0 && c < n) return 0;
  if (c < 0 && c >= -n) return 1;
  if (c >= n && c < 2 * n) return -1;
  return (wrapc(c, n) - c) / n;
}

// ---------------------------------------------------------------------------
// K7: cell lists of the batch boxes
__device__ __forceinline__ int cell_index(const BoxDev& b, double x, double y, double z) {
  int c[3];
  double p[3] = {x, y, z};
  for (int d = 0; d < 3; ++d) {
    double w = p[d] - b.L[d] * floor((p[d] + b.hL[d]) / b.L[d]);  // wrapped into [-L/2, L/2)
    int k = (int)floor((w + b.hL[d]) * b.cell_inv[d]);
    c[d] = min(max(k, 0), b.nc[d] - 1);
  }
  return (c[2] * b.nc[1] + c[1]) * b.nc[0] + c[0];
}

__global__ void k_cell_count(const BoxSrc* src, const BoxDev* boxes, int* cell_of, int* count) {
  int k = blockIdx.y;
  const BoxDev& b = boxes[k];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.natoms) return;
  double4_32a p = src[k].p64[i];
  int c = cell_index(b, p.x, p.y, p.z);
  cell_of[b.atom_off + i] = c;
  atomicAdd(&count[b.cell_off + c], 1);
}

// exclusive scan of the box's cell counts; cstart holds local atom indices
__global__ void k_cell_scan(const BoxDev* boxes, const int* count, int* cstart, int* fill) {
  int k = blockIdx.x;
  const BoxDev& b = boxes[k];
  int nc = b.nc[0] * b.nc[1] * b.nc[2];
  __shared__ int carry;
  __shared__ int warp_tot[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  int* cs = cstart + b.cell_off + k;
  for (int base = 0; base < nc; base += blockDim.x) {
    int c = base + threadIdx.x;
    int v = c < nc ? count[b.cell_off + c] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) warp_tot[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      int nw = blockDim.x >> 5;
      int t = threadIdx.x < nw ? warp_tot[threadIdx.x] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, t, o);
        if (threadIdx.x >= o) t += y;
      }
      if (threadIdx.x < nw) warp_tot[threadIdx.x] = t;
    }
    __syncthreads();
    int w = threadIdx.x >> 5;
    int excl = x - v + (w > 0 ? warp_tot[w - 1] : 0) + carry;
    if (c < nc) {
      cs[c] = excl;
      fill[b.cell_off + c] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) cs[nc] = carry;
}

__global__ void k_cell_scatter(const BoxSrc* src, const BoxDev* boxes, const int* cell_of, const int* cstart,
                               int* fill, double4_32a* c64, float4* c32, int* ctype, float* cq32, int* corig) {
  int k = blockIdx.y;
  const BoxDev& b = boxes[k];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.natoms) return;
  int c = cell_of[b.atom_off + i];
  int pos = cstart[b.cell_off + k + c] + atomicAdd(&fill[b.cell_off + c], 1);
  int g = b.atom_off + pos;
  // the copies hold the positions their cells were chosen from, wrapped into
  // [-L/2, L/2) (an atom of a molecule folded by its COM may stick out of the
  // box), so that a query's per-row image shift is the whole periodic shift
  double4_32a p = src[k].p64[i];
  p.x = p.x - b.L[0] * floor((p.x + b.hL[0]) / b.L[0]);
  p.y = p.y - b.L[1] * floor((p.y + b.hL[1]) / b.L[1]);
  p.z = p.z - b.L[2] * floor((p.z + b.hL[2]) / b.L[2]);
  c64[g] = p;
  const float4 q = src[k].p32[i];
  c32[g] = make_float4((float)p.x, (float)p.y, (float)p.z, q.w);
  ctype[g] = src[k].meta[i].y;
  cq32[g] = (float)p.w;
  corig[g] = i;
}

// insertion sort of each cell by packed index: a deterministic order
__global__ void k_cell_sort(const BoxDev* boxes, int nb, const int* cstart, double4_32a* c64, float4* c32, int* ctype,
                            float* cq32, int* corig) {
  int k = blockIdx.y;
  if (k >= nb) return;
  const BoxDev& b = boxes[k];
  int nc = b.nc[0] * b.nc[1] * b.nc[2];
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int* cs = cstart + b.cell_off + k;
  int s = b.atom_off + cs[c], e = b.atom_off + cs[c + 1];
  for (int i = s + 1; i < e; ++i) {
    int key = corig[i];
    double4_32a a64 = c64[i];
    float4 a32 = c32[i];
    int at = ctype[i];
    float aq = cq32[i];
    int j = i - 1;
    while (j >= s && corig[j] > key) {
      corig[j + 1] = corig[j];
      c64[j + 1] = c64[j];
      c32[j + 1] = c32[j];
      ctype[j + 1] = ctype[j];
      cq32[j + 1] = cq32[j];
      --j;
    }
    corig[j + 1] = key;
    c64[j + 1] = a64;
    c32[j + 1] = a32;
    ctype[j + 1] = at;
    cq32[j + 1] = aq;
  }
}

// ---------------------------------------------------------------------------
// box queries

struct BoxView {
  const BoxDev* b;          // shared-memory copy
  const double4_32a* p64;   // cell-sorted FP64 atoms (x, y, z, q) of this box (smem or global)
  const int* ptype;         // their types (smem or global)
  const int* cstart;        // cell starts, local atom indices (smem or global)
  const int* corig;         // packed index of each cell-sorted atom (global; molecule-pair boxes)
  double rc_cbmc, rc_full;
};

// The test molecule of one energy call as Check_MoleculePair_Cutoff sees it
// (energy_routines.f90:3027-3088): the COM and max_dcom of its existing atoms
struct QueryMol {
  double com[3];
  double dcom;
};

// Energy of one test atom at p against every box atom within the cutoff.
// Returns true on core overlap (r^2 < rcut_low^2), as Compute_MoleculePair_Energy
// (energy_routines.f90:1676-1679) does.
struct PairCount {
  unsigned long long visited = 0, in_cut = 0;
  double eabs = 0.0;  // sum of |pair energy| of the current query
};

// With qm (a box with a molecule-pair cutoff) a candidate atom counts only when
// its molecule passes Check_MoleculePair_Cutoff against the test molecule:
// |COM - COM_j| <= (rcut_cbmc or rcut_max) + max_dcom + max_dcom_j, as the
// molecule loop of Compute_Molecule_Nonbond_Inter_Energy_Widom applies it
// (energy_routines.f90:1266-1297) -- the overlap test included.
__device__ bool query_box(const BoxView& V, const PairTable& T, const double p[3], int qt, double qch, bool cbmc,
                          bool want_qq, double& eout, PairCount& pc, const QueryMol* qm = nullptr) {
  const BoxDev& b = *V.b;
  double rc = cbmc ? V.rc_cbmc : V.rc_full;
  // minimum-image charges count every pair of a molecule within the
  // molecule-pair cutoff, in CBMC calls too: the whole box is searched
  if (qm && cbmc && want_qq && b.charge_style == CASS_CHARGE_COUL && b.charge_sum_style == CASS_QQ_MINIMUM)
    rc = 1e30;
  const double rint0 = cbmc ? V.rc_cbmc : b.rcut_max;
  int lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double u = (p[d] + b.hL[d]) * b.cell_inv[d];
    double w = fmin(rc * b.cell_inv[d], 1.0e6);
    int l = (int)floor(u - w - 1e-6), h = (int)floor(u + w + 1e-6);
    if (h - l + 1 >= b.nc[d]) {
      l = 0;
      h = b.nc[d] - 1;
    }
    lo[d] = l;
    hi[d] = h;
  }
  const bool qq_on = want_qq && b.charge_style == CASS_CHARGE_COUL;
  const double4_32a* P = V.p64;
  double acc = 0.0, eabs = 0.0;
  // rows of the stencil trimmed to the cutoff sphere: the distance from p to a
  // row's y and z slabs (less a margin of 1e-6 cell) leaves a chord in x
  const double rc2 = rc * rc;
  const bool fully = hi[1] - lo[1] + 1 >= b.nc[1], fullz = hi[2] - lo[2] + 1 >= b.nc[2];
  double ch[3];
  for (int d = 0; d < 3; ++d) ch[d] = b.L[d] / (double)b.nc[d];
  auto slab_d2 = [&](int c, int d) {
    const double c0 = (double)c * ch[d] - b.hL[d];
    const double e = fmax(fmax(c0 - p[d], p[d] - (c0 + ch[d])) - 1.0e-6 * ch[d], 0.0);
    return e * e;
  };
  for (int cz = lo[2]; cz <= hi[2]; ++cz) {
    int wz = wrapc(cz, b.nc[2]);
    const double dz2 = fullz ? 0.0 : slab_d2(cz, 2);
    if (dz2 > rc2) continue;
    for (int cy = lo[1]; cy <= hi[1]; ++cy) {
      const double d2 = fully ? dz2 : dz2 + slab_d2(cy, 1);
      if (d2 > rc2) continue;
      int xlo, xhi;
      {
        const double u = (p[0] + b.hL[0]) * b.cell_inv[0];
        const double w = fmin(sqrt(rc2 - d2) * b.cell_inv[0], 1.0e6);
        xlo = (int)floor(u - w - 1e-6);
        xhi = (int)floor(u + w + 1e-6);
        if (xhi - xlo + 1 >= b.nc[0]) {
          xlo = 0;
          xhi = b.nc[0] - 1;
        }
      }
      int row = (wz * b.nc[1] + wrapc(cy, b.nc[1])) * b.nc[0];
      int cx = xlo;
      while (cx <= xhi) {
        int wx = wrapc(cx, b.nc[0]);
        int run = min(xhi - cx, b.nc[0] - 1 - wx) + 1;
        int j1 = V.cstart[row + wx + run];
        pc.visited += (unsigned long long)(j1 - V.cstart[row + wx]);
        for (int j = V.cstart[row + wx]; j < j1; ++j) {
          if (qm) {  // Check_MoleculePair_Cutoff
            const double4_32a mc = b.mcom[V.corig[j]];
            const double cx = fold(qm->com[0] - mc.x, b.hL[0], b.L[0]);
            const double cy = fold(qm->com[1] - mc.y, b.hL[1], b.L[1]);
            const double cz = fold(qm->com[2] - mc.z, b.hL[2], b.L[2]);
            if (sqrt(cx * cx + cy * cy + cz * cz) > rint0 + qm->dcom + mc.w) continue;
          }
          double4_32a a = P[j];
          double dx = fold(p[0] - a.x, b.hL[0], b.L[0]);
          double dy = fold(p[1] - a.y, b.hL[1], b.L[1]);
          double dz = fold(p[2] - a.z, b.hL[2], b.L[2]);
          double r2 = dx * dx + dy * dy + dz * dz;
          if (cbmc && b.sector && r2 < rmin2_pair(b, T.ntypes, qt, V.ptype[j])) return true;  // check_overlap
          if (cbmc && b.tab_res > 0) {  // Estimate_MoleculePair_Energy
            double et = 0.0;
            const int k = table_pair(b, T.ntypes, r2, qt, V.ptype[j], qch, a.w, et);
            if (k == 2) return true;
            if (k == 1) {
              ++pc.in_cut;
              acc += et;
              eabs += fabs(et);
            }
            continue;
          }
          if (r2 < b.rcut_lowsq) return true;
          int m = cutoff_mask(b, r2, cbmc);
          if (!qq_on) m &= 1;
          if (m) ++pc.in_cut;
          if (m & 1) {
            double ev = vdw_pair(T, b, qt, V.ptype[j], r2, 1.0);
            acc += ev;
            eabs += fabs(ev);
          }
          if (m & 2) {
            double eq = qq_pair_inter(b, qch * a.w, r2);
            acc += eq;
            eabs += fabs(eq);
          }
        }
        cx += run;
      }
    }
  }
  eout = acc;
  pc.eabs = eabs;
  return false;
}

// Compute_Max_COM_Distance (get_com.f90:220-295) over the atoms of `mask`
__device__ inline double max_dcom_of(const double* r, unsigned mask, const double com[3], int n) {
  double dmax = 0.0;
  for (int k = 0; k < n; ++k) {
    if (!((mask >> k) & 1u)) continue;
    const double dx = r[3 * k] - com[0], dy = r[3 * k + 1] - com[1], dz = r[3 * k + 2] - com[2];
    dmax = fmax(dmax, dx * dx + dy * dy + dz * dz);
  }
  return sqrt(dmax);
}

// ---------------------------------------------------------------------------
// K8: one Widom insertion per thread

__device__ void run_insertion(const WidomSpecies& S, const SpeciesPools& P, const PairTable& T, const BoxView& V,
                              const double* __restrict__ lib, Lfsr rng, WRec& rec, int& status, double* xyz_out,
                              CassWidomTrace* tr, PairCount& pc) {
  const BoxDev& b = *V.b;
  const SpeciesDevHdr& H = P.hdr[S.is0];
  const int n = S.natoms;
  const double beta = b.beta;
  double r[3 * kMaxAtoms];
  unsigned exist = 0u;
  double ln_pbias = 0.0, ln_pseq;
  double first_sum = 0.0;
  int selected = 0;
  bool cbmc_overlap = false;

  // Step 1: first fragment and growth order (fragment_growth.f90:218-253, 1317-1446)
  double u = rng.next();
  int fstart = 0;
  while (fstart < S.nfrag && !(u < S.cum_prob_ins[fstart])) ++fstart;
  if (fstart >= S.nfrag) fstart = S.nfrag - 1;
  ln_pseq = S.ln_prob_ins[fstart];
  int order[kMaxFrags];
  int norder = 1;
  order[0] = fstart;
  unsigned live = 1u << fstart;
  if (S.nfrag > 1) {
    int hang[kMaxFrags];
    int nh = 0;
    for (int k = 0; k < S.frag_nconnect[fstart]; ++k) {
      int f = S.frag_connect[fstart][k];
      if (!((live >> f) & 1u)) hang[nh++] = f;
    }
    while (nh > 0) {
      double prob[kMaxFrags], cum[kMaxFrags];
      for (int k = 0; k < nh; ++k) {
        prob[k] = (double)(S.frag_natoms[hang[k]] - 2);
        cum[k] = (k == 0 ? 0.0 : cum[k - 1]) + prob[k];
      }
      double tot = cum[nh - 1];
      for (int k = 0; k < nh; ++k) {
        prob[k] = prob[k] / tot;
        cum[k] = cum[k] / tot;
      }
      double uu = rng.next();
      int k = 0;
      while (k < nh && !(uu < cum[k])) ++k;
      if (k >= nh) k = nh - 1;
      int f = hang[k];
      ln_pseq = ln_pseq + log(prob[k]);
      order[norder++] = f;
      live |= 1u << f;
      for (int q = k; q + 1 < nh; ++q) hang[q] = hang[q + 1];
      --nh;
      for (int q = 0; q < S.frag_nconnect[f]; ++q) {
        int g = S.frag_connect[f][q];
        if (!((live >> g) & 1u) && nh < kMaxFrags) hang[nh++] = g;
      }
    }
  }

  // Step 2: library conformation of the first fragment (:274-304)
  const int nfa = S.frag_natoms[fstart];
  {
    int nconf = S.nconfig[fstart];
    int conf = (int)(rng.next() * nconf);
    if (conf >= nconf) conf = nconf - 1;
    const double* L0 = lib + S.lib_off[fstart] + (size_t)conf * nfa * 3;
    for (int i = 0; i < nfa; ++i) {
      int a = S.frag_atoms[fstart][i];
      r[3 * a] = L0[3 * i];
      r[3 * a + 1] = L0[3 * i + 1];
      r[3 * a + 2] = L0[3 * i + 2];
      exist |= 1u << a;
    }
  }

  // Step 3: Get_COM + Rotate_Molecule_Eulerian (rotation_routines.f90:41-137)
  double com[3];
  get_com(S, r, exist, com);
  {
    double theta = acos(1.0 - 2.0 * rng.next());
    double phi = (1.0 - 2.0 * rng.next()) * kPI;
    double psi = (1.0 - 2.0 * rng.next()) * kPI;
    double st, ct, sp, cp, ss, cs;
    sincos(theta, &st, &ct);
    sincos(phi, &sp, &cp);
    sincos(psi, &ss, &cs);
    double r11 = cs * cp - ct * sp * ss, r12 = cs * sp + ct * cp * ss, r13 = ss * st;
    double r21 = -ss * cp - ct * sp * cs, r22 = -ss * sp + ct * cp * cs, r23 = cs * st;
    double r31 = st * sp, r32 = -st * cp, r33 = ct;
    for (int i = 0; i < nfa; ++i) {
      int a = S.frag_atoms[fstart][i];
      double x = r[3 * a] - com[0], y = r[3 * a + 1] - com[1], z = r[3 * a + 2] - com[2];
      r[3 * a] = (r11 * x + r12 * y + r13 * z) + com[0];
      r[3 * a + 1] = (r21 * x + r22 * y + r23 * z) + com[1];
      r[3 * a + 2] = (r31 * x + r32 * y + r33 * z) + com[2];
    }
  }

  // Step 4: kappa_ins trial positions of the first fragment (:383-620)
  const int ki = S.kappa_ins;
  double nrg[kMaxKappa], w[kMaxKappa];
  unsigned ovm = 0u;
  double r0[3 * kMaxAtoms];
  for (int i = 0; i < 3 * n; ++i) r0[i] = r[i];
  const double com_old[3] = {com[0], com[1], com[2]};
  // molecule-pair cutoff boxes: the fragment at a trial centre has that COM
  // and the max_dcom of its atoms about it
  const bool mp = b.mcom != nullptr;
  QueryMol qm;
  qm.dcom = 0.0;
  if (mp) qm.dcom = max_dcom_of(r0, exist, com_old, n);
  Lfsr replay = rng;
  for (int it = 0; it < ki; ++it) {
    double ax = (0.5 - rng.next()) * b.L[0];
    double ay = (0.5 - rng.next()) * b.L[1];
    double az = (0.5 - rng.next()) * b.L[2];
    qm.com[0] = ax;
    qm.com[1] = ay;
    qm.com[2] = az;
    double e = 0.0;
    bool ov = false;
    for (int i = 0; i < nfa && !ov; ++i) {
      int a = S.frag_atoms[fstart][i];
      double p[3] = {r0[3 * a] - com_old[0] + ax, r0[3 * a + 1] - com_old[1] + ay, r0[3 * a + 2] - com_old[2] + az};
      double ea;
      ov = query_box(V, T, p, S.type[a], S.q[a], true, S.want_qq_cbmc != 0, ea, pc, mp ? &qm : nullptr);
      e += ea;
    }
    nrg[it] = e;
    w[it] = 0.0;
    if (ov) {
      ovm |= 1u << it;
    } else {
      double nk = beta * nrg[it];
      if (nk >= kMAX_KBT) {
        ovm |= 1u << it;
      } else {
        w[it] = exp(-nk);
        first_sum += nrg[it];
      }
    }
    if (it > 0) w[it] = w[it - 1] + w[it];
  }
  int sel = -1;
  if (ovm == ((ki >= 32) ? 0xffffffffu : ((1u << ki) - 1u))) {
    cbmc_overlap = true;
  } else {
    double rn = rng.next() * w[ki - 1];
    int i = 0;
    while (i < ki && !(rn < w[i])) ++i;
    if (i == ki) cbmc_overlap = true;
    else sel = i;
  }
  if (!cbmc_overlap) {
    ln_pbias = ln_pbias - beta * nrg[sel] - log(w[ki - 1]);
    double ax = 0, ay = 0, az = 0;
    for (int k = 0; k <= sel; ++k) {
      ax = (0.5 - replay.next()) * b.L[0];
      ay = (0.5 - replay.next()) * b.L[1];
      az = (0.5 - replay.next()) * b.L[2];
    }
    for (int i = 0; i < nfa; ++i) {
      int a = S.frag_atoms[fstart][i];
      r[3 * a] = r0[3 * a] - com_old[0] + ax;
      r[3 * a + 1] = r0[3 * a + 1] - com_old[1] + ay;
      r[3 * a + 2] = r0[3 * a + 2] - com_old[2] + az;
    }
    selected = sel + 1;
  }

  // Step 5: Fragment_Placement (:1449-2132)
  if (!cbmc_overlap && norder > 1) {
    double e_prev = dihedral_masked(H, P, r, exist);
    unsigned placed = 1u << fstart;
    const int kd = S.kappa_dih;
    double dn[kMaxKappa], dd[kMaxKappa];
    for (int oi = 1; oi < norder && !cbmc_overlap; ++oi) {
      const int f = order[oi];
      const int nf = S.frag_natoms[f];
      unsigned grown = exist;
      int nconf = S.nconfig[f];
      int cf = (int)(rng.next() * nconf);
      cf = (int)(rng.next() * nconf);  // the duplicated draw of fragment_growth.f90:1578,1584
      if (cf >= nconf) cf = nconf - 1;
      double cfg[3 * kMaxAtoms];
      const double* Lf = lib + S.lib_off[f] + (size_t)cf * nf * 3;
      for (int j = 0; j < nf; ++j) {
        int a = S.frag_atoms[f][j];
        exist |= 1u << a;
        cfg[3 * a] = Lf[3 * j];
        cfg[3 * a + 1] = Lf[3 * j + 1];
        cfg[3 * a + 2] = Lf[3 * j + 2];
      }
      const unsigned combined = exist, newex = combined & ~grown;
      int fc = -1;
      for (int q = 0; q < S.frag_nconnect[f]; ++q) {
        int g = S.frag_connect[f][q];
        if ((placed >> g) & 1u) {
          fc = g;
          break;
        }
      }
      if (fc < 0) {  // no placed neighbour: the fragment graph is not connected
        cbmc_overlap = true;
        break;
      }
      const int anc_i = S.frag_atoms[f][0], anc_c = S.frag_atoms[fc][0];
      int ids[kMaxAtoms], nid = 0;
      for (int j = 0; j < nf; ++j) {
        int a = S.frag_atoms[f][j];
        if (a != anc_i && a != anc_c) ids[nid++] = a;
      }
      unsigned idmask = 0u;
      for (int j = 0; j < nid; ++j) idmask |= 1u << ids[j];
      int atom_ifrag = nid > 0 ? ids[0] : S.frag_atoms[f][nf - 1];
      int atom_fc = S.frag_atoms[fc][S.frag_natoms[fc] - 1];
      for (int j = 0; j < S.frag_natoms[fc]; ++j) {
        int a = S.frag_atoms[fc][j];
        if (a != anc_i && a != anc_c) {
          atom_fc = a;
          break;
        }
      }
      double v1[3], v2[3], al_i[9], hg_i[9], al_c[9], hg_c[9];
      for (int d = 0; d < 3; ++d) {
        v1[d] = cfg[3 * anc_i + d] - cfg[3 * anc_c + d];
        v2[d] = cfg[3 * atom_ifrag + d] - cfg[3 * anc_c + d];
      }
      aligner_hanger(v1, v2, al_i, hg_i);
      for (int d = 0; d < 3; ++d) {
        v1[d] = r[3 * anc_i + d] - r[3 * anc_c + d];
        v2[d] = r[3 * atom_fc + d] - r[3 * anc_c + d];
      }
      aligner_hanger(v1, v2, al_c, hg_c);
      const double tx = cfg[3 * anc_c], ty = cfg[3 * anc_c + 1], tz = cfg[3 * anc_c + 2];
      for (int j = 0; j < nf; ++j) {
        int a = S.frag_atoms[f][j];
        double x = cfg[3 * a] - tx, y = cfg[3 * a + 1] - ty, z = cfg[3 * a + 2] - tz;
        cfg[3 * a] = x * al_i[0] + y * al_i[1] + z * al_i[2];
        cfg[3 * a + 1] = x * al_i[3] + y * al_i[4] + z * al_i[5];
        cfg[3 * a + 2] = x * al_i[6] + y * al_i[7] + z * al_i[8];
      }
      const double theta0 = kTWOPI * rng.next();
      const double dtheta = kTWOPI / (double)kd;
      unsigned dov = 0u;
      double dw[kMaxKappa];
      double theta = theta0;
      for (int ii = 0; ii < kd; ++ii) {
        if (ii > 0) theta = theta + dtheta;
        double sth, cth;
        sincos(theta, &sth, &cth);
        for (int j = 0; j < nid; ++j) {
          int a = ids[j];
          double x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
          double yr = cth * y + sth * z, zr = -sth * y + cth * z;
          r[3 * a] = (x * hg_c[0] + yr * hg_c[1] + zr * hg_c[2]) + r[3 * anc_c];
          r[3 * a + 1] = (x * hg_c[3] + yr * hg_c[4] + zr * hg_c[5]) + r[3 * anc_c + 1];
          r[3 * a + 2] = (x * hg_c[6] + yr * hg_c[7] + zr * hg_c[8]) + r[3 * anc_c + 2];
        }
        dn[ii] = 0.0;
        dd[ii] = 0.0;
        exist &= ~idmask;
        double niv = 0.0, niq = 0.0, noq = 0.0;
        bool ov = false;
        for (int j = 0; j < nid; ++j) {
          exist |= 1u << ids[j];
          double eiv, eiq, eoq;
          if (atom_intra(H, P, b, T, ids[j], r, exist, eiv, eiq, eoq)) {
            ov = true;
            break;
          }
          niv += eiv;
          niq += eiq;
          noq += eoq;
        }
        if (ov) {
          dw[ii] = ii > 0 ? dw[ii - 1] : 0.0;
          dov |= 1u << ii;
          exist |= idmask;
          continue;
        }
        double einter = 0.0;
        if (mp) {  // the new atoms of the trial (fragment_growth.f90 Fragment_Placement energy call)
          get_com(S, r, newex, qm.com);
          qm.dcom = max_dcom_of(r, newex, qm.com, n);
        }
        for (int a = 0; a < n && !ov; ++a) {
          if (!((newex >> a) & 1u)) continue;
          double p[3] = {r[3 * a], r[3 * a + 1], r[3 * a + 2]};
          double ea;
          ov = query_box(V, T, p, S.type[a], S.q[a], true, S.want_qq_cbmc != 0, ea, pc, mp ? &qm : nullptr);
          einter += ea;
        }
        exist = combined;
        if (ov) {
          dw[ii] = 0.0;
          dov |= 1u << ii;
        } else {
          double ed = dihedral_masked(H, P, r, exist);
          dd[ii] = ed;
          dn[ii] = ed + niv + niq + einter + noq - e_prev;
          double nk = beta * dn[ii];
          if (nk >= kMAX_KBT) {
            dw[ii] = 0.0;
            dov |= 1u << ii;
          } else {
            dw[ii] = exp(-nk);
          }
        }
        if (ii > 0) dw[ii] = dw[ii - 1] + dw[ii];
      }
      if (dov == ((kd >= 32) ? 0xffffffffu : ((1u << kd) - 1u))) {
        cbmc_overlap = true;
        break;
      }
      double pp = rng.next() * dw[kd - 1];
      int trl = 0;
      while (trl < kd && !(pp < dw[trl])) ++trl;
      if (trl == kd) {
        cbmc_overlap = true;
        break;
      }
      ln_pbias = ln_pbias - beta * dn[trl] - log(dw[kd - 1]);
      theta = theta0;
      for (int ii = 1; ii <= trl; ++ii) theta = theta + dtheta;
      double sth, cth;
      sincos(theta, &sth, &cth);
      for (int j = 0; j < nid; ++j) {
        int a = ids[j];
        double x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
        double yr = cth * y + sth * z, zr = -sth * y + cth * z;
        r[3 * a] = (x * hg_c[0] + yr * hg_c[1] + zr * hg_c[2]) + r[3 * anc_c];
        r[3 * a + 1] = (x * hg_c[3] + yr * hg_c[4] + zr * hg_c[5]) + r[3 * anc_c + 1];
        r[3 * a + 2] = (x * hg_c[6] + yr * hg_c[7] + zr * hg_c[8]) + r[3 * anc_c + 2];
      }
      e_prev = dd[trl];
      placed |= 1u << f;
    }
    if (!cbmc_overlap) get_com(S, r, exist, com);
  }

  // widom_insert.f90:350-447
  ln_pbias = ln_pbias + ln_pseq;
  ln_pbias = ln_pbias + S.ln_kappa_ins;
  ln_pbias = ln_pbias + S.ln_kappa_dih_term;
  if (tr) {
    tr->ln_pbias = ln_pbias;
    tr->e_first_trial_sum = first_sum;
    tr->selected_trial = selected;
    tr->e_inter = 0.0;
    tr->e_inter_abs = 0.0;
  }
  rec = make_double4_32a(0.0, 0.0, 0.0, ln_pbias);
  if (cbmc_overlap) {
    status = 1;
    return;
  }
  const unsigned all = (n >= 32) ? 0xffffffffu : ((1u << n) - 1u);
  exist = all;
  if (S.nfrag > 1) {  // Fold_Molecule, orthorhombic branch
    for (int d = 0; d < 3; ++d) {
      if (com[d] > b.hL[d]) {
        com[d] = com[d] - b.L[d];
        for (int a = 0; a < n; ++a) r[3 * a + d] -= b.L[d];
      } else if (com[d] < -b.hL[d]) {
        com[d] = com[d] + b.L[d];
        for (int a = 0; a < n; ++a) r[3 * a + d] += b.L[d];
      }
    }
  }
  double e_inter = 0.0, e_abs = 0.0;
  if (mp) {  // the whole molecule, folded
    get_com(S, r, exist, qm.com);
    qm.dcom = max_dcom_of(r, exist, qm.com, n);
  }
  for (int a = 0; a < n; ++a) {
    double p[3] = {r[3 * a], r[3 * a + 1], r[3 * a + 2]};
    double ea;
    if (query_box(V, T, p, S.type[a], S.q[a], false, true, ea, pc, mp ? &qm : nullptr)) {
      status = 2;
      return;
    }
    e_inter += ea;
    e_abs += pc.eabs;
  }
  IntraOut io = molecule_intra(P, S.is0, b, T, r);
  if (io.overlap) {
    status = 3;
    return;
  }
  e_inter = e_inter + io.pqq;
  double dE_inter = e_inter + b.e_inter_constant;
  double dE_intra = io.ivdw + io.iqq;
  dE_intra = dE_intra + io.bond + io.angle + io.dih + io.imp;
  rec = make_double4_32a(dE_intra, dE_inter, io.angle, ln_pbias);
  status = 0;
  if (tr) {
    tr->e_inter = e_inter;
    tr->e_inter_abs = e_abs;
  }
  if (xyz_out)
    for (int i = 0; i < 3 * n; ++i) xyz_out[i] = r[i];
}

// ---------------------------------------------------------------------------
// Mixed-precision Widom kernel: one insertion per thread, FP32 throughout.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so this kernel reads only FP32
// tables (species, box constants, fragment libraries, cell-sorted atoms) and
// keeps the test molecule, the trial energies and the Boltzmann weights in
// FP32; pair energies accumulate in compensated FP32 sums.  Only the
// per-insertion record is widened to FP64 (adding the box's FP64 constant
// E_lrc_diff + E_self - E_recip_old).  Cell stencils carry a per-row
// periodic image shift, so the minimum-image fold per pair is needed only in
// a dimension whose stencil spans the whole box.

// Cell-list view of the CTA's box
struct BoxViewF {
  const BoxF* f;
  const float4* p32;   // cell-sorted atoms (x, y, z, type bits), smem or global
  const double4_32a* p64;  // the same atoms in FP64 (global): cutoff decisions near a cutoff
  const float* q32;    // their charges (global)
  const int* cstart;   // cell starts, local atom indices, smem or global
  const float2* ljp;   // (eps, sigma^2) [kMaxTypes][kMaxTypes], smem
};

// A pair of the full-cutoff pass whose FP32 r^2 lies within the band of a
// cutoff (kind 0: rcut_vdw^2 or rcut_coul^2; kind 1: rcut_low^2) where the
// FP32 and the FP64 decisions can differ: box atom j, test atom `atom`
struct BandPair {
  int j;
  float r2;
  unsigned char atom, kind, pad0, pad1;
};
constexpr int kMaxBand = 4;

struct QueryAcc {
  KahanF e;
  float eabs = 0.0f;
  unsigned long long visited = 0, in_cut = 0;
  int nband = 0, atom = 0;      // kQDetect: band pairs met, the current test atom
  BandPair* band = nullptr;     // kQDetect: the first kMaxBand of them
};

// Query modes.  kQPlain: FP32 decisions.  kQDetect (the full-cutoff pass of
// the FP32 growth): FP32 decisions, every pair within a band noted in A (a
// pair in the band of rcut_low^2 counts as no overlap and adds its energy;
// only an FP32 r^2 below the band is a certain overlap).  kQExact: decisions
// inside a band made in FP64 from the FP64 coordinates p64.
constexpr int kQPlain = 0, kQDetect = 1, kQExact = 2;

__device__ __forceinline__ void band_note(QueryAcc& A, int j, float r2, int kind) {
  if (A.nband < kMaxBand) A.band[A.nband] = BandPair{j, r2, (unsigned char)A.atom, (unsigned char)kind, 0, 0};
  ++A.nband;
}

// r^2 to a stored atom, through the row's image shift (folded in full dimensions)
__device__ __forceinline__ float pair_r2(const BoxF& f, const bool (&full)[3], bool fold_any, float qx, float qy,
                                         float qz, const float4& a) {
  float dx = qx - a.x, dy = qy - a.y, dz = qz - a.z;
  if (fold_any) {
    if (full[0]) dx = fold(dx, f.hL[0], f.L[0]);
    if (full[1]) dy = fold(dy, f.hL[1], f.L[1]);
    if (full[2]) dz = fold(dz, f.hL[2], f.L[2]);
  }
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// r^2 of two stored atoms at once on the packed FP32x2 pipe (FFMA2, sm_100 and
// later): the same operations and rounding as pair_r2 without a fold,
// qx - a.x formed as fma(a.x, -1, qx)
__device__ __forceinline__ float2 pair_r2_x2(float qx, float qy, float qz, const float4& a0, const float4& a1) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  const float2 dx = __ffma2_rn(make_float2(a0.x, a1.x), m1, make_float2(qx, qx));
  const float2 dy = __ffma2_rn(make_float2(a0.y, a1.y), m1, make_float2(qy, qy));
  const float2 dz = __ffma2_rn(make_float2(a0.z, a1.z), m1, make_float2(qz, qz));
  return __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
}

// Squared distance from coordinate p to the slab of unwrapped cell c (edge h,
// cells numbered from -hL), less a margin of 1e-3 cell so that FP32 rounding
// never drops a cell that holds an atom within the cutoff.
__device__ __forceinline__ float slab_d2_f(int c, float h, float hl, float p) {
  const float c0 = (float)c * h - hl;
  const float d = fmaxf(fmaxf(c0 - p, p - (c0 + h)) - 1.0e-3f * h, 0.0f);
  return d * d;
}

// The x-cells of a stencil row whose y / z slabs lie at squared distance d2
// from the query: the chord of the cutoff sphere, rem = rc^2 - d2 >= 0.  A row
// chord spanning the whole box is visited once with the minimum-image fold.
__device__ __forceinline__ void row_x_cells_f(const BoxF& f, float px, float rem, int& lo, int& hi, bool& fullx) {
  const float w = fminf(sqrtf(rem) * f.cinv[0], 1.0e5f);
  const float u = (px + f.hL[0]) * f.cinv[0];
  const int l = (int)floorf(fminf(fmaxf(u - w - 1e-3f, -1.0e6f), 1.0e6f));
  const int h = (int)floorf(fminf(fmaxf(u + w + 1e-3f, -1.0e6f), 1.0e6f));
  fullx = h - l + 1 >= f.nc[0];
  lo = fullx ? 0 : l;
  hi = fullx ? f.nc[0] - 1 : h;
}

// FP64 minimum-image r^2 between p and cell-sorted atom j, as the FP64 query
// forms it (Minimum_Image_Separation, orthorhombic branch)
__device__ __noinline__ double exact_r2(const BoxF& f, const double4_32a* p64, int j, const double* p) {
  const double4_32a a = p64[j];
  const double dx = fold(p[0] - a.x, f.hL64[0], f.L64[0]);
  const double dy = fold(p[1] - a.y, f.hL64[1], f.L64[1]);
  const double dz = fold(p[2] - a.z, f.hL64[2], f.L64[2]);
  return dx * dx + dy * dy + dz * dz;
}

// Core overlap of the full-cutoff pass: an FP32 r^2 within band_low of
// rcut_low^2 is decided from the FP64 coordinates
__device__ __forceinline__ bool overlap_exact(const BoxViewF& V, float r2, int j, const double* p64) {
  const BoxF& f = *V.f;
  if (r2 < f.low2 - f.band_low) return true;
  if (r2 >= f.low2 + f.band_low) return false;
  return exact_r2(f, V.p64, j, p64) < f.low2d;
}

// LJ and real-space Ewald energy of one pair inside the selection radius.
// kQDetect flags a pair at or above the lower edge rlo of the cutoff bands;
// kQExact compares an FP32 r^2 within a band of the vdW or Coulomb cutoff with
// the cutoff in FP64, from the FP64 coordinates, so that the pair counts
// exactly when the FP64 energy counts it.
template <bool COUNT, int MODE = kQPlain>
__device__ __forceinline__ void pair_energy(const BoxViewF& V, QueryAcc& A, const float4& a, int j, float r2,
                                            const float2* lrow, bool vdw_on, bool qq_on, float rv2, float rq2,
                                            float qa, float rlo = 0.0f, const double* p64 = nullptr) {
  bool in_v = r2 <= rv2, in_q = r2 <= rq2;
  if (MODE == kQDetect && r2 >= rlo) band_note(A, j, r2, 0);
  if (MODE == kQExact) {
    const BoxF& f = *V.f;
    if (fabsf(r2 - rv2) <= f.band_v || fabsf(r2 - rq2) <= f.band_q) {
      const double d2 = exact_r2(f, V.p64, j, p64);
      in_v = d2 <= f.rv2d;
      in_q = d2 <= f.rq2d;
    }
    if (!in_v && !in_q) return;
  }
  if (COUNT) ++A.in_cut;
  const int tj = __float_as_int(a.w);
  if (vdw_on && tj >= 0 && in_v) {
    const float2 es = lrow[tj];
    const float ev = lj_pair_f(es.x, es.y, r2);
    A.e.add(ev);
    A.eabs += fabsf(ev);
  }
  if (qq_on && in_q) {
    const float eq = qq_ewald_inter_f(V.f->alpha, qa * V.q32[j], r2);
    A.e.add(eq);
    A.eabs += fabsf(eq);
  }
}

// FP32 energy of one test atom at p against the box atoms within the cutoff,
// added to A.  Returns true on core overlap (r^2 < rcut_low^2), as
// Compute_MoleculePair_Energy (energy_routines.f90:1676-1679) does.
// A CBMC query with the CBMC options: check_overlap against r_min^2 of the
// type pair and, with the energy table, Estimate_MoleculePair_Energy per pair
// (FP32 table; a pair's bin can differ from FP64 within rounding of a bin edge)
__device__ bool query_f_opt(const BoxViewF& V, QueryAcc& A, float px, float py, float pz, int ta, float qa) {
  const BoxF& f = *V.f;
  const float rc = f.rc_cbmc;
  const float p[3] = {px, py, pz};
  int lo[3], hi[3];
  bool full[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float w = fminf(rc * f.cinv[d], 1.0e5f);
    const float ul = fminf(fmaxf((p[d] + f.hL[d]) * f.cinv[d] - w - 1e-3f, -1.0e6f), 1.0e6f);
    const float uh = fminf(fmaxf((p[d] + f.hL[d]) * f.cinv[d] + w + 1e-3f, -1.0e6f), 1.0e6f);
    const int l = (int)floorf(ul), h = (int)floorf(uh);
    full[d] = h - l + 1 >= f.nc[d];
    lo[d] = full[d] ? 0 : l;
    hi[d] = full[d] ? f.nc[d] - 1 : h;
  }
  const bool vdw_on = ta >= 0;
  const bool qq_on = f.charge_on && qa != 0.0f;
  const float rsel2 = f.rcb2;
  const float rc2 = rc * rc;
  const float2* lrow = V.ljp + (vdw_on ? ta : 0) * kMaxTypes;
  const float* rmrow = f.rmin2 + (vdw_on ? ta : 0) * kMaxTypes;
  const float qicf = qa * (float)kCHARGE_FACTOR;
  const int nc0 = f.nc[0], nc1 = f.nc[1], nc2 = f.nc[2];
  for (int cz = lo[2]; cz <= hi[2]; ++cz) {
    const int sz = cell_image(cz, nc2);
    const int wz = cz + sz * nc2;
    const float qz = pz + (float)sz * f.L[2];
    const float dz2 = full[2] ? 0.0f : slab_d2_f(cz, f.ch[2], f.hL[2], pz);
    if (dz2 > rc2) continue;
    for (int cy = lo[1]; cy <= hi[1]; ++cy) {
      const float d2 = full[1] ? dz2 : dz2 + slab_d2_f(cy, f.ch[1], f.hL[1], py);
      if (d2 > rc2) continue;
      int xlo, xhi;
      bool fl[3] = {false, full[1], full[2]};
      row_x_cells_f(f, px, rc2 - d2, xlo, xhi, fl[0]);
      const bool fold_any = fl[0] || fl[1] || fl[2];
      const int sy = cell_image(cy, nc1);
      const int wy = cy + sy * nc1;
      const float qy = py + (float)sy * f.L[1];
      const int row = (wz * nc1 + wy) * nc0;
      int cx = xlo;
      while (cx <= xhi) {
        const int sx = cell_image(cx, nc0);
        const int wx = cx + sx * nc0;
        const int run = min(xhi - cx, nc0 - 1 - wx) + 1;
        const float qx = px + (float)sx * f.L[0];
        const int j0 = V.cstart[row + wx], j1 = V.cstart[row + wx + run];
        for (int j = j0; j < j1; ++j) {
          const float4 a = V.p32[j];
          const float r2 = pair_r2(f, fl, fold_any, qx, qy, qz, a);
          const int tj = __float_as_int(a.w);
          if (f.sector && r2 < (vdw_on && tj >= 0 ? rmrow[tj] : f.low2)) return true;
          if (f.tab_res > 0) {
            float e = 0.0f;
            const int k = table_pair_f(f.tab_v, f.tab_f2, f.tab_res, f.tab_shift, f.tab_rcs, f.tab_step,
                                       f.tab_inv_step, f.ntypes, r2, ta, tj, qicf, qq_on ? V.q32[j] : 0.0f, e);
            if (k == 2) return true;
            if (k == 1) {
              A.e.add(e);
              A.eabs += fabsf(e);
            }
          } else {
            if (r2 < f.low2) return true;
            if (r2 <= rsel2) pair_energy<false>(V, A, a, j, r2, lrow, vdw_on, qq_on, f.rcb2, f.rcb2, qa);
          }
        }
        cx += run;
      }
    }
  }
  return false;
}

// MODE: kQPlain, kQDetect or kQExact (then p64 holds the FP64 coordinates of
// the query atom).
template <bool COUNT, bool OPT = false, int MODE = kQPlain>
__device__ bool query_f(const BoxViewF& V, QueryAcc& A, float px, float py, float pz, int ta, float qa, bool cbmc,
                        bool want_qq, const double* p64 = nullptr) {
  if (OPT && cbmc) return query_f_opt(V, A, px, py, pz, ta, qa);
  const BoxF& f = *V.f;
  const float rc = cbmc ? f.rc_cbmc : f.rc_full;
  const float p[3] = {px, py, pz};
  int lo[3], hi[3];
  bool full[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float w = fminf(rc * f.cinv[d], 1.0e5f);
    const float ul = fminf(fmaxf((p[d] + f.hL[d]) * f.cinv[d] - w - 1e-3f, -1.0e6f), 1.0e6f);
    const float uh = fminf(fmaxf((p[d] + f.hL[d]) * f.cinv[d] + w + 1e-3f, -1.0e6f), 1.0e6f);
    const int l = (int)floorf(ul), h = (int)floorf(uh);
    full[d] = h - l + 1 >= f.nc[d];
    lo[d] = full[d] ? 0 : l;
    hi[d] = full[d] ? f.nc[d] - 1 : h;
  }
  const float rv2 = cbmc ? f.rcb2 : f.rv2;
  const float rq2 = cbmc ? f.rcb2 : f.rq2;
  const float low2 = f.low2;
  const bool vdw_on = ta >= 0;
  const bool qq_on = want_qq && f.charge_on && qa != 0.0f;
  // the selection and overlap radii, widened by the FP32 bands in the
  // kQDetect and kQExact modes; rlo: the lower edge of the cutoff bands
  const float band = MODE != kQPlain ? fmaxf(vdw_on ? f.band_v : 0.0f, qq_on ? f.band_q : 0.0f) : 0.0f;
  const float rsel2 = fmaxf(vdw_on ? rv2 : -1.0f, qq_on ? rq2 : -1.0f) + band;
  const float low2q = MODE != kQPlain ? low2 + f.band_low : low2;
  const float rlo = fminf(vdw_on ? rv2 : 3.0e38f, qq_on ? rq2 : 3.0e38f) - band;
  const float rc2 = rc * rc;
  const float2* lrow = V.ljp + (vdw_on ? ta : 0) * kMaxTypes;
  const int nc0 = f.nc[0], nc1 = f.nc[1], nc2 = f.nc[2];
  for (int cz = lo[2]; cz <= hi[2]; ++cz) {
    const int sz = cell_image(cz, nc2);
    const int wz = cz + sz * nc2;
    const float qz = pz + (float)sz * f.L[2];
    const float dz2 = full[2] ? 0.0f : slab_d2_f(cz, f.ch[2], f.hL[2], pz);
    if (dz2 > rc2) continue;
    for (int cy = lo[1]; cy <= hi[1]; ++cy) {
      const float d2 = full[1] ? dz2 : dz2 + slab_d2_f(cy, f.ch[1], f.hL[1], py);
      if (d2 > rc2) continue;
      int xlo, xhi;
      bool fl[3] = {false, full[1], full[2]};
      row_x_cells_f(f, px, rc2 - d2, xlo, xhi, fl[0]);
      const bool fold_any = fl[0] || fl[1] || fl[2];
      const int sy = cell_image(cy, nc1);
      const int wy = cy + sy * nc1;
      const float qy = py + (float)sy * f.L[1];
      const int row = (wz * nc1 + wy) * nc0;
      int cx = xlo;
      while (cx <= xhi) {
        const int sx = cell_image(cx, nc0);
        const int wx = cx + sx * nc0;
        const int run = min(xhi - cx, nc0 - 1 - wx) + 1;
        const float qx = px + (float)sx * f.L[0];
        const int j0 = V.cstart[row + wx], j1 = V.cstart[row + wx + run];
        if (COUNT) A.visited += (unsigned long long)(j1 - j0);
        // two candidates per iteration: independent distance chains
        int j = j0;
        for (; j + 1 < j1; j += 2) {
          const float4 a0 = V.p32[j], a1 = V.p32[j + 1];
          float r20, r21;
          if (!fold_any) {
            const float2 r2 = pair_r2_x2(qx, qy, qz, a0, a1);
            r20 = r2.x;
            r21 = r2.y;
          } else {
            r20 = pair_r2(f, fl, fold_any, qx, qy, qz, a0);
            r21 = pair_r2(f, fl, fold_any, qx, qy, qz, a1);
          }
          if (fminf(r20, r21) < low2q) {
            if (MODE == kQPlain) return true;
            if (MODE == kQDetect) {
              if (fminf(r20, r21) < low2 - f.band_low) return true;  // a certain overlap
              if (r20 < low2q) band_note(A, j, r20, 1);
              if (r21 < low2q) band_note(A, j + 1, r21, 1);
            } else if (overlap_exact(V, r20, j, p64) || overlap_exact(V, r21, j + 1, p64)) {
              return true;
            }
          }
          if (r20 <= rsel2) pair_energy<COUNT, MODE>(V, A, a0, j, r20, lrow, vdw_on, qq_on, rv2, rq2, qa, rlo, p64);
          if (r21 <= rsel2) pair_energy<COUNT, MODE>(V, A, a1, j + 1, r21, lrow, vdw_on, qq_on, rv2, rq2, qa, rlo, p64);
        }
        if (j < j1) {
          const float4 a0 = V.p32[j];
          const float r20 = pair_r2(f, fl, fold_any, qx, qy, qz, a0);
          if (r20 < low2q) {
            if (MODE == kQPlain) return true;
            if (MODE == kQDetect) {
              if (r20 < low2 - f.band_low) return true;
              band_note(A, j, r20, 1);
            } else if (overlap_exact(V, r20, j, p64)) {
              return true;
            }
          }
          if (r20 <= rsel2) pair_energy<COUNT, MODE>(V, A, a0, j, r20, lrow, vdw_on, qq_on, rv2, rq2, qa, rlo, p64);
        }
        cx += run;
      }
    }
  }
  return false;
}

// Record of one insertion (FP32 parts; the full-cutoff energy as a two-term sum)
struct RecF {
  float dE_intra, dE_frag, ln_pbias, e_abs, first_sum;
  double e_inter;
  int status, selected;
  bool fix;  // the full-cutoff pass met a band: k_widom_fix redoes it
};

// An insertion queued for k_widom_fix: its index in the box and the choices of
// its FP32 growth (growth order, first-fragment trial, dihedral trials)
struct FixEntry {
  int ins;
  unsigned char sel, norder, pad0, pad1;
  unsigned char order[kMaxFrags];
  unsigned char trl[kMaxFrags];
  int nband;                   // band pairs met (more than kMaxBand: the pass is redone)
  BandPair band[kMaxBand];
};

// Get_Aligner_Hanger with reciprocal square roots (row-major): the frame of
// aligner_hanger to a few ulps
__device__ inline void aligner_hanger_rs(double v1[3], double v2[3], double al[9], double hg[9]) {
  const double n1 = rsqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  for (int i = 0; i < 3; ++i) v1[i] = v1[i] * n1;
  const double n2 = rsqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  for (int i = 0; i < 3; ++i) v2[i] = v2[i] * n2;
  double p1[3] = {v1[1] * v2[2] - v1[2] * v2[1], -v1[0] * v2[2] + v1[2] * v2[0], v1[0] * v2[1] - v1[1] * v2[0]};
  const double np1 = rsqrt(p1[0] * p1[0] + p1[1] * p1[1] + p1[2] * p1[2]);
  for (int i = 0; i < 3; ++i) p1[i] = p1[i] * np1;
  double p2[3] = {v1[1] * p1[2] - v1[2] * p1[1], -v1[0] * p1[2] + v1[2] * p1[0], v1[0] * p1[1] - v1[1] * p1[0]};
  const double np2 = rsqrt(p2[0] * p2[0] + p2[1] * p2[1] + p2[2] * p2[2]);
  for (int i = 0; i < 3; ++i) p2[i] = p2[i] * np2;
  for (int i = 0; i < 3; ++i) {
    al[i] = v1[i];
    al[3 + i] = p2[i];
    al[6 + i] = p1[i];
    hg[i * 3 + 0] = v1[i];
    hg[i * 3 + 1] = p2[i];
    hg[i * 3 + 2] = p1[i];
  }
}

// The grown molecule again in FP64 (the arithmetic of run_insertion): the
// same lfsr258 stream from the insertion's first draw, the choices the FP32
// growth made (first fragment and order, selected first-fragment trial, the
// selected dihedral trial of each later fragment) and the FP64 fragment
// library.  Library conformations are taken with the same 32-bit rule as the
// FP32 growth; every geometry uniform is the full FP64 draw, and the angles'
// sines and cosines and the frames' normalisations agree with the FP64 path's
// to a few ulps, so the coordinates are those of the FP64 path for the same
// choices to about 1e-15 A.  Ends with
// Fold_Molecule (orthorhombic branch) as Widom_Insert does before the
// full-cutoff energy.
__device__ inline void replay_molecule_f64(const WidomSpecies& S, const BoxF& f, const double* __restrict__ lib,
                                           Lfsr g, const int* order, int norder, int sel, const int* trls,
                                           double* r) {
  const int n = S.natoms;
  for (int k = 0; k < norder; ++k) g.next_bits();  // first fragment, growth order
  const int f0 = order[0];
  const int nfa = S.frag_natoms[f0];
  unsigned exist = 0u;
  {
    const int conf = index_of(draw_u32(g), S.nconfig[f0]);
    const double* L0 = lib + S.lib_off[f0] + (size_t)conf * nfa * 3;
    for (int i = 0; i < nfa; ++i) {
      const int a = S.frag_atoms[f0][i];
      r[3 * a] = L0[3 * i];
      r[3 * a + 1] = L0[3 * i + 1];
      r[3 * a + 2] = L0[3 * i + 2];
      exist |= 1u << a;
    }
  }
  double com[3];
  get_com(S, r, exist, com);
  {
    // theta = acos(1 - 2u): cos theta = 1 - 2u, sin theta = 2 sqrt(u (1 - u));
    // phi, psi = (1 - 2u) pi through sincospi (the same angles to a few ulps)
    const double ut = g.next();
    const double ct = 1.0 - 2.0 * ut, st = 2.0 * sqrt(ut * (1.0 - ut));
    double sp, cp, ss, cs;
    sincospi(1.0 - 2.0 * g.next(), &sp, &cp);
    sincospi(1.0 - 2.0 * g.next(), &ss, &cs);
    const double r11 = cs * cp - ct * sp * ss, r12 = cs * sp + ct * cp * ss, r13 = ss * st;
    const double r21 = -ss * cp - ct * sp * cs, r22 = -ss * sp + ct * cp * cs, r23 = cs * st;
    const double r31 = st * sp, r32 = -st * cp, r33 = ct;
    for (int i = 0; i < nfa; ++i) {
      const int a = S.frag_atoms[f0][i];
      const double x = r[3 * a] - com[0], y = r[3 * a + 1] - com[1], z = r[3 * a + 2] - com[2];
      r[3 * a] = (r11 * x + r12 * y + r13 * z) + com[0];
      r[3 * a + 1] = (r21 * x + r22 * y + r23 * z) + com[1];
      r[3 * a + 2] = (r31 * x + r32 * y + r33 * z) + com[2];
    }
  }
  for (int k = 0; k < 3 * sel; ++k) g.next_bits();
  const double ax = (0.5 - g.next()) * f.L64[0];
  const double ay = (0.5 - g.next()) * f.L64[1];
  const double az = (0.5 - g.next()) * f.L64[2];
  for (int i = 0; i < nfa; ++i) {
    const int a = S.frag_atoms[f0][i];
    r[3 * a] = r[3 * a] - com[0] + ax;
    r[3 * a + 1] = r[3 * a + 1] - com[1] + ay;
    r[3 * a + 2] = r[3 * a + 2] - com[2] + az;
  }
  for (int k = 0; k < 3 * (S.kappa_ins - sel - 1) + 1; ++k) g.next_bits();  // later trials, selection
  unsigned placed = 1u << f0;
  const int kd = S.kappa_dih;
  for (int oi = 1; oi < norder; ++oi) {
    const int fr = order[oi];
    const int nf = S.frag_natoms[fr];
    g.next_bits();  // the duplicated draw of fragment_growth.f90:1578,1584
    const int cf = index_of(draw_u32(g), S.nconfig[fr]);
    double cfg[3 * kMaxAtoms];
    const double* Lf = lib + S.lib_off[fr] + (size_t)cf * nf * 3;
    for (int j = 0; j < nf; ++j) {
      const int a = S.frag_atoms[fr][j];
      exist |= 1u << a;
      cfg[3 * a] = Lf[3 * j];
      cfg[3 * a + 1] = Lf[3 * j + 1];
      cfg[3 * a + 2] = Lf[3 * j + 2];
    }
    int fc = 0;
    for (int q = 0; q < S.frag_nconnect[fr]; ++q) {
      const int gg = S.frag_connect[fr][q];
      if ((placed >> gg) & 1u) {
        fc = gg;
        break;
      }
    }
    const int anc_i = S.frag_atoms[fr][0], anc_c = S.frag_atoms[fc][0];
    int ids[kMaxAtoms], nid = 0;
    for (int j = 0; j < nf; ++j) {
      const int a = S.frag_atoms[fr][j];
      if (a != anc_i && a != anc_c) ids[nid++] = a;
    }
    const int atom_ifrag = nid > 0 ? ids[0] : S.frag_atoms[fr][nf - 1];
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
      v1[d] = cfg[3 * anc_i + d] - cfg[3 * anc_c + d];
      v2[d] = cfg[3 * atom_ifrag + d] - cfg[3 * anc_c + d];
    }
    aligner_hanger_rs(v1, v2, al_i, hg_i);
    for (int d = 0; d < 3; ++d) {
      v1[d] = r[3 * anc_i + d] - r[3 * anc_c + d];
      v2[d] = r[3 * atom_fc + d] - r[3 * anc_c + d];
    }
    aligner_hanger_rs(v1, v2, al_c, hg_c);
    const double tx = cfg[3 * anc_c], ty = cfg[3 * anc_c + 1], tz = cfg[3 * anc_c + 2];
    // theta0 + trl (2 pi / kappa_dih), theta0 = 2 pi u, in units of pi
    const double t = 2.0 * g.next() + (double)trls[oi] * (2.0 / (double)kd);
    double sth, cth;
    sincospi(t, &sth, &cth);
    for (int j = 0; j < nid; ++j) {
      const int a = ids[j];
      const double x0 = cfg[3 * a] - tx, y0 = cfg[3 * a + 1] - ty, z0 = cfg[3 * a + 2] - tz;
      const double x = x0 * al_i[0] + y0 * al_i[1] + z0 * al_i[2];
      const double y = x0 * al_i[3] + y0 * al_i[4] + z0 * al_i[5];
      const double z = x0 * al_i[6] + y0 * al_i[7] + z0 * al_i[8];
      const double yr = cth * y + sth * z, zr = -sth * y + cth * z;
      r[3 * a] = (x * hg_c[0] + yr * hg_c[1] + zr * hg_c[2]) + r[3 * anc_c];
      r[3 * a + 1] = (x * hg_c[3] + yr * hg_c[4] + zr * hg_c[5]) + r[3 * anc_c + 1];
      r[3 * a + 2] = (x * hg_c[6] + yr * hg_c[7] + zr * hg_c[8]) + r[3 * anc_c + 2];
    }
    g.next_bits();  // trial selection
    placed |= 1u << fr;
  }
  if (S.nfrag > 1) {
    get_com(S, r, exist, com);
    for (int d = 0; d < 3; ++d) {
      const double sh = com[d] > f.hL64[d] ? -f.L64[d] : (com[d] < -f.hL64[d] ? f.L64[d] : 0.0);
      if (sh != 0.0)
        for (int a = 0; a < n; ++a) r[3 * a + d] += sh;
    }
  }
}

// Energy of atoms `ids` against the box: sum into e, true on overlap
template <bool COUNT, bool OPT>
__device__ __forceinline__ bool query_atoms_f(const BoxViewF& V, QueryAcc& A, const SpeciesF& S, const float* r,
                                              const int* ids, int n, float sx, float sy, float sz, bool cbmc,
                                              bool want_qq) {
  for (int i = 0; i < n; ++i) {
    const int a = ids[i];
    if (query_f<COUNT, OPT>(V, A, r[3 * a] + sx, r[3 * a + 1] + sy, r[3 * a + 2] + sz, S.type[a], S.q[a], cbmc, want_qq))
      return true;
  }
  return false;
}

// One Widom insertion: Widom_Insert (widom_insert.f90:250-447) with the CBMC
// growth of Build_Molecule (fragment_growth.f90:120-900) and
// Fragment_Placement (:1449-2132), in FP32
template <bool COUNT, bool OPT>
__device__ RecF run_insertion_f(const WidomSpecies& S, const SpeciesF& SF, const BoxViewF& V,
                                const float* __restrict__ lib, Lfsr rng, double* xyz_out, QueryAcc& cnt,
                                FixEntry& fe) {
  const BoxF& f = *V.f;
  const int n = S.natoms;
  RecF out{0, 0, 0, 0, 0, 0.0, 0, 0, false};
  int sel_first = 0;
  int trls[kMaxFrags];
  float r[3 * kMaxAtoms];
  unsigned exist = 0u;
  float ln_pbias = 0.0f;
  bool cbmc_overlap = false;

  // Step 1: first fragment and growth order (fragment_growth.f90:218-253, 1317-1446)
  const unsigned v0 = draw_u32(rng);
  int fstart = 0;
  while (fstart < S.nfrag && !((unsigned long long)v0 < SF.cumthr[fstart])) ++fstart;
  if (fstart >= S.nfrag) fstart = S.nfrag - 1;
  float ln_pseq = (float)S.ln_prob_ins[fstart];
  int order[kMaxFrags];
  int norder = 1;
  order[0] = fstart;
  unsigned live = 1u << fstart;
  if (S.nfrag > 1) {
    int hang[kMaxFrags];
    int nh = 0;
    for (int k = 0; k < S.frag_nconnect[fstart]; ++k) {
      const int g = S.frag_connect[fstart][k];
      if (!((live >> g) & 1u)) hang[nh++] = g;
    }
    while (nh > 0) {
      float tot = 0.0f;
      for (int k = 0; k < nh; ++k) tot += (float)(S.frag_natoms[hang[k]] - 2);
      const float uu = unit_of(draw_u32(rng));
      int k = 0;
      float cum = 0.0f;
      for (; k < nh; ++k) {
        cum += (float)(S.frag_natoms[hang[k]] - 2) / tot;
        if (uu < cum) break;
      }
      if (k >= nh) k = nh - 1;
      const int g = hang[k];
      if (nh > 1) ln_pseq += logf((float)(S.frag_natoms[g] - 2) / tot);
      order[norder++] = g;
      live |= 1u << g;
      for (int q = k; q + 1 < nh; ++q) hang[q] = hang[q + 1];
      --nh;
      for (int q = 0; q < S.frag_nconnect[g]; ++q) {
        const int h = S.frag_connect[g][q];
        if (!((live >> h) & 1u) && nh < kMaxFrags) hang[nh++] = h;
      }
    }
  }
  // Step 2: library conformation of the first fragment (:274-304)
  const int nfa = S.frag_natoms[fstart];
  int fa_ids[kMaxAtoms];
  {
    const int nconf = S.nconfig[fstart];
    const int conf = index_of(draw_u32(rng), nconf);
    const float* L0 = lib + S.lib_off[fstart] + (size_t)conf * nfa * 3;
    for (int i = 0; i < nfa; ++i) {
      const int a = S.frag_atoms[fstart][i];
      fa_ids[i] = a;
      r[3 * a] = L0[3 * i];
      r[3 * a + 1] = L0[3 * i + 1];
      r[3 * a + 2] = L0[3 * i + 2];
      exist |= 1u << a;
    }
  }
  // Step 3: random orientation about the COM (rotation_routines.f90:41-137);
  // the fragment is kept relative to its COM until a position is chosen
  float com[3];
  get_com_f(SF, r, exist, com);
  {
    const float theta = acosf(1.0f - 2.0f * unit_of(draw_u32(rng)));
    const float phi = (1.0f - 2.0f * unit_of(draw_u32(rng))) * (float)kPI;
    const float psi = (1.0f - 2.0f * unit_of(draw_u32(rng))) * (float)kPI;
    float st, ct, sp, cp, ss, cs;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    sincosf(psi, &ss, &cs);
    const float r11 = cs * cp - ct * sp * ss, r12 = cs * sp + ct * cp * ss, r13 = ss * st;
    const float r21 = -ss * cp - ct * sp * cs, r22 = -ss * sp + ct * cp * cs, r23 = cs * st;
    const float r31 = st * sp, r32 = -st * cp, r33 = ct;
    for (int i = 0; i < nfa; ++i) {
      const int a = fa_ids[i];
      const float x = r[3 * a] - com[0], y = r[3 * a + 1] - com[1], z = r[3 * a + 2] - com[2];
      r[3 * a] = r11 * x + r12 * y + r13 * z;
      r[3 * a + 1] = r21 * x + r22 * y + r23 * z;
      r[3 * a + 2] = r31 * x + r32 * y + r33 * z;
    }
  }
  // Step 4: kappa_ins trial positions of the first fragment (:383-620)
  const int ki = S.kappa_ins;
  const bool cbmc_qq = S.want_qq_cbmc != 0;
  float nrg[kMaxKappa];
  unsigned ovm = 0u;
  const Lfsr replay = rng;
  for (int it = 0; it < ki; ++it) {
    const float ax = centre_of(draw_u32(rng), f.L[0], f.Llo[0]);
    const float ay = centre_of(draw_u32(rng), f.L[1], f.Llo[1]);
    const float az = centre_of(draw_u32(rng), f.L[2], f.Llo[2]);
    QueryAcc A;
    bool ov = query_atoms_f<COUNT, OPT>(V, A, SF, r, fa_ids, nfa, ax, ay, az, true, cbmc_qq);
    cnt.visited += A.visited;
    cnt.in_cut += A.in_cut;
    const float e = A.e.s + A.e.c;
    ov = ov || e >= f.kmaxE;
    nrg[it] = e;
    if (ov) ovm |= 1u << it;
    else out.first_sum += e;
  }
  {
    float lnw = 0.0f;
    const int sel = select_trial_f(ki, nrg, ovm, f.beta, unit_of(draw_u32(rng)), &lnw);
    if (sel < 0) {
      cbmc_overlap = true;
    } else {
      ln_pbias = ln_pbias - f.beta * nrg[sel] - lnw;
      Lfsr rp = replay;
      float ax = 0, ay = 0, az = 0;
      for (int k = 0; k <= sel; ++k) {
        ax = centre_of(draw_u32(rp), f.L[0], f.Llo[0]);
        ay = centre_of(draw_u32(rp), f.L[1], f.Llo[1]);
        az = centre_of(draw_u32(rp), f.L[2], f.Llo[2]);
      }
      for (int i = 0; i < nfa; ++i) {
        const int a = fa_ids[i];
        r[3 * a] += ax;
        r[3 * a + 1] += ay;
        r[3 * a + 2] += az;
      }
      com[0] = ax;
      com[1] = ay;
      com[2] = az;
      out.selected = sel + 1;
      sel_first = sel;
    }
  }
  // Step 5: Fragment_Placement, kappa_dih dihedral trials per fragment
  if (!cbmc_overlap && norder > 1) {
    float e_prev = dihedral_f(SF, r, exist);
    unsigned placed = 1u << fstart;
    const int kd = S.kappa_dih;
    float dn[kMaxKappa], dd[kMaxKappa];
    for (int oi = 1; oi < norder && !cbmc_overlap; ++oi) {
      const int fr = order[oi];
      const int nf = S.frag_natoms[fr];
      const unsigned grown = exist;
      const int nconf = S.nconfig[fr];
      draw_u32(rng);  // the duplicated draw of fragment_growth.f90:1578,1584
      const int cf = index_of(draw_u32(rng), nconf);
      float cfg[3 * kMaxAtoms];
      const float* Lf = lib + S.lib_off[fr] + (size_t)cf * nf * 3;
      for (int j = 0; j < nf; ++j) {
        const int a = S.frag_atoms[fr][j];
        exist |= 1u << a;
        cfg[3 * a] = Lf[3 * j];
        cfg[3 * a + 1] = Lf[3 * j + 1];
        cfg[3 * a + 2] = Lf[3 * j + 2];
      }
      const unsigned combined = exist;
      int fc = -1;
      for (int q = 0; q < S.frag_nconnect[fr]; ++q) {
        const int g = S.frag_connect[fr][q];
        if ((placed >> g) & 1u) {
          fc = g;
          break;
        }
      }
      if (fc < 0) {  // no placed neighbour: the fragment graph is not connected
        cbmc_overlap = true;
        break;
      }
      const int anc_i = S.frag_atoms[fr][0], anc_c = S.frag_atoms[fc][0];
      int ids[kMaxAtoms], nid = 0;
      for (int j = 0; j < nf; ++j) {
        const int a = S.frag_atoms[fr][j];
        if (a != anc_i && a != anc_c) ids[nid++] = a;
      }
      int newids[kMaxAtoms], nnew = 0;
      for (int a = 0; a < n; ++a)
        if (((combined & ~grown) >> a) & 1u) newids[nnew++] = a;
      unsigned idmask = 0u;
      for (int j = 0; j < nid; ++j) idmask |= 1u << ids[j];
      const int atom_ifrag = nid > 0 ? ids[0] : S.frag_atoms[fr][nf - 1];
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
        v1[d] = cfg[3 * anc_i + d] - cfg[3 * anc_c + d];
        v2[d] = cfg[3 * atom_ifrag + d] - cfg[3 * anc_c + d];
      }
      aligner_hanger_f(v1, v2, al_i, hg_i);
      for (int d = 0; d < 3; ++d) {
        v1[d] = r[3 * anc_i + d] - r[3 * anc_c + d];
        v2[d] = r[3 * atom_fc + d] - r[3 * anc_c + d];
      }
      aligner_hanger_f(v1, v2, al_c, hg_c);
      const float tx = cfg[3 * anc_c], ty = cfg[3 * anc_c + 1], tz = cfg[3 * anc_c + 2];
      for (int j = 0; j < nid; ++j) {
        const int a = ids[j];
        const float x = cfg[3 * a] - tx, y = cfg[3 * a + 1] - ty, z = cfg[3 * a + 2] - tz;
        cfg[3 * a] = x * al_i[0] + y * al_i[1] + z * al_i[2];
        cfg[3 * a + 1] = x * al_i[3] + y * al_i[4] + z * al_i[5];
        cfg[3 * a + 2] = x * al_i[6] + y * al_i[7] + z * al_i[8];
      }
      const float theta0 = (float)kTWOPI * unit_of(draw_u32(rng));
      const float dtheta = (float)kTWOPI / (float)kd;
      unsigned dov = 0u;
      for (int ii = 0; ii < kd; ++ii) {
        float sth, cth;
        sincosf(theta0 + (float)ii * dtheta, &sth, &cth);
        for (int j = 0; j < nid; ++j) {
          const int a = ids[j];
          const float x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
          const float yr = cth * y + sth * z, zr = -sth * y + cth * z;
          r[3 * a] = (x * hg_c[0] + yr * hg_c[1] + zr * hg_c[2]) + r[3 * anc_c];
          r[3 * a + 1] = (x * hg_c[3] + yr * hg_c[4] + zr * hg_c[5]) + r[3 * anc_c + 1];
          r[3 * a + 2] = (x * hg_c[6] + yr * hg_c[7] + zr * hg_c[8]) + r[3 * anc_c + 2];
        }
        dn[ii] = 0.0f;
        dd[ii] = 0.0f;
        exist &= ~idmask;
        float niv = 0.0f, niq = 0.0f, noq = 0.0f;
        bool ov = false;
        for (int j = 0; j < nid && !ov; ++j) {
          exist |= 1u << ids[j];
          float eiv, eiq, eoq;
          ov = atom_intra_f(SF, f, V.ljp, ids[j], r, exist, eiv, eiq, eoq);
          niv += eiv;
          niq += eiq;
          noq += eoq;
        }
        if (ov) {
          exist = combined;
          dov |= 1u << ii;
          continue;
        }
        QueryAcc A;
        ov = query_atoms_f<COUNT, OPT>(V, A, SF, r, newids, nnew, 0.0f, 0.0f, 0.0f, true, cbmc_qq);
        cnt.visited += A.visited;
        cnt.in_cut += A.in_cut;
        exist = combined;
        if (!ov) {
          const float ed = dihedral_f(SF, r, exist);
          dd[ii] = ed;
          dn[ii] = ed + niv + niq + (A.e.s + A.e.c) + noq - e_prev;
          ov = dn[ii] >= f.kmaxE;
        }
        if (ov) dov |= 1u << ii;
      }
      float lnw = 0.0f;
      const int trl = select_trial_f(kd, dn, dov, f.beta, unit_of(draw_u32(rng)), &lnw);
      if (trl < 0) {
        cbmc_overlap = true;
        break;
      }
      ln_pbias = ln_pbias - f.beta * dn[trl] - lnw;
      float sth, cth;
      sincosf(theta0 + (float)trl * dtheta, &sth, &cth);
      for (int j = 0; j < nid; ++j) {
        const int a = ids[j];
        const float x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
        const float yr = cth * y + sth * z, zr = -sth * y + cth * z;
        r[3 * a] = (x * hg_c[0] + yr * hg_c[1] + zr * hg_c[2]) + r[3 * anc_c];
        r[3 * a + 1] = (x * hg_c[3] + yr * hg_c[4] + zr * hg_c[5]) + r[3 * anc_c + 1];
        r[3 * a + 2] = (x * hg_c[6] + yr * hg_c[7] + zr * hg_c[8]) + r[3 * anc_c + 2];
      }
      e_prev = dd[trl];
      trls[oi] = trl;
      placed |= 1u << fr;
    }
    if (!cbmc_overlap) get_com_f(SF, r, exist, com);
  }
  // widom_insert.f90:350-447
  ln_pbias = ln_pbias + ln_pseq + (float)S.ln_kappa_ins + (float)S.ln_kappa_dih_term;
  out.ln_pbias = ln_pbias;
  if (cbmc_overlap) {
    out.status = 1;
    return out;
  }
  if (S.nfrag > 1) {  // Fold_Molecule, orthorhombic branch
    for (int d = 0; d < 3; ++d) {
      const float sh = com[d] > f.hL[d] ? -f.L[d] : (com[d] < -f.hL[d] ? f.L[d] : 0.0f);
      if (sh != 0.0f)
        for (int a = 0; a < n; ++a) r[3 * a + d] += sh;
    }
  }
  QueryAcc A;
  A.band = fe.band;
  bool ov = false;
  for (int a = 0; a < n && !ov; ++a) {
    A.atom = a;
    ov = query_f<COUNT, false, kQDetect>(V, A, r[3 * a], r[3 * a + 1], r[3 * a + 2], SF.type[a], SF.q[a], false,
                                         true);
  }
  cnt.visited += A.visited;
  cnt.in_cut += A.in_cut;
  if (!ov && A.nband > 0) {  // pairs within FP32 rounding of a cutoff: k_widom_fix decides them in FP64
    out.fix = true;
    fe.nband = A.nband;
    fe.sel = (unsigned char)sel_first;
    fe.norder = (unsigned char)norder;
    for (int k = 0; k < norder; ++k) {
      fe.order[k] = (unsigned char)order[k];
      fe.trl[k] = (unsigned char)(k > 0 ? trls[k] : 0);
    }
  }
  if (ov) {
    out.status = 2;
    return out;
  }
  const IntraF io = molecule_intra_f(SF, f, V.ljp, r);
  if (io.overlap) {
    out.status = 3;
    return out;
  }
  out.e_inter = (A.e.value() + (double)io.pqq);
  out.e_abs = A.eabs;
  out.dE_intra = (io.ivdw + io.iqq) + io.bond + io.angle + io.dih + io.imp;
  out.dE_frag = io.angle;
  out.status = 0;
  if (xyz_out)
    for (int i = 0; i < 3 * n; ++i) xyz_out[i] = (double)r[i];
  return out;
}

// 16 warps per staged box and two CTAs per SM (64 registers): the kernel is
// latency-bound, and warps per scheduler matter more than the few spills.  The
// launch autotuner may choose 256-thread CTAs instead (four per SM by
// registers, fewer by shared memory for large boxes; more CTAs per box).
constexpr int kF32Threads = 512;
constexpr int kF32Waves = 8;  // CTAs per resident slot: many short waves even out uneven boxes

// FP32 constants of box b (thread 0), the FP64 edges and squared cutoffs
// and the FP32 error bands of the full-cutoff pass
__device__ inline void widom_boxf(BoxF& sf, const BoxDev& b, double band_scale) {
  double lmax = 0.0;
  for (int d = 0; d < 3; ++d) {
    sf.L[d] = (float)b.L[d];
    sf.Llo[d] = (float)(b.L[d] - (double)sf.L[d]);
    sf.hL[d] = (float)b.hL[d];
    sf.cinv[d] = (float)b.cell_inv[d];
    sf.ch[d] = (float)(b.L[d] / (double)b.nc[d]);
    sf.nc[d] = b.nc[d];
    sf.L64[d] = b.L[d];
    sf.hL64[d] = b.hL[d];
    lmax = fmax(lmax, b.L[d]);
  }
  sf.rcb2 = (float)b.rcut_cbmcsq;
  sf.rv2 = (float)b.rcut_vdwsq;
  sf.rq2 = (float)b.rcut_coulsq;
  sf.low2 = (float)b.rcut_lowsq;
  sf.rc_cbmc = (float)sqrt(b.rcut_cbmcsq);
  sf.rc_full = (float)sqrt(fmax(b.rcut_vdwsq, b.rcut_coulsq));
  sf.beta = (float)b.beta;
  sf.kmaxE = (float)(kMAX_KBT / b.beta);
  sf.alpha = (float)b.alpha;
  sf.charge_on = b.charge_style == CASS_CHARGE_COUL;
  // |r2_32 - r2_64| <= 2 sqrt(3) r delta + the rounding of r^2, where delta
  // bounds the FP32 error of a coordinate difference: the FP32 growth of the
  // test molecule (its centre of mass rounded once, rotations of a few A), the
  // rounding of the stored box atom, of a row's image shift and of the
  // difference -- about 12 half-ulps of the largest coordinate, up to
  // L / 2 + rcut; delta = 5e-7 (L + 20 A) exceeds it by a factor of 2 or more
  const double delta = 5.0e-7 * (lmax + 20.0) * band_scale;
  auto band = [&](double rc2) { return (float)(3.5 * sqrt(rc2) * delta + 1.0e-6 * rc2); };
  sf.rv2d = b.rcut_vdwsq;
  sf.rq2d = b.rcut_coulsq;
  sf.low2d = b.rcut_lowsq;
  sf.band_v = band(b.rcut_vdwsq);
  sf.band_q = band(b.rcut_coulsq);
  sf.band_low = band(b.rcut_lowsq);
}

__device__ inline void widom_ljp(float2* s_ljp, const PairTable& T) {
  for (int i = threadIdx.x; i < kMaxTypes * kMaxTypes; i += blockDim.x) {
    const int a = i / kMaxTypes, c = i % kMaxTypes;
    const bool ok = a < T.ntypes && c < T.ntypes;
    s_ljp[i] = ok ? make_float2(T.epsf[a * T.ntypes + c], T.sig2f[a * T.ntypes + c]) : make_float2(0.f, 0.f);
  }
}

template <bool SMEM, bool COUNT, bool OPT, int NT = kF32Threads>
__global__ void __launch_bounds__(NT, 1024 / NT) k_widom_f32(WidomSpecies S, SpeciesF SF, PairTable T, const BoxDev* boxes,
                                                   const int* box_ids, const float4* c32, const float* cq32,
                                                   const int* cstart, const float* __restrict__ libf, long long n_ins,
                                                   uint64_t seed, WRec* rec, signed char* status, double* xyz,
                                                   int want_xyz, CassWidomTrace* trace, FixEntry* fix_q,
                                                   int* fix_n, double band_scale,
                                                   unsigned long long* pair_counts) {
  extern __shared__ __align__(32) unsigned char smem[];
  __shared__ BoxF sf;
  __shared__ float2 s_ljp[kMaxTypes * kMaxTypes];
  __shared__ int s_atom_off, s_cell_off, s_natoms;
  __shared__ double s_ec;
  const int k = blockIdx.y;
  if (threadIdx.x == 0) {
    const BoxDev& b = boxes[k];
    widom_boxf(sf, b, band_scale);
    s_atom_off = b.atom_off;
    s_cell_off = b.cell_off;
    s_natoms = b.natoms;
    s_ec = b.e_inter_constant;
  }
  if (OPT) boxf_options(sf, boxes[k], T.ntypes);
  widom_ljp(s_ljp, T);
  __syncthreads();
  const int ncell = sf.nc[0] * sf.nc[1] * sf.nc[2];
  BoxViewF V;
  V.f = &sf;
  V.q32 = cq32 + s_atom_off;
  V.p64 = nullptr;
  V.ljp = s_ljp;
  if (SMEM) {
    int* cs = reinterpret_cast<int*>(smem);
    for (int c = threadIdx.x; c <= ncell; c += blockDim.x) cs[c] = cstart[s_cell_off + k + c];
    const size_t off = ((size_t)(ncell + 1) * sizeof(int) + 31) & ~(size_t)31;
    float4* s32 = reinterpret_cast<float4*>(smem + off);
    for (int j = threadIdx.x; j < s_natoms; j += blockDim.x) s32[j] = c32[s_atom_off + j];
    V.p32 = s32;
    V.cstart = cs;
    __syncthreads();
  } else {
    V.p32 = c32 + s_atom_off;
    V.cstart = cstart + s_cell_off + k;
  }
  const long long stride = (long long)gridDim.x * blockDim.x;
  QueryAcc cnt;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_ins; i += stride) {
    const size_t g = (size_t)k * n_ins + i;
    const Lfsr rng = seed_stream(seed, box_ids[k], i);
    FixEntry fe;
    const RecF o = run_insertion_f<COUNT, OPT>(S, SF, V, libf, rng, want_xyz ? xyz + g * 3 * S.natoms : nullptr,
                                               cnt, fe);
    const double e_int = o.e_inter;
    rec[g] = make_double4_32a((double)o.dE_intra, e_int + s_ec, (double)o.dE_frag, (double)o.ln_pbias);
    status[g] = (signed char)o.status;
    if (trace) {
      CassWidomTrace& t = trace[g];
      t.ln_pbias = (double)o.ln_pbias;
      t.e_first_trial_sum = (double)o.first_sum;
      t.selected_trial = o.selected;
      t.e_inter = o.status == 0 ? e_int : 0.0;
      t.e_inter_abs = o.status == 0 ? (double)o.e_abs : 0.0;
      t.overlap = o.status;
    }
    if (o.fix) {
      fe.ins = (int)i;
      const int slot = atomicAdd(&fix_n[k], 1);  // < n_ins: one entry per insertion at most
      fix_q[(size_t)k * n_ins + slot] = fe;
    }
  }
  if (pair_counts) {
    atomicAdd(&pair_counts[0], cnt.visited);
    atomicAdd(&pair_counts[1], cnt.in_cut);
  }
}

// The insertions whose full-cutoff pass met pairs within a band of FP32
// rounding about a cutoff, one thread each: the selected molecule again in
// FP64 (replay_molecule_f64, the same choices), each band pair's r^2 in FP64
// from it (the FP64 path's r^2 to about 1e-15 A^2), and the FP64 decision:
// an overlap makes the insertion an overlap (status 2); a vdW or Coulomb term
// on the other side of its cutoff than in FP32 is added or removed (its FP32
// pair energy).  An insertion with more than kMaxBand band pairs has its whole
// full-cutoff pass redone from the FP64 coordinates (kQExact).  Record, status
// and trace are corrected in place; the box stays in global memory.
__global__ void __launch_bounds__(128) k_widom_fix(WidomSpecies S, SpeciesF SF, PairTable T, const BoxDev* boxes,
                                                   const int* box_ids, const float4* c32, const float* cq32,
                                                   const double4_32a* c64, const int* cstart,
                                                   const double* __restrict__ lib64, long long n_ins, uint64_t seed,
                                                   const FixEntry* fix_q, const int* fix_n, WRec* rec,
                                                   signed char* status, double* xyz, int want_xyz,
                                                   CassWidomTrace* trace, double band_scale) {
  __shared__ BoxF sf;
  __shared__ float2 s_ljp[kMaxTypes * kMaxTypes];
  __shared__ int s_atom_off, s_cell_off;
  __shared__ double s_ec;
  const int k = blockIdx.y;
  const int nq = fix_n[k];
  if ((long long)blockIdx.x * blockDim.x >= nq) return;  // nothing queued for this block
  if (threadIdx.x == 0) {
    const BoxDev& b = boxes[k];
    widom_boxf(sf, b, band_scale);
    s_atom_off = b.atom_off;
    s_cell_off = b.cell_off;
    s_ec = b.e_inter_constant;
  }
  widom_ljp(s_ljp, T);
  __syncthreads();
  BoxViewF V;
  V.f = &sf;
  V.p32 = c32 + s_atom_off;
  V.p64 = c64 + s_atom_off;
  V.q32 = cq32 + s_atom_off;
  V.cstart = cstart + s_cell_off + k;
  V.ljp = s_ljp;
  const int n = S.natoms;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nq; e += gridDim.x * blockDim.x) {
    const FixEntry& fe = fix_q[(size_t)k * n_ins + e];
    const size_t g = (size_t)k * n_ins + fe.ins;
    int order[kMaxFrags], trls[kMaxFrags];
    const int norder = fe.norder;
    for (int q = 0; q < norder; ++q) {
      order[q] = fe.order[q];
      trls[q] = fe.trl[q];
    }
    double r64[3 * kMaxAtoms];
    replay_molecule_f64(S, sf, lib64, seed_stream(seed, box_ids[k], fe.ins), order, norder, fe.sel, trls, r64);
    const double lnp = rec[g].w;
    if (fe.nband > kMaxBand) {  // redo the pass from the FP64 coordinates
      float r[3 * kMaxAtoms];
      for (int i = 0; i < 3 * n; ++i) r[i] = (float)r64[i];
      QueryAcc A;
      bool ov = false;
      for (int a = 0; a < n && !ov; ++a)
        ov = query_f<false, false, kQExact>(V, A, r[3 * a], r[3 * a + 1], r[3 * a + 2], SF.type[a], SF.q[a], false,
                                            true, r64 + 3 * a);
      int st = 2;
      double e_int = 0.0, e_abs = 0.0, dE_intra = 0.0, dE_frag = 0.0;
      if (!ov) {
        const IntraF io = molecule_intra_f(SF, sf, V.ljp, r);
        st = io.overlap ? 3 : 0;
        if (st == 0) {
          e_int = A.e.value() + (double)io.pqq;
          e_abs = (double)A.eabs;
          dE_intra = (double)((io.ivdw + io.iqq) + io.bond + io.angle + io.dih + io.imp);
          dE_frag = (double)io.angle;
        }
      }
      rec[g] = make_double4_32a(dE_intra, e_int + s_ec, dE_frag, lnp);
      status[g] = (signed char)st;
      if (trace) {
        trace[g].e_inter = e_int;
        trace[g].e_inter_abs = e_abs;
        trace[g].overlap = st;
      }
      if (want_xyz && st == 0)
        for (int i = 0; i < 3 * n; ++i) xyz[g * 3 * n + i] = r64[i];
      continue;
    }
    bool ov = false;
    double de = 0.0, dab = 0.0;
    for (int q = 0; q < fe.nband; ++q) {
      const BandPair bp = fe.band[q];
      const int a = bp.atom;
      const double d2 = exact_r2(sf, V.p64, bp.j, r64 + 3 * a);
      if (bp.kind == 1) {
        ov = ov || d2 < sf.low2d;
        continue;
      }
      const float4 at = V.p32[bp.j];
      const int ta = SF.type[a], tj = __float_as_int(at.w);
      if (ta >= 0 && tj >= 0 && (bp.r2 <= sf.rv2) != (d2 <= sf.rv2d)) {
        const float2 es = s_ljp[ta * kMaxTypes + tj];
        const double ev = (double)lj_pair_f(es.x, es.y, bp.r2);
        de += d2 <= sf.rv2d ? ev : -ev;
        dab += d2 <= sf.rv2d ? fabs(ev) : -fabs(ev);
      }
      const float qa = SF.q[a];
      if (sf.charge_on && qa != 0.0f && (bp.r2 <= sf.rq2) != (d2 <= sf.rq2d)) {
        const double eq = (double)qq_ewald_inter_f(sf.alpha, qa * V.q32[bp.j], bp.r2);
        de += d2 <= sf.rq2d ? eq : -eq;
        dab += d2 <= sf.rq2d ? fabs(eq) : -fabs(eq);
      }
    }
    if (ov) {
      rec[g] = make_double4_32a(0.0, s_ec, 0.0, lnp);
      status[g] = 2;
      if (trace) {
        trace[g].e_inter = 0.0;
        trace[g].e_inter_abs = 0.0;
        trace[g].overlap = 2;
      }
    } else if (status[g] == 0 && (de != 0.0 || dab != 0.0)) {
      rec[g].y += de;
      if (trace) {
        trace[g].e_inter += de;
        trace[g].e_inter_abs += dab;
      }
    }
  }
}

// FP64 kernel: one insertion per thread (the reference's arithmetic)
template <bool SMEM>
__global__ void __launch_bounds__(128) k_widom(WidomSpecies S, PairTable T, SpeciesPools P, const BoxDev* boxes,
                                               const int* box_ids, const double4_32a* c64, const int* ctype,
                                               const int* corig, const int* cstart,
                                               const double* __restrict__ lib, long long n_ins,
                                               uint64_t seed, WRec* rec, signed char* status, double* xyz,
                                               int want_xyz, CassWidomTrace* trace, unsigned long long* pair_counts) {
  extern __shared__ __align__(32) unsigned char smem[];
  __shared__ BoxDev sb;
  const int k = blockIdx.y;
  if (threadIdx.x == 0) sb = boxes[k];
  __syncthreads();
  const int na = sb.natoms;
  const int ncell = sb.nc[0] * sb.nc[1] * sb.nc[2];
  BoxView V;
  V.b = &sb;
  V.rc_cbmc = sqrt(sb.rcut_cbmcsq);
  double rfull = sqrt(fmax(sb.rcut_vdwsq, sb.rcut_coulsq));
  if (sb.vdw_sum_style == CASS_VDW_SUM_MINIMUM || sb.vdw_sum_style == CASS_VDW_SUM_CHARMM ||
      (sb.charge_style == CASS_CHARGE_COUL && sb.charge_sum_style == CASS_QQ_MINIMUM))
    rfull = 1e30;
  if (sb.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) rfull = fmax(rfull, sqrt(sb.roff_switch_sq));
  V.rc_full = rfull;
  V.corig = corig + sb.atom_off;
  if (SMEM) {
    int* cs = reinterpret_cast<int*>(smem);
    for (int c = threadIdx.x; c <= ncell; c += blockDim.x) cs[c] = cstart[sb.cell_off + k + c];
    size_t off = ((size_t)(ncell + 1) * sizeof(int) + 31) & ~(size_t)31;
    double4_32a* s64 = reinterpret_cast<double4_32a*>(smem + off);
    int* st = reinterpret_cast<int*>(smem + off + (size_t)na * sizeof(double4_32a));
    for (int j = threadIdx.x; j < na; j += blockDim.x) {
      s64[j] = c64[sb.atom_off + j];
      st[j] = ctype[sb.atom_off + j];
    }
    V.p64 = s64;
    V.ptype = st;
    V.cstart = cs;
    __syncthreads();
  } else {
    V.cstart = cstart + sb.cell_off + k;
    V.p64 = c64 + sb.atom_off;
    V.ptype = ctype + sb.atom_off;
  }
  const long long stride = (long long)gridDim.x * blockDim.x;
  PairCount pc;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_ins; i += stride) {
    size_t g = (size_t)k * n_ins + i;
    Lfsr rng = seed_stream(seed, box_ids[k], i);
    WRec rr;
    int st = 0;
    run_insertion(S, P, T, V, lib, rng, rr, st, want_xyz ? xyz + g * 3 * S.natoms : nullptr,
                  trace ? trace + g : nullptr, pc);
    rec[g] = rr;
    status[g] = (signed char)st;
    if (trace) trace[g].overlap = st;
  }
  if (pair_counts) {
    atomicAdd(&pair_counts[0], pc.visited);
    atomicAdd(&pair_counts[1], pc.in_cut);
  }
}

// E_recip of each surviving insertion (absolute, as the reference computes it)
__global__ void __launch_bounds__(256) k_widom_recip(const BoxDev* boxes, const double4_32a* kvec_all,
                                                     const double* cos_all, const double* sin_all,
                                                     const int* kvec_box_off, const int* ewald_box, long long n_ins,
                                                     int na, const double* q, const signed char* status,
                                                     const double* xyz, WRec* rec, CassWidomTrace* trace) {
  __shared__ double sh[32];
  long long gi = blockIdx.x;
  int k = (int)(gi / n_ins);
  if (!ewald_box[k] || status[gi] != 0) return;
  const double4_32a* kv = kvec_all + kvec_box_off[k];
  const double* cs = cos_all + kvec_box_off[k];
  const double* sn = sin_all + kvec_box_off[k];
  int nv = boxes[k].nvecs;
  const double* r = xyz + (size_t)gi * 3 * na;
  double e = 0.0;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    double4_32a h = kv[i];
    double dc = 0.0, ds = 0.0;
    for (int a = 0; a < na; ++a) {
      double hdotr = h.x * r[3 * a] + h.y * r[3 * a + 1] + h.z * r[3 * a + 2];
      double s, c;
      sincos(hdotr, &s, &c);
      dc += q[a] * c;
      ds += q[a] * s;
    }
    double c = cs[i] + dc, s = sn[i] + ds;
    e = e + h.w * (c * c + s * s);
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    double er = t * kCHARGE_FACTOR;
    rec[gi].y = rec[gi].y + er;
    if (trace) trace[gi].e_inter += er;
  }
}

// widom_var and per-box sums; block per box, fixed-order reduction
__global__ void __launch_bounds__(256) k_widom_finalize(const BoxDev* boxes, long long n_ins, const WRec* rec,
                                                        const signed char* status, double* box_sum,
                                                        long long* box_ov, CassWidomTrace* trace) {
  __shared__ double shs[32];
  __shared__ long long sho[32];
  int k = blockIdx.x;
  double beta = boxes[k].beta, ec = boxes[k].e_inter_constant;
  double s = 0.0;
  long long nov = 0;
  for (long long i = threadIdx.x; i < n_ins; i += blockDim.x) {
    size_t g = (size_t)k * n_ins + i;
    double v = 0.0;
    if (status[g] == 0) {
      WRec r = rec[g];
      double dE = r.x + r.y;
      v = exp(-beta * (dE - r.z) - r.w);
      s += v;
    } else {
      ++nov;
    }
    if (trace) {
      trace[g].widom_var = v;
      if (status[g] == 0) trace[g].e_inter = rec[g].y - ec;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    nov += __shfl_down_sync(0xffffffffu, nov, o);
  }
  if ((threadIdx.x & 31) == 0) {
    shs[threadIdx.x >> 5] = s;
    sho[threadIdx.x >> 5] = nov;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    long long o = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      t += shs[w];
      o += sho[w];
    }
    box_sum[k] = t;
    box_ov[k] = o;
  }
}

}  // namespace cassgpu

using namespace cassgpu;

namespace {

double lrc_host(cass_ctx* c, const BoxH& B, const std::vector<double>& nb) {
  int nt = c->ntypes;
  double e = 0.0;
  if (B.desc.vdw_style == CASS_VDW_LJ) {
    for (int ia = 0; ia < nt; ++ia) {
      double eij = 0.0;
      for (int ja = 0; ja < nt; ++ja) {
        double eps = c->pt.eps[pidx(ia, ja, nt)], s2 = c->pt.sig2[pidx(ia, ja, nt)];
        double s6 = s2 * s2 * s2, s12 = s6 * s6;
        eij = eij + nb[ja] * 4.0 * eps * (s12 / (9.0 * B.rcut9) - (s6 / (3.0 * B.rcut3)));
      }
      e = e + nb[ia] * eij;
    }
    e = 2.0 * kPI * e / B.dev.volume;
  } else if (B.desc.vdw_style == CASS_VDW_MIE) {
    for (int ia = 0; ia < nt; ++ia) {
      double eij = 0.0;
      for (int ja = 0; ja < nt; ++ja) {
        int k = pidx(ia, ja, nt);
        double sor = std::sqrt(c->pt.sig2[k]) / B.desc.rcut_vdw;
        eij = eij + nb[ja] * c->pt.mie_c[k] * c->pt.eps[k] * std::pow(B.desc.rcut_vdw, 3.0) *
                        ((std::pow(sor, c->pt.mie_n[k]) / (3.0 - c->pt.mie_n[k])) +
                         (std::pow(sor, c->pt.mie_m[k]) / (c->pt.mie_m[k] - 3.0)));
      }
      e = e + nb[ia] * eij;
    }
    e = -2.0 * kPI * e / B.dev.volume;
  }
  return e;
}

// FP32 tables of the test species for k_widom_mixed; false when the species
// does not fit them (the FP64-geometry kernel runs instead)
}  // namespace

namespace cassgpu {
// FP32 copy of species s for the mixed kernels; false when a table exceeds the
// fixed capacities (the caller then runs the FP64 kernel)
bool species_f(const SpeciesH& s, SpeciesF& F) {
  memset(&F, 0, sizeof(F));
  const int n = s.natoms;
  const int nb = (int)s.bond_kind.size(), na = (int)s.angle_kind.size();
  const int nd = (int)(s.dih_atoms.size() / 4), ni = (int)(s.imp_atoms.size() / 4);
  if (n > kMaxAtoms || nb > kMaxBonded || na > kMaxBonded || nd > kMaxBonded || ni > kMaxBonded) return false;
  F.natoms = n;
  F.nbonds = nb;
  F.nangles = na;
  F.ndih = nd;
  F.nimp = ni;
  for (int a = 0; a < n; ++a) {
    F.q[a] = (float)s.q[a];
    F.mass[a] = (float)s.mass[a];
    F.type[a] = s.type[a];
    for (int b = 0; b < n; ++b) {
      F.vs[a * n + b] = (float)s.vscale[a * n + b];
      F.qs[a * n + b] = (float)s.qscale[a * n + b];
      if (s.bonded[a * n + b]) F.bonded[a] |= 1u << b;
    }
  }
  for (int k = 0; k < nb; ++k) {
    F.bond_atoms[k][0] = (signed char)s.bond_atoms[2 * k];
    F.bond_atoms[k][1] = (signed char)s.bond_atoms[2 * k + 1];
    F.bond_harm[k] = s.bond_kind[k] == CASS_BONDED_HARMONIC;
    F.bond_k[k] = (float)s.bond_param[2 * k];
    F.bond_l0[k] = (float)s.bond_param[2 * k + 1];
  }
  for (int k = 0; k < na; ++k) {
    for (int j = 0; j < 3; ++j) F.angle_atoms[k][j] = (signed char)s.angle_atoms[3 * k + j];
    F.angle_harm[k] = s.angle_kind[k] == CASS_BONDED_HARMONIC;
    F.angle_k[k] = (float)s.angle_param[2 * k];
    F.angle_t0[k] = (float)s.angle_param[2 * k + 1];
  }
  for (int k = 0; k < nd; ++k) {
    for (int j = 0; j < 4; ++j) F.dih_atoms[k][j] = (signed char)s.dih_atoms[4 * k + j];
    for (int j = 0; j < 6; ++j) F.rb[k][j] = (float)s.dih_rb[6 * k + j];
  }
  for (int k = 0; k < ni; ++k) {
    for (int j = 0; j < 4; ++j) F.imp_atoms[k][j] = (signed char)s.imp_atoms[4 * k + j];
    F.imp_k[k] = (float)s.imp_param[2 * k];
    F.imp_p0[k] = (float)s.imp_param[2 * k + 1];
  }
  for (int f = 0; f < s.nfrag; ++f) {
    F.cum_prob_ins[f] = (float)s.cum_prob_ins[f];
    const double c = f == s.nfrag - 1 ? 1.0 : std::min(1.0, s.cum_prob_ins[f]);
    F.cumthr[f] = (unsigned long long)std::floor(c * 4294967296.0);
  }
  return true;
}


// Growth tables of species s (0-based is0) for kernels that build molecules
void fill_growth_species(const SpeciesH& s, int is0, int kappa_ins, int kappa_dih, WidomSpecies& S) {
  memset(&S, 0, sizeof(S));
  S.natoms = s.natoms;
  S.nfrag = s.nfrag;
  S.is0 = is0;
  S.kappa_ins = kappa_ins;
  S.kappa_dih = s.nfrag > 1 ? kappa_dih : 0;
  S.want_qq_cbmc = s.l_coul_cbmc ? 1 : 0;
  S.ln_kappa_ins = std::log((double)kappa_ins);
  S.ln_kappa_dih_term = kappa_dih != 0 ? (double)(s.nfrag - 1) * std::log((double)kappa_dih) : 0.0;
  for (int a = 0; a < s.natoms; ++a) {
    S.mass[a] = s.mass[a];
    S.q[a] = s.q[a];
    S.type[a] = s.type[a];
  }
  for (int f = 0; f < s.nfrag; ++f) {
    S.frag_natoms[f] = (int)s.frag_atoms[f].size();
    for (size_t j = 0; j < s.frag_atoms[f].size(); ++j) S.frag_atoms[f][j] = (signed char)s.frag_atoms[f][j];
    S.frag_nconnect[f] = (int)s.frag_connect[f].size();
    for (size_t j = 0; j < s.frag_connect[f].size(); ++j) S.frag_connect[f][j] = (signed char)s.frag_connect[f][j];
    S.nconfig[f] = s.frag_nconfig[f];
    S.lib_off[f] = s.lib_off[f];
    S.prob_ins[f] = s.prob_ins[f];
    S.cum_prob_ins[f] = s.cum_prob_ins[f];
    S.ln_prob_ins[f] = std::log(s.prob_ins[f]);
  }
}

int ensure_pools(cass_ctx* c);
int pack_box_ext(cass_ctx* c, int ibox);
const std::vector<int>& members_ext(cass_ctx* c, int ibox);
}  // namespace cassgpu

static int widom_insert_impl(cass_ctx* c, int32_t is1, int32_t nboxes, const int32_t* iboxes, int64_t n_ins,
                                 int32_t kappa_ins, int32_t kappa_dih, uint64_t seed, CassWidomResult* out,
                                 CassWidomTrace* trace) {
  if (!c || is1 < 1 || is1 > c->nspecies || nboxes < 1 || !iboxes || !out || n_ins < 0)
    return set_error(CASS_EINVAL, "bad widom arguments");
  if (kappa_ins < 1 || kappa_ins > kMaxKappa) return set_error(CASS_EINVAL, "kappa_ins must be in 1..32");
  const SpeciesH& s = c->sp[is1 - 1];
  if (!s.defined) return set_error(CASS_ESTATE, "species not defined");
  if (s.nfrag < 1) return set_error(CASS_EINVAL, "species has no CBMC fragments");
  if (s.nfrag > 1 && (kappa_dih < 1 || kappa_dih > kMaxKappa)) return set_error(CASS_EINVAL, "kappa_dih must be in 1..32");
  if (s.natoms > kMaxAtoms) return set_error(CASS_ECAPACITY, "test species has more than 16 atoms");
  if (s.nfrag > kMaxFrags) return set_error(CASS_ECAPACITY, "test species has more than 8 fragments");
  for (int f = 0; f < s.nfrag; ++f) {
    if (s.frag_nconfig[f] < 1) return set_error(CASS_EINVAL, "fragment library is empty");
    if (s.frag_connect[f].size() > (size_t)kMaxFrags) return set_error(CASS_ECAPACITY, "too many fragment connections");
  }
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  for (int k = 0; k < nboxes; ++k) {
    int ib = iboxes[k] - 1;
    if (ib < 0 || ib >= c->nboxes) return set_error(CASS_EINVAL, "box index out of range");
    if (!c->box[ib].energy_valid && !c->box[ib].frame_ready)
      return set_error(CASS_ESTATE, "system energy of box not computed");
  }
  int rc;
  CASS_CUDA(cudaSetDevice(c->device));
  if ((rc = ensure_pools(c))) return rc;
  if ((rc = ensure_cbmc(c))) return rc;
  const int is0 = is1 - 1;

  WidomSpecies S;
  fill_growth_species(s, is0, kappa_ins, kappa_dih, S);

  // per-box constants and cell grids
  std::vector<BoxDev> bd(nboxes);
  std::vector<BoxSrc> src(nboxes);
  std::vector<int> kvoff(nboxes, 0), has_ew(nboxes, 0);
  int atom_off = 0, cell_off = 0, kv_total = 0, max_na = 0;
  size_t max_smem32 = 0, max_smem64 = 0;
  const bool mixed = c->precision == CASS_PREC_MIXED;
  bool any_recip = false;
  // the FP32 warp kernel covers LJ cut / cut_tail with no charges or Ewald
  bool fast_mixed = c->pt.ntypes <= kMaxTypes;
  for (int k = 0; k < nboxes; ++k) {
    int ib = iboxes[k] - 1;
    if ((rc = pack_box_ext(c, ib))) return rc;
    BoxH& B = c->box[ib];
    BoxDev v = B.dev;
    // cells of about half the CBMC cutoff: the row-trimmed stencils then visit
    // little more than the cutoff sphere
    const double cpc = c->widom_cells > 0.0 ? c->widom_cells
                                             : (c->precision == CASS_PREC_MIXED ? kCellsPerCutoffMixed : kCellsPerCutoffFP64);
    double rcell = (B.desc.rcut_cbmc > 0.0 ? B.desc.rcut_cbmc : B.rcut_max) / cpc;
    int ncell = 1;
    for (int d = 0; d < 3; ++d) {
      v.nc[d] = std::max(1, (int)std::floor(v.L[d] / rcell));
      v.nc[d] = std::min(v.nc[d], 64);
      v.cell_inv[d] = (double)v.nc[d] / v.L[d];
      ncell *= v.nc[d];
    }
    v.atom_off = atom_off;
    v.natoms = B.npacked;
    v.cell_off = cell_off;
    v.mcom = B.comcut ? B.d_com.as<double4_32a>() : nullptr;  // built with the packed arrays
    v.rcut_max = B.rcut_max;
    // Widom_Insert set-up (widom_insert.f90:201-245)
    const std::vector<int>& mem = members_ext(c, ib);
    int nmols = 1;
    for (int slot : mem)
      if (c->slot_sp[slot] == is0) ++nmols;
    v.prefactor = v.volume / (double)nmols;
    double lrc_diff = 0.0;
    if (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) {
      std::vector<double> nb(c->ntypes, 0.0);
      for (int slot : mem) {
        const SpeciesH& t = c->sp[c->slot_sp[slot]];
        for (int a = 0; a < t.natoms; ++a)
          if (t.type[a] >= 0) nb[t.type[a]] += 1.0;
      }
      for (int a = 0; a < s.natoms; ++a)
        if (s.type[a] >= 0) nb[s.type[a]] += 1.0;
      lrc_diff = lrc_host(c, B, nb) - B.energy.lrc;
    }
    double e_self = 0.0, e_recip_in = 0.0;
    if (B.desc.charge_style == CASS_CHARGE_COUL && s.has_charge) {
      double qq = 0.0;
      for (int a = 0; a < s.natoms; ++a) qq += s.q[a] * s.q[a];
      if (B.desc.charge_sum_style == CASS_QQ_EWALD) e_self = -qq * kCHARGE_FACTOR * v.alpha / kROOTPI;
      else if (B.desc.charge_sum_style == CASS_QQ_DSF)
        e_self = -qq * (v.alpha_dsf / kROOTPI + v.dsf_factor1 / 2.0) * kCHARGE_FACTOR;
      e_recip_in = B.energy.reciprocal;
    }
    v.e_inter_constant = lrc_diff + e_self - e_recip_in;
    fast_mixed = fast_mixed && B.desc.vdw_style == CASS_VDW_LJ &&
                 (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT || B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) &&
                 (B.desc.charge_style == CASS_CHARGE_NONE || B.desc.charge_sum_style == CASS_QQ_EWALD);
    if (B.desc.charge_style == CASS_CHARGE_COUL && B.desc.charge_sum_style == CASS_QQ_EWALD && s.has_charge &&
        B.nvecs > 0) {
      has_ew[k] = 1;
      any_recip = true;
    }
    kvoff[k] = kv_total;
    kv_total += B.nvecs;
    bd[k] = v;
    src[k].p64 = B.d_p64.as<double4_32a>();
    src[k].p32 = B.d_p32.as<float4>();
    src[k].meta = B.d_meta.as<int4>();
    const size_t sm_cells = ((size_t)(ncell + 1) * sizeof(int) + 31) & ~(size_t)31;
    max_smem32 = std::max(max_smem32, sm_cells + (size_t)B.npacked * sizeof(float4));
    max_smem64 = std::max(max_smem64, sm_cells + (size_t)B.npacked * (sizeof(double4_32a) + sizeof(int)));
    max_na = std::max(max_na, B.npacked);
    atom_off += B.npacked;
    cell_off += ncell;
  }
  const int total_atoms = std::max(1, atom_off), total_cells = cell_off;
  // device buffers
  DevBuf& dbox = c->d_boxdev;
  if ((rc = dbox.reserve(nboxes * sizeof(BoxDev) + nboxes * sizeof(BoxSrc) + 3 * nboxes * sizeof(int) + 64))) return rc;
  BoxDev* d_bd = dbox.as<BoxDev>();
  BoxSrc* d_src = reinterpret_cast<BoxSrc*>(d_bd + nboxes);
  int* d_ids = reinterpret_cast<int*>(d_src + nboxes);
  int* d_kvoff = d_ids + nboxes;
  int* d_hasew = d_kvoff + nboxes;
  if ((rc = c->d_c64.reserve((size_t)total_atoms * sizeof(double4_32a)))) return rc;
  if ((rc = c->d_c32.reserve((size_t)total_atoms * sizeof(float4) + (size_t)total_atoms * 2 * sizeof(int)))) return rc;
  if ((rc = c->d_cq32.reserve((size_t)total_atoms * sizeof(float)))) return rc;
  if ((rc = c->d_cell_start.reserve(((size_t)total_cells + nboxes) * sizeof(int)))) return rc;
  if ((rc = c->d_cell_count.reserve(((size_t)total_cells * 2 + 64) * sizeof(int)))) return rc;
  if ((rc = c->d_cell_of.reserve((size_t)total_atoms * sizeof(int)))) return rc;
  float4* d_c32 = c->d_c32.as<float4>();
  int* d_ctype = reinterpret_cast<int*>(d_c32 + total_atoms);
  int* d_corig = d_ctype + total_atoms;
  int* d_count = c->d_cell_count.as<int>();
  int* d_fill = d_count + total_cells;
  CASS_CUDA(h2d(c, d_bd, bd.data(), nboxes * sizeof(BoxDev)));
  CASS_CUDA(h2d(c, d_src, src.data(), nboxes * sizeof(BoxSrc)));
  CASS_CUDA(h2d(c, d_ids, iboxes, nboxes * sizeof(int)));
  CASS_CUDA(h2d(c, d_kvoff, kvoff.data(), nboxes * sizeof(int)));
  CASS_CUDA(h2d(c, d_hasew, has_ew.data(), nboxes * sizeof(int)));
  CASS_CUDA(cudaEventRecord(c->ev[0], c->stream));
  CASS_CUDA(cudaMemsetAsync(d_count, 0, (size_t)std::max(1, total_cells) * sizeof(int), c->stream));
  // K7
  if (max_na > 0) {
    dim3 g((max_na + 255) / 256, nboxes);
    k_cell_count<<<g, 256, 0, c->stream>>>(d_src, d_bd, c->d_cell_of.as<int>(), d_count);
    k_cell_scan<<<nboxes, 1024, 0, c->stream>>>(d_bd, d_count, c->d_cell_start.as<int>(), d_fill);
    k_cell_scatter<<<g, 256, 0, c->stream>>>(d_src, d_bd, c->d_cell_of.as<int>(), c->d_cell_start.as<int>(), d_fill,
                                             c->d_c64.as<double4_32a>(), d_c32, d_ctype, c->d_cq32.as<float>(), d_corig);
    int maxc = 1;
    for (int k = 0; k < nboxes; ++k) maxc = std::max(maxc, bd[k].nc[0] * bd[k].nc[1] * bd[k].nc[2]);
    dim3 gs((maxc + 127) / 128, nboxes);
    k_cell_sort<<<gs, 128, 0, c->stream>>>(d_bd, nboxes, c->d_cell_start.as<int>(), c->d_c64.as<double4_32a>(), d_c32,
                                           d_ctype, c->d_cq32.as<float>(), d_corig);
  } else {
    k_cell_scan<<<nboxes, 1024, 0, c->stream>>>(d_bd, d_count, c->d_cell_start.as<int>(), d_fill);
  }
  CASS_CUDA(cudaGetLastError());
  count_launch(c, max_na > 0 ? 4 : 1);
  // per-insertion records
  size_t nrec = (size_t)nboxes * (size_t)std::max<int64_t>(1, n_ins);
  DevBuf& drec = c->d_widom_out;
  if ((rc = drec.reserve(nrec * (sizeof(WRec) + 1) + 64))) return rc;
  WRec* d_rec = drec.as<WRec>();
  signed char* d_status = reinterpret_cast<signed char*>(d_rec + nrec);
  double* d_xyz = nullptr;
  if (any_recip) {
    if ((rc = c->d_widom_xyz.reserve(nrec * 3 * s.natoms * sizeof(double) + s.natoms * sizeof(double)))) return rc;
    d_xyz = c->d_widom_xyz.as<double>();
  }
  CassWidomTrace* d_trace = nullptr;
  if (trace) {
    if ((rc = c->d_trace.reserve(nrec * sizeof(CassWidomTrace)))) return rc;
    d_trace = c->d_trace.as<CassWidomTrace>();
  }
  if ((rc = c->d_box_sums.reserve((size_t)nboxes * (sizeof(double) + sizeof(long long)) + 2 * sizeof(long long))))
    return rc;
  double* d_bsum = c->d_box_sums.as<double>();
  long long* d_bov = reinterpret_cast<long long*>(d_bsum + nboxes);
  unsigned long long* d_pairs = c->count_pairs ? reinterpret_cast<unsigned long long*>(d_bov + nboxes) : nullptr;
  if (d_pairs) CASS_CUDA(cudaMemsetAsync(d_pairs, 0, 2 * sizeof(unsigned long long), c->stream));
  // K8 launch shape: 128-thread CTAs, enough CTAs per box to fill every SM;
  // the box is staged in shared memory when it fits
  SpeciesF SF;
  const bool f32 = mixed && fast_mixed && species_f(s, SF);
  const size_t max_smem = f32 ? max_smem32 : max_smem64;
  const bool use_smem = max_smem <= (size_t)200 * 1024;
  int dev_sms = 0;
  CASS_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  const int threads = 128;
  auto launch = [&](auto kern) -> int {
    if (use_smem) CASS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem));
    int per_sm = 1;
    CASS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, use_smem ? max_smem : 0));
    per_sm = std::max(per_sm, 1);
    long long want = ((long long)dev_sms * per_sm * 2 + nboxes - 1) / nboxes;
    long long need = (n_ins + threads - 1) / threads;
    int chunks = (int)std::max<long long>(1, std::min(want, need));
    dim3 g(chunks, nboxes);
    c->stats.widom_grid_x = chunks;
    c->stats.widom_grid_y = nboxes;
    c->stats.widom_block = threads;
    c->stats.widom_smem_bytes = use_smem ? (int)max_smem : 0;
    CASS_CUDA(cudaEventRecord(c->ev[1], c->stream));
    kern<<<g, threads, use_smem ? max_smem : 0, c->stream>>>(
        S, c->pt, c->pools, d_bd, d_ids, c->d_c64.as<double4_32a>(), d_ctype, d_corig, c->d_cell_start.as<int>(),
        s.d_library.as<double>(), (long long)n_ins, seed, d_rec, d_status, d_xyz, any_recip ? 1 : 0, d_trace, d_pairs);
    CASS_CUDA(cudaGetLastError());
    CASS_CUDA(cudaEventRecord(c->ev[2], c->stream));
    count_launch(c);
    return CASS_OK;
  };
  // FP32 kernel of the mixed path, then the FP64 fix-up of the insertions it
  // queued (both inside the kernel timing)
  int* d_fixn = nullptr;
  FixEntry* d_fixq = nullptr;
  auto launch_f32 = [&](auto kern, const SpeciesF& SF, int nthreads) -> int {
    int rc2 = c->d_widom_fix.reserve((size_t)nboxes * sizeof(int) + 64 + nrec * sizeof(FixEntry));
    if (rc2) return rc2;
    d_fixn = c->d_widom_fix.as<int>();
    d_fixq = reinterpret_cast<FixEntry*>(c->d_widom_fix.as<unsigned char>() +
                                         (((size_t)nboxes * sizeof(int) + 63) & ~(size_t)63));
    CASS_CUDA(cudaMemsetAsync(d_fixn, 0, (size_t)nboxes * sizeof(int), c->stream));
    if (use_smem) CASS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem));
    int per_sm = 1;
    CASS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nthreads, use_smem ? max_smem : 0));
    per_sm = std::max(per_sm, 1);
    const int waves = c->widom_waves > 0 ? c->widom_waves : kF32Waves;
    long long want = ((long long)dev_sms * per_sm * waves + nboxes - 1) / nboxes;
    long long need = (n_ins + nthreads - 1) / nthreads;
    int chunks = (int)std::max<long long>(1, std::min(want, need));
    dim3 g(chunks, nboxes);
    c->stats.widom_grid_x = chunks;
    c->stats.widom_grid_y = nboxes;
    c->stats.widom_block = nthreads;
    c->stats.widom_smem_bytes = use_smem ? (int)max_smem : 0;
    CASS_CUDA(cudaEventRecord(c->ev[1], c->stream));
    kern<<<g, nthreads, use_smem ? max_smem : 0, c->stream>>>(
        S, SF, c->pt, d_bd, d_ids, d_c32, c->d_cq32.as<float>(), c->d_cell_start.as<int>(), s.d_library_f.as<float>(),
        (long long)n_ins, seed, d_rec, d_status, d_xyz, any_recip ? 1 : 0, d_trace, d_fixq, d_fixn, c->widom_band,
        d_pairs);
    CASS_CUDA(cudaGetLastError());
    // one thread per queued insertion, the grid sized for 3 % of the
    // insertions (one to two per cent are queued; a longer queue is strided)
    const int fix_chunks = (int)std::max<long long>(1, std::min<long long>(64, (n_ins * 3 / 100 + 127) / 128));
    k_widom_fix<<<dim3(fix_chunks, nboxes), 128, 0, c->stream>>>(
        S, SF, c->pt, d_bd, d_ids, d_c32, c->d_cq32.as<float>(), c->d_c64.as<double4_32a>(), c->d_cell_start.as<int>(),
        s.d_library.as<double>(), (long long)n_ins, seed, d_fixq, d_fixn, d_rec, d_status, d_xyz, any_recip ? 1 : 0,
        d_trace, c->widom_band);
    CASS_CUDA(cudaGetLastError());
    CASS_CUDA(cudaEventRecord(c->ev[2], c->stream));
    count_launch(c, 2);
    return CASS_OK;
  };
  if (n_ins > 0) {
    const bool opt = c->cbmc_opt.energy_table_res > 0 || c->cbmc_opt.sector_overlap;  // no pair counts with options
    const int nt = opt || d_pairs ? kF32Threads : (c->widom_threads == 256 ? 256 : kF32Threads);
    if (f32 && opt) rc = use_smem ? launch_f32(k_widom_f32<true, false, true>, SF, nt) : launch_f32(k_widom_f32<false, false, true>, SF, nt);
    else if (f32 && d_pairs) rc = use_smem ? launch_f32(k_widom_f32<true, true, false>, SF, nt) : launch_f32(k_widom_f32<false, true, false>, SF, nt);
    else if (f32 && nt == 256)
      rc = use_smem ? launch_f32(k_widom_f32<true, false, false, 256>, SF, nt) : launch_f32(k_widom_f32<false, false, false, 256>, SF, nt);
    else if (f32) rc = use_smem ? launch_f32(k_widom_f32<true, false, false>, SF, nt) : launch_f32(k_widom_f32<false, false, false>, SF, nt);
    else rc = use_smem ? launch(k_widom<true>) : launch(k_widom<false>);
    if (rc) return rc;
    if (any_recip) {
      // k-vectors and structure factors of the batch boxes, concatenated
      if ((rc = c->d_partial.reserve((size_t)std::max(1, kv_total) * sizeof(double) * 6))) return rc;
      double4_32a* d_kv = reinterpret_cast<double4_32a*>(c->d_partial.p);
      double* d_cs = reinterpret_cast<double*>(d_kv + kv_total);
      double* d_sn = d_cs + kv_total;
      for (int k = 0; k < nboxes; ++k) {
        BoxH& B = c->box[iboxes[k] - 1];
        if (!B.nvecs) continue;
        CASS_CUDA(cudaMemcpyAsync(d_kv + kvoff[k], B.d_kvec.p, B.nvecs * sizeof(double4_32a), cudaMemcpyDeviceToDevice,
                                  c->stream));
        CASS_CUDA(cudaMemcpyAsync(d_cs + kvoff[k], B.d_cos_sum.p, B.nvecs * sizeof(double), cudaMemcpyDeviceToDevice,
                                  c->stream));
        CASS_CUDA(cudaMemcpyAsync(d_sn + kvoff[k], B.d_sin_sum.p, B.nvecs * sizeof(double), cudaMemcpyDeviceToDevice,
                                  c->stream));
      }
      double* d_q = d_xyz + nrec * 3 * s.natoms;
      CASS_CUDA(h2d(c, d_q, s.q.data(), s.natoms * sizeof(double)));
      k_widom_recip<<<(unsigned)nrec, 256, 0, c->stream>>>(d_bd, d_kv, d_cs, d_sn, d_kvoff, d_hasew, (long long)n_ins,
                                                          s.natoms, d_q, d_status, d_xyz, d_rec, d_trace);
      CASS_CUDA(cudaGetLastError());
  count_launch(c);
    }
  }
  k_widom_finalize<<<nboxes, 256, 0, c->stream>>>(d_bd, (long long)n_ins, d_rec, d_status, d_bsum, d_bov, d_trace);
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  CASS_CUDA(cudaEventRecord(c->ev[3], c->stream));
  unsigned long long hpairs[2] = {0, 0};
  if (d_pairs) CASS_CUDA(d2h(c, hpairs, d_pairs, sizeof(hpairs)));
  std::vector<int> hfix(d_fixn ? nboxes : 0);
  if (d_fixn) CASS_CUDA(d2h(c, hfix.data(), d_fixn, nboxes * sizeof(int)));
  std::vector<double> hs(nboxes);
  std::vector<long long> ho(nboxes);
  CASS_CUDA(d2h(c, hs.data(), d_bsum, nboxes * sizeof(double)));
  CASS_CUDA(d2h(c, ho.data(), d_bov, nboxes * sizeof(long long)));
  if (trace)
    CASS_CUDA(d2h(c, trace, d_trace, nrec * sizeof(CassWidomTrace)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  float ms_all = 0.0f, ms_k = 0.0f;
  CASS_CUDA(cudaEventElapsedTime(&ms_all, c->ev[0], c->ev[3]));
  if (n_ins > 0) CASS_CUDA(cudaEventElapsedTime(&ms_k, c->ev[1], c->ev[2]));
  c->stats.widom_ms = ms_all;
  c->stats.widom_kernel_ms = ms_k;
  c->stats.widom_pairs_visited = (int64_t)hpairs[0];
  c->stats.widom_pairs_in_cutoff = (int64_t)hpairs[1];
  c->stats.widom_fixups = 0;
  for (int v : hfix) c->stats.widom_fixups += v;
  for (int k = 0; k < nboxes; ++k) {
    out[k].widom_sum = hs[k] * bd[k].prefactor;
    out[k].prefactor = bd[k].prefactor;
    out[k].n_insertions = n_ins;
    out[k].n_overlaps = ho[k];
    out[k].n_trials = n_ins * (int64_t)(kappa_ins + (s.nfrag - 1) * (s.nfrag > 1 ? kappa_dih : 0));
  }
  return CASS_OK;
}

// The launch-shape autotuner: the first call with a new batch signature
// (species, boxes, precision, CBMC options, order of magnitude of the insertion
// count) times the Widom kernel with each candidate cell edge on a sample of the
// insertions with its own seed (the faster of two runs after a first that sizes
// the buffers), keeps the fastest
// for the context, and then runs the call.  A shape changes neither the
// insertions' random streams nor the per-box sums (fixed order over
// insertions); the cell edge changes only the order of each query's pair sum.
extern "C" int cass_widom_insert(cass_ctx* c, int32_t is1, int32_t nboxes, const int32_t* iboxes, int64_t n_ins,
                                 int32_t kappa_ins, int32_t kappa_dih, uint64_t seed, CassWidomResult* out,
                                 CassWidomTrace* trace) {
  if (!c || !iboxes || nboxes < 1 || !out || n_ins < 64 || !c->widom_autotune || c->widom_cells > 0.0 ||
      c->widom_waves > 0 || c->widom_threads > 0)
    return widom_insert_impl(c, is1, nboxes, iboxes, n_ins, kappa_ins, kappa_dih, seed, out, trace);
  std::vector<long long> key = {is1, c->precision, kappa_ins, kappa_dih, c->cbmc_opt.energy_table_res,
                                c->cbmc_opt.sector_overlap, (long long)std::log2((double)n_ins)};
  for (int k = 0; k < nboxes; ++k) key.push_back(iboxes[k]);
  auto run_with = [&](const cass_ctx_impl::WidomShape& sh, int64_t n, uint64_t sd, CassWidomResult* o,
                      CassWidomTrace* tr) {
    c->widom_cells = sh.cells;
    c->widom_waves = sh.waves;
    c->widom_threads = sh.threads;
    const int rc = widom_insert_impl(c, is1, nboxes, iboxes, n, kappa_ins, kappa_dih, seed ^ sd, o, tr);
    c->widom_cells = 0.0;
    c->widom_waves = 0;
    c->widom_threads = 0;
    return rc;
  };
  for (const auto& e : c->widom_tuned)
    if (e.first == key) return run_with(e.second, n_ins, 0, out, trace);
  const bool mixed = c->precision == CASS_PREC_MIXED;
  // candidate shapes: the cell edge (cells per rcut_cbmc) and, for the FP32
  // kernel, the CTA size (512 threads two per SM, or 256 threads)
  std::vector<cass_ctx_impl::WidomShape> shapes;
  if (mixed)
    for (int nt : {512, 256})
      for (double cc : {1.0, 1.25}) shapes.push_back({cc, kF32Waves, nt});
  else
    for (double cc : {3.0, 4.0}) shapes.push_back({cc, kF32Waves, 512});
  // the CTAs per box follow the insertion count, so the mixed kernel is timed at
  // the call's own count (up to 32,768 per box); the FP64 kernel on 4,096
  const int64_t sample = std::min<int64_t>(n_ins, mixed ? 32768 : 4096);
  std::vector<CassWidomResult> tmp(nboxes);
  cass_ctx_impl::WidomShape best = shapes[0];
  float best_ms = -1.0f;
  for (const auto& sh : shapes) {
    float ms = 0.0f;
    for (int rep = 0; rep < 3; ++rep) {  // the first run of a shape also sizes its buffers
      const int rc = run_with(sh, sample, 0x5bd1e995ULL, tmp.data(), nullptr);
      if (rc) return rc;
      if (rep == 1 || (rep == 2 && c->stats.widom_kernel_ms < ms)) ms = c->stats.widom_kernel_ms;
    }
    if (best_ms < 0.0f || ms < best_ms) {
      best_ms = ms;
      best = sh;
    }
  }
  c->widom_tuned.push_back({key, best});
  return run_with(best, n_ins, 0, out, trace);
}
