// cass_abi.cu -- C-ABI entry points of libcassgpu.so and the energy kernels
// that back them:
//   k_mol_inter      Compute_Molecule_Nonbond_Inter_Energy   (energy_routines.f90:1088-1206)
//   k_pair_total     inter-molecular part of Compute_System_Total_Energy (:2775-2917)
//   k_intra_total    intra + bonded part of Compute_System_Total_Energy  (:2697-2769)
//   k_sfac / k_sfac_reduce  Compute_System_Ewald_Reciprocal_Energy     (:4111-4231)
//   k_ewald_update   Update_System_Ewald_Reciprocal_Energy   (:2326-2497)
//   k_ewald_widom    Update_System_Ewald_Reciprocal_Energy_Widom (:2500-2550)
// Reductions are deterministic: each block writes a partial, the last block to
// finish sums the partials in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "cass_cbmc.cuh"
#include "cass_ctx.h"

namespace cassgpu {

static thread_local std::string g_err;

int set_error(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_error(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return CASS_ECUDA;
}

cudaError_t h2d(cass_ctx_impl* c, void* dst, const void* src, size_t n) {
  c->stats.h2d_bytes += (int64_t)n;
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, c->stream);
}

cudaError_t d2h(cass_ctx_impl* c, void* dst, const void* src, size_t n) {
  c->stats.d2h_bytes += (int64_t)n;
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, c->stream);
}

// packed molecule record: mol slot, species (0-based), first packed atom, natoms
using MolInfo = int4;

struct BoxPtrs {
  double4_32a* p64;
  float4* p32;
};

__global__ void k_patch_atoms(const PatchRec* rec, int n, const BoxPtrs* bp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PatchRec r = rec[i];
  const BoxPtrs b = bp[r.box];
  double4_32a p = b.p64[r.atom];
  p.x = r.x;
  p.y = r.y;
  p.z = r.z;
  b.p64[r.atom] = p;
  float4 f = b.p32[r.atom];
  f.x = (float)r.x;
  f.y = (float)r.y;
  f.z = (float)r.z;
  b.p32[r.atom] = f;
}

constexpr int kBlock = 256;

// Check_MoleculePair_Cutoff (energy_routines.f90:3027-3088): the molecules
// interact unless their COMs (minimum image) are farther apart than rmax
// (rcut_max, or rcut_cbmc with the CBMC flag) plus both max_dcom
__device__ __forceinline__ bool molpair_in(const BoxDev& b, double rmax, const double4_32a& ci, const double4_32a& cj) {
  const double dx = fold(ci.x - cj.x, b.hL[0], b.L[0]), dy = fold(ci.y - cj.y, b.hL[1], b.L[1]),
               dz = fold(ci.z - cj.z, b.hL[2], b.L[2]);
  const double rcom = sqrt(dx * dx + dy * dy + dz * dz);
  return !(rcom > rmax + ci.w + cj.w);
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;  // valid in thread 0
}

// Writes NV partial sums of this block, then the last block to finish sums
// all partials (fixed order) into out[0..NV).  counter must start at 0 and is
// reset by the last block.
template <int NV>
__device__ void reduce_partials(double (&v)[NV], double* partial, unsigned* counter, double* out, int* flag_in,
                                int flag_val) {
  __shared__ double sh[32];
  __shared__ bool last;
  int nb = gridDim.x * gridDim.y;
  int bid = blockIdx.y * gridDim.x + blockIdx.x;
  for (int k = 0; k < NV; ++k) {
    double s = block_sum(v[k], sh);
    if (threadIdx.x == 0) partial[(size_t)bid * NV + k] = s;
  }
  (void)flag_in;
  (void)flag_val;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == (unsigned)(nb - 1));
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += __ldcg(&partial[(size_t)b * NV + k]);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[k] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// ---------------------------------------------------------------------------
// K1: one molecule against every other live molecule of its box.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_mol_inter(BoxDev b, PairTable t, const double4_32a* __restrict__ p64,
                                                      const float4* __restrict__ p32, const int4* __restrict__ meta,
                                                      int n, int qslot, int qoff, int qn, int cbmc, int want_qq,
                                                      const double4_32a* __restrict__ com, double rmax,
                                                      double* partial, unsigned* counter, double* out, int* ovflag) {
  __shared__ double4_32a qa[kMaxAtoms * 4];
  __shared__ int qt[kMaxAtoms * 4];
  for (int a = threadIdx.x; a < qn; a += blockDim.x) {
    qa[a] = p64[qoff + a];
    qt[a] = meta[qoff + a].y;
  }
  __syncthreads();
  double ev = 0.0, eq = 0.0;
  KahanF fv, fq;
  bool ov = false;
  const bool table = cbmc && b.tab_res > 0;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    int4 mj = meta[j];
    if (mj.x == qslot) continue;
    if (com && !molpair_in(b, rmax, com[qoff], com[j])) continue;
    double4_32a pj = p64[j];
    for (int a = 0; a < qn; ++a) {
      double dx = fold(qa[a].x - pj.x, b.hL[0], b.L[0]);
      double dy = fold(qa[a].y - pj.y, b.hL[1], b.L[1]);
      double dz = fold(qa[a].z - pj.z, b.hL[2], b.L[2]);
      double r2 = dx * dx + dy * dy + dz * dz;
      if (table) {  // Estimate_MoleculePair_Energy: the combined energy goes to the vdW sum
        if (table_pair(b, t.ntypes, r2, qt[a], mj.y, qa[a].w, pj.w, ev) == 2) ov = true;
        continue;
      }
      if (r2 < b.rcut_lowsq) {
        ov = true;
        continue;
      }
      int m = cutoff_mask(b, r2, cbmc != 0);
      if (!want_qq) m &= 1;
      if (MIXED && lj_plain_style(b)) {
        if ((m & 1) && qt[a] >= 0 && mj.y >= 0) {
          int k = pidx(qt[a], mj.y, t.ntypes);
          fv.add(lj_pair_f(t.epsf[k], t.sig2f[k], (float)r2));
        }
      } else if (m & 1) {
        ev += vdw_pair(t, b, qt[a], mj.y, r2, 1.0);
      }
      if (m & 2) {
        if (MIXED && b.charge_sum_style == CASS_QQ_EWALD)
          fq.add(qq_ewald_inter_f((float)b.alpha, (float)(qa[a].w * pj.w), (float)r2));
        else
          eq += qq_pair_inter(b, qa[a].w * pj.w, r2);
      }
    }
  }
  if (ov) atomicOr(ovflag, 1);
  double v[2] = {ev + fv.value(), eq + fq.value()};
  reduce_partials<2>(v, partial, counter, out, nullptr, 0);
}

// ---------------------------------------------------------------------------
// K2/K3 trial energies: one CTA per CBMC trial position, threads over the box
// atoms, the trial's atoms in shared memory; block sum in a fixed order.
constexpr int kTrialMaxAtoms = 64;

// tcom (may be NULL): per trial its atoms' COM and max_dcom, with com the box
// atoms' COM records, for Check_MoleculePair_Cutoff with radius rmax
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_trial_energy(BoxDev b, PairTable t, const double4_32a* __restrict__ p64,
                                                         const int4* __restrict__ meta, int n, int skip_slot,
                                                         const double4_32a* __restrict__ trial, const int* ttype,
                                                         int nat, int cbmc, int want_qq, const double4_32a* __restrict__ tcom,
                                                         const double4_32a* __restrict__ com, double rmax, double* e,
                                                         int* overlap) {
  __shared__ double4_32a qa[kTrialMaxAtoms];
  __shared__ int qt[kTrialMaxAtoms];
  __shared__ double sh[32];
  __shared__ int ovs;
  const double4_32a* tr = trial + (size_t)blockIdx.x * nat;
  for (int a = threadIdx.x; a < nat; a += blockDim.x) {
    qa[a] = tr[a];
    qt[a] = ttype[a];
  }
  if (threadIdx.x == 0) ovs = 0;
  __syncthreads();
  double ev = 0.0, eq = 0.0;
  KahanF fv, fq;
  bool ov = false;
  const bool table = cbmc && b.tab_res > 0;
  for (int j = threadIdx.x; j < n && !ov; j += blockDim.x) {
    const int4 mj = meta[j];
    if (mj.x == skip_slot) continue;
    if (tcom && !molpair_in(b, rmax, tcom[blockIdx.x], com[j])) continue;
    const double4_32a pj = p64[j];
    for (int a = 0; a < nat; ++a) {
      const double dx = fold(qa[a].x - pj.x, b.hL[0], b.L[0]);
      const double dy = fold(qa[a].y - pj.y, b.hL[1], b.L[1]);
      const double dz = fold(qa[a].z - pj.z, b.hL[2], b.L[2]);
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (table) {  // Estimate_MoleculePair_Energy
        if (table_pair(b, t.ntypes, r2, qt[a], mj.y, qa[a].w, pj.w, ev) == 2) {
          ov = true;
          break;
        }
        continue;
      }
      if (r2 < b.rcut_lowsq) {
        ov = true;
        break;
      }
      int m = cutoff_mask(b, r2, cbmc != 0);
      if (!want_qq) m &= 1;
      if (MIXED && lj_plain_style(b)) {
        if ((m & 1) && qt[a] >= 0 && mj.y >= 0) {
          const int k = pidx(qt[a], mj.y, t.ntypes);
          fv.add(lj_pair_f(t.epsf[k], t.sig2f[k], (float)r2));
        }
      } else if (m & 1) {
        ev += vdw_pair(t, b, qt[a], mj.y, r2, 1.0);
      }
      if (m & 2) {
        if (MIXED && b.charge_sum_style == CASS_QQ_EWALD)
          fq.add(qq_ewald_inter_f((float)b.alpha, (float)(qa[a].w * pj.w), (float)r2));
        else
          eq += qq_pair_inter(b, qa[a].w * pj.w, r2);
      }
    }
  }
  if (ov) atomicOr(&ovs, 1);
  const double s = block_sum(ev + fv.value() + eq + fq.value(), sh);
  __syncthreads();
  if (threadIdx.x == 0) {
    overlap[blockIdx.x] = ovs;
    e[blockIdx.x] = ovs ? 0.0 : s;
  }
}

// ---------------------------------------------------------------------------
// K6a: all inter-molecular pairs of a box (pairs (i,j), j > i, different
// molecules).  Block (x, y) takes atoms i of row block x against the j tile y,
// staged in shared memory.  FAST (mixed precision, LJ cut / cut_tail with no
// charges or Ewald): FP32 minimum image, r^2 and pair energies with
// compensated FP32 sums; otherwise the FP64 pair functions.
constexpr int kTileJ = 512;

template <bool FAST>
// pre2 (FP64 kernel): an FP32 bound on r^2 beyond every cutoff of the box with
// a margin far above FP32 rounding; pairs past it skip the FP64 arithmetic,
// which decides every cutoff exactly (FLT_MAX where a style has no cutoff)
// com (FP64 kernel, may be NULL): per-atom molecule COM records for
// Check_MoleculePair_Cutoff with radius rmax
__global__ void __launch_bounds__(kBlock) k_pair_total(BoxDev b, PairTable t, const double4_32a* __restrict__ p64,
                                                       const int4* __restrict__ meta, int n, float pre2,
                                                       const double4_32a* __restrict__ com, double rmax,
                                                       double* partial, unsigned* counter, double* out, int* ovflag) {
  __shared__ double4_32a sj[FAST ? 1 : kBlock];
  __shared__ float4 sf[kBlock];
  __shared__ int2 sm[kBlock];  // molecule slot, type
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double4_32a pi = i < n ? p64[i] : make_double4_32a(0, 0, 0, 0);
  const int4 mi = i < n ? meta[i] : make_int4(-1, -1, -1, -1);
  const float4 pif = make_float4((float)pi.x, (float)pi.y, (float)pi.z, (float)pi.w);
  double ev = 0.0, eq = 0.0;
  KahanF fv, fq;
  bool ov = false;
  const int j0 = blockIdx.y * kTileJ;
  const int j1 = min(n, j0 + kTileJ);
  const int ilo = blockIdx.x * blockDim.x;
  const float rv2f = (float)b.rcut_vdwsq, rq2f = (float)b.rcut_coulsq, low2f = (float)b.rcut_lowsq;
  const float alphaf = (float)b.alpha;
  const bool qq_on = b.charge_style == CASS_CHARGE_COUL;
  float eps_row[kMaxTypes], sig_row[kMaxTypes];
  if (FAST)
#pragma unroll
    for (int q = 0; q < kMaxTypes; ++q) {
      const bool ok = mi.y >= 0 && q < t.ntypes;
      eps_row[q] = ok ? t.epsf[pidx(mi.y, q, t.ntypes)] : 0.0f;
      sig_row[q] = ok ? t.sig2f[pidx(mi.y, q, t.ntypes)] : 0.0f;
    }
  if (j1 > ilo + 1) {
    for (int jt = max(j0, ilo); jt < j1; jt += kBlock) {
      __syncthreads();
      const int jj = jt + threadIdx.x;
      if (jj < j1) {
        const double4_32a pj = p64[jj];
        const int4 mj = meta[jj];
        sf[threadIdx.x] = make_float4((float)pj.x, (float)pj.y, (float)pj.z, (float)pj.w);
        if (!FAST) sj[threadIdx.x] = pj;
        sm[threadIdx.x] = make_int2(mj.x, mj.y);
      }
      __syncthreads();
      const int cnt = min(kBlock, j1 - jt);
      if (i >= n) continue;
      for (int k = 0; k < cnt; ++k) {
        const int j = jt + k;
        if (j <= i) continue;
        const int2 mj = sm[k];
        if (mj.x == mi.x) continue;
        if (FAST) {
          const float4 pj = sf[k];
          const float dx = fold(pif.x - pj.x, b.hLf[0], b.Lf[0]);
          const float dy = fold(pif.y - pj.y, b.hLf[1], b.Lf[1]);
          const float dz = fold(pif.z - pj.z, b.hLf[2], b.Lf[2]);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          if (r2 < low2f) {
            ov = true;
            continue;
          }
          if (r2 <= rv2f && mj.y >= 0) {
            float e = 0.0f, s2 = 0.0f;
#pragma unroll
            for (int q = 0; q < kMaxTypes; ++q)
              if (q == mj.y) {
                e = eps_row[q];
                s2 = sig_row[q];
              }
            fv.add(lj_pair_f(e, s2, r2));
          }
          if (qq_on && r2 <= rq2f) fq.add(qq_ewald_inter_f(alphaf, pif.w * pj.w, r2));
        } else {
          {
            const float4 q = sf[k];
            const float ex = fold(pif.x - q.x, b.hLf[0], b.Lf[0]), ey = fold(pif.y - q.y, b.hLf[1], b.Lf[1]),
                        ez = fold(pif.z - q.z, b.hLf[2], b.Lf[2]);
            if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > pre2) continue;
          }
          if (com && !molpair_in(b, rmax, com[i], com[j])) continue;
          const double4_32a pj = sj[k];
          const double dx = fold(pi.x - pj.x, b.hL[0], b.L[0]);
          const double dy = fold(pi.y - pj.y, b.hL[1], b.L[1]);
          const double dz = fold(pi.z - pj.z, b.hL[2], b.L[2]);
          const double r2 = dx * dx + dy * dy + dz * dz;
          if (r2 < b.rcut_lowsq) {
            ov = true;
            continue;
          }
          const int m = cutoff_mask(b, r2, false);
          if (m & 1) ev += vdw_pair(t, b, mi.y, mj.y, r2, 1.0);
          if (m & 2) eq += qq_pair_inter(b, pi.w * pj.w, r2);
        }
      }
    }
  }
  if (ov) atomicOr(ovflag, 1);
  double v[2] = {ev + fv.value(), eq + fq.value()};
  reduce_partials<2>(v, partial, counter, out, nullptr, 0);
}

__global__ void __launch_bounds__(kBlock) k_intra_total(BoxDev b, PairTable t, SpeciesPools P,
                                                        const double4_32a* __restrict__ p64,
                                                        const MolInfo* __restrict__ mols, int nm, double* partial,
                                                        unsigned* counter, double* out, int* ovflag, int cbmc = 0) {
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  double r[3 * 64];
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    MolInfo mi = mols[m];
    int na = min(mi.w, 64);
    for (int a = 0; a < na; ++a) {
      double4_32a p = p64[mi.z + a];
      r[3 * a] = p.x;
      r[3 * a + 1] = p.y;
      r[3 * a + 2] = p.z;
    }
    IntraOut o = molecule_intra(P, mi.y, b, t, r, cbmc != 0);
    if (o.overlap) {
      atomicOr(ovflag, 1);
      continue;
    }
    v[0] += o.bond;
    v[1] += o.angle;
    v[2] += o.dih;
    v[3] += o.imp;
    v[4] += o.ivdw;
    v[5] += o.iqq;
    v[6] += o.pqq;
  }
  reduce_partials<7>(v, partial, counter, out, nullptr, 0);
}

// ---------------------------------------------------------------------------
// Ewald structure factors.  kvec[k] = (hx, hy, hz, Cn).
constexpr int kSfacMolChunk = 64;

// F32: the mixed path's FP32 phases (a molecule's sums in FP32, stored and
// accumulated in FP64), as its MC moves compute the rows of moved molecules
template <bool F32>
__global__ void __launch_bounds__(128) k_sfac(const double4_32a* __restrict__ kvec, int nv, const double4_32a* __restrict__ p64,
                                              const MolInfo* __restrict__ mols, int nm, const int* __restrict__ charged,
                                              double* cos_mol, double* sin_mol, int stride, double2* part) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  int m0 = blockIdx.y * kSfacMolChunk, m1 = min(nm, m0 + kSfacMolChunk);
  if (k >= nv) return;
  double4_32a h = kvec[k];
  const float hx = (float)h.x, hy = (float)h.y, hz = (float)h.z;
  double cs = 0.0, sn = 0.0;
  for (int m = m0; m < m1; ++m) {
    MolInfo mi = mols[m];
    if (!charged[mi.y]) continue;
    double c = 0.0, s = 0.0;
    if (F32) {
      float cf = 0.0f, sf = 0.0f;
      for (int a = 0; a < mi.w; ++a) {
        double4_32a p = p64[mi.z + a];
        float sv, cv;
        sincosf(hx * (float)p.x + hy * (float)p.y + hz * (float)p.z, &sv, &cv);
        cf += (float)p.w * cv;
        sf += (float)p.w * sv;
      }
      c = (double)cf;
      s = (double)sf;
    } else
    for (int a = 0; a < mi.w; ++a) {
      double4_32a p = p64[mi.z + a];
      double hdotr = h.x * p.x + h.y * p.y + h.z * p.z;
      double sv, cv;
      sincos(hdotr, &sv, &cv);
      c = c + p.w * cv;
      s = s + p.w * sv;
    }
    cos_mol[(size_t)mi.x * stride + k] = c;
    sin_mol[(size_t)mi.x * stride + k] = s;
    cs += c;
    sn += s;
  }
  part[(size_t)blockIdx.y * nv + k] = make_double2(cs, sn);
}

// FP64 rebuild of the molecule rows along k-vector rows: thread per (row,
// molecule); a sincos per atom at the row's start and for its step
// e^{i 2 pi x / Lx}, then one complex product per k-vector and atom
constexpr int kSfacRowAtoms = 4;  // molecules of up to this many atoms
__global__ void __launch_bounds__(128) k_sfac_rows(const double4_32a* __restrict__ kvec, const int2* __restrict__ rows,
                                                   int nrows, double hx1, const double4_32a* __restrict__ p64,
                                                   const MolInfo* __restrict__ mols, int nm,
                                                   const int* __restrict__ charged, double* cos_mol, double* sin_mol,
                                                   int stride) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int2 rw = rows[r];
  const double4_32a h0 = kvec[rw.x];
  for (int m = blockIdx.y; m < nm; m += gridDim.y) {
    const MolInfo mi = mols[m];
    if (!charged[mi.y]) continue;
    double c[kSfacRowAtoms], s[kSfacRowAtoms], uc[kSfacRowAtoms], us[kSfacRowAtoms], q[kSfacRowAtoms];
#pragma unroll
    for (int a = 0; a < kSfacRowAtoms; ++a) {
      c[a] = s[a] = us[a] = q[a] = 0.0;
      uc[a] = 1.0;
      if (a < mi.w) {
        const double4_32a p = p64[mi.z + a];
        sincos(h0.x * p.x + h0.y * p.y + h0.z * p.z, &s[a], &c[a]);
        sincos(hx1 * p.x, &us[a], &uc[a]);
        q[a] = p.w;
      }
    }
    double* cm = cos_mol + (size_t)mi.x * stride + rw.x;
    double* sm = sin_mol + (size_t)mi.x * stride + rw.x;
    for (int j = 0; j < rw.y; ++j) {
      double cs = 0.0, sn = 0.0;
#pragma unroll
      for (int a = 0; a < kSfacRowAtoms; ++a)
        if (a < mi.w) {
          cs = cs + q[a] * c[a];
          sn = sn + q[a] * s[a];
          const double c1 = c[a] * uc[a] - s[a] * us[a];
          s[a] = s[a] * uc[a] + c[a] * us[a];
          c[a] = c1;
        }
      cm[j] = cs;
      sm[j] = sn;
    }
  }
}

// per (molecule chunk, k) sums of the molecule rows (charged species, packed
// order), reduced over the chunks in order by k_sfac_reduce
__global__ void __launch_bounds__(kBlock) k_sfac_sum(int nv, const MolInfo* __restrict__ mols, int nm,
                                                     const int* __restrict__ charged, const double* __restrict__ cos_mol,
                                                     const double* __restrict__ sin_mol, int stride, double2* part) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nv) return;
  const int m0 = blockIdx.y * kSfacMolChunk, m1 = min(nm, m0 + kSfacMolChunk);
  double cs = 0.0, sn = 0.0;
  for (int m = m0; m < m1; ++m) {
    const MolInfo mi = mols[m];
    if (!charged[mi.y]) continue;
    cs += cos_mol[(size_t)mi.x * stride + k];
    sn += sin_mol[(size_t)mi.x * stride + k];
  }
  part[(size_t)blockIdx.y * nv + k] = make_double2(cs, sn);
}

__global__ void __launch_bounds__(kBlock) k_sfac_reduce(const double4_32a* __restrict__ kvec, int nv, const double2* part,
                                                        int nchunks, double* cos_sum, double* sin_sum, double* partial,
                                                        unsigned* counter, double* out) {
  double e = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += gridDim.x * blockDim.x) {
    double c = 0.0, s = 0.0;
    for (int ch = 0; ch < nchunks; ++ch) {
      double2 p = part[(size_t)ch * nv + k];
      c += p.x;
      s += p.y;
    }
    cos_sum[k] = c;
    sin_sum[k] = s;
    e += kvec[k].w * (c * c + s * s);
  }
  double v[1] = {e};
  reduce_partials<1>(v, partial, counter, out, nullptr, 0);
}

// Update_System_Ewald_Reciprocal_Energy: thread per k-vector.
__global__ void __launch_bounds__(kBlock) k_ewald_update(const double4_32a* __restrict__ kvec, int nv,
                                                         const double4_32a* __restrict__ q_atoms, int qn, int move_flag,
                                                         double* cos_sum, double* sin_sum, double* cos_mol,
                                                         double* sin_mol, double* partial, unsigned* counter,
                                                         double* out) {
  double e = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += gridDim.x * blockDim.x) {
    double4_32a h = kvec[k];
    double c = cos_sum[k], s = sin_sum[k];
    if (move_flag == CASS_MOVE_DELETION) {
      c = c - cos_mol[k];
      s = s - sin_mol[k];
    } else {
      double cn = 0.0, sn = 0.0;
      for (int a = 0; a < qn; ++a) {
        double4_32a p = q_atoms[a];
        double hdotr = h.x * p.x + h.y * p.y + h.z * p.z;
        double sv, cv;
        sincos(hdotr, &sv, &cv);
        cn = cn + p.w * cv;
        sn = sn + p.w * sv;
      }
      if (move_flag == CASS_MOVE_INSERTION) {
        c = c + cn;
        s = s + sn;
      } else {
        c = c + (cn - cos_mol[k]);
        s = s + (sn - sin_mol[k]);
      }
      cos_mol[k] = cn;
      sin_mol[k] = sn;
    }
    cos_sum[k] = c;
    sin_sum[k] = s;
    e = e + h.w * (c * c + s * s);
  }
  double v[1] = {e};
  reduce_partials<1>(v, partial, counter, out, nullptr, 0);
}

// Update_System_Ewald_Reciprocal_Energy_Widom: block per test molecule.
__global__ void __launch_bounds__(kBlock) k_ewald_widom(const double4_32a* __restrict__ kvec, int nv,
                                                        const double* __restrict__ cos_sum,
                                                        const double* __restrict__ sin_sum, const double* __restrict__ xyz,
                                                        const double* __restrict__ q, int na, double* out) {
  __shared__ double sh[32];
  const double* r = xyz + (size_t)blockIdx.x * 3 * na;
  double e = 0.0;
  for (int k = threadIdx.x; k < nv; k += blockDim.x) {
    double4_32a h = kvec[k];
    double dc = 0.0, ds = 0.0;
    for (int a = 0; a < na; ++a) {
      double hdotr = h.x * r[3 * a] + h.y * r[3 * a + 1] + h.z * r[3 * a + 2];
      double sv, cv;
      sincos(hdotr, &sv, &cv);
      dc += q[a] * cv;
      ds += q[a] * sv;
    }
    double c = cos_sum[k] + dc, s = sin_sum[k] + ds;
    e = e + h.w * (c * c + s * s);
  }
  e = block_sum(e, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = e * kCHARGE_FACTOR;
}

// Compute_Atom_Nonbond_Intra_Energy for one trial configuration per thread
__global__ void k_atom_intra(BoxDev b, PairTable t, SpeciesPools P, int is0, int ia, const double* __restrict__ xyz,
                             int natoms, unsigned exist, int ntrial, int cbmc, double* e, int* ov) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ntrial) return;
  double eiv, eiq, eoq;
  const bool o = atom_intra(P.hdr[is0], P, b, t, ia, xyz + (size_t)k * natoms * 3, exist, eiv, eiq, eoq, cbmc != 0);
  e[3 * k] = o ? 0.0 : eiv;
  e[3 * k + 1] = o ? 0.0 : eiq;
  e[3 * k + 2] = o ? 0.0 : eoq;
  ov[k] = o ? 1 : 0;
}

// ---------------------------------------------------------------------------
// host helpers

static int ensure_scratch(cass_ctx* c, int nblocks, int nv) {
  int rc = c->d_partial.reserve((size_t)nblocks * nv * sizeof(double));
  if (rc) return rc;
  if (!c->d_counter.p) {
    rc = c->d_counter.reserve(64);
    if (rc) return rc;
    CASS_CUDA(cudaMemsetAsync(c->d_counter.p, 0, 64, c->stream));
  }
  rc = c->d_result.reserve(64 * sizeof(double));
  return rc;
}

static int species_pool_upload(cass_ctx* c, DevBuf& d_hdr, DevBuf& d_ip, DevBuf& d_dp, SpeciesPools& P) {
  std::vector<SpeciesDevHdr> hdr(c->nspecies);
  std::vector<int> ip;
  std::vector<double> dp;
  for (int is = 0; is < c->nspecies; ++is) {
    const SpeciesH& s = c->sp[is];
    SpeciesDevHdr& h = hdr[is];
    memset(&h, 0, sizeof(h));
    h.natoms = s.natoms;
    h.has_charge = s.has_charge;
    h.l_coul_cbmc = s.l_coul_cbmc;
    h.type_off = (int)ip.size();
    ip.insert(ip.end(), s.type.begin(), s.type.end());
    h.bonded_off = (int)ip.size();
    ip.insert(ip.end(), s.bonded.begin(), s.bonded.end());
    h.q_off = (int)dp.size();
    dp.insert(dp.end(), s.q.begin(), s.q.end());
    h.mass_off = (int)dp.size();
    dp.insert(dp.end(), s.mass.begin(), s.mass.end());
    h.vs_off = (int)dp.size();
    dp.insert(dp.end(), s.vscale.begin(), s.vscale.end());
    h.qs_off = (int)dp.size();
    dp.insert(dp.end(), s.qscale.begin(), s.qscale.end());
    h.nbonds = (int)s.bond_kind.size();
    h.bond_atoms_off = (int)ip.size();
    ip.insert(ip.end(), s.bond_atoms.begin(), s.bond_atoms.end());
    h.bond_kind_off = (int)ip.size();
    ip.insert(ip.end(), s.bond_kind.begin(), s.bond_kind.end());
    h.bond_param_off = (int)dp.size();
    dp.insert(dp.end(), s.bond_param.begin(), s.bond_param.end());
    h.nangles = (int)s.angle_kind.size();
    h.angle_atoms_off = (int)ip.size();
    ip.insert(ip.end(), s.angle_atoms.begin(), s.angle_atoms.end());
    h.angle_kind_off = (int)ip.size();
    ip.insert(ip.end(), s.angle_kind.begin(), s.angle_kind.end());
    h.angle_param_off = (int)dp.size();
    dp.insert(dp.end(), s.angle_param.begin(), s.angle_param.end());
    h.ndih = (int)s.dih_atoms.size() / 4;
    h.dih_atoms_off = (int)ip.size();
    ip.insert(ip.end(), s.dih_atoms.begin(), s.dih_atoms.end());
    h.dih_rb_off = (int)dp.size();
    dp.insert(dp.end(), s.dih_rb.begin(), s.dih_rb.end());
    h.nimp = (int)s.imp_atoms.size() / 4;
    h.imp_atoms_off = (int)ip.size();
    ip.insert(ip.end(), s.imp_atoms.begin(), s.imp_atoms.end());
    h.imp_param_off = (int)dp.size();
    dp.insert(dp.end(), s.imp_param.begin(), s.imp_param.end());
  }
  ip.push_back(0);
  dp.push_back(0.0);
  int rc = d_hdr.reserve(hdr.size() * sizeof(SpeciesDevHdr));
  if (!rc) rc = d_ip.reserve(ip.size() * sizeof(int));
  if (!rc) rc = d_dp.reserve(dp.size() * sizeof(double));
  if (rc) return rc;
  CASS_CUDA(h2d(c, d_hdr.p, hdr.data(), hdr.size() * sizeof(SpeciesDevHdr)));
  CASS_CUDA(h2d(c, d_ip.p, ip.data(), ip.size() * sizeof(int)));
  CASS_CUDA(h2d(c, d_dp.p, dp.data(), dp.size() * sizeof(double)));
  P.hdr = d_hdr.as<SpeciesDevHdr>();
  P.ip = d_ip.as<int>();
  P.dp = d_dp.as<double>();
  return CASS_OK;
}

int ensure_pools(cass_ctx* c) {
  if (!c->pools_dirty) return CASS_OK;
  int rc = species_pool_upload(c, c->d_sp_hdr, c->d_sp_ip, c->d_sp_dp, c->pools);
  if (!rc) c->pools_dirty = false;
  return rc;
}

}  // namespace cassgpu

using namespace cassgpu;

namespace cassgpu {
// One upload of a frame load: `bytes` (a multiple of 16) from offset `src` of
// the staged frame to the device array `dst`
struct StageCopy {
  long long src, bytes;
  void* dst;
  long long pad;
};

// Copies of a frame load out of the device copy of the staging area, one CTA
// per copy, 16-byte words
__global__ void k_stage_scatter(const unsigned char* stage, const StageCopy* cp) {
  const StageCopy d = cp[blockIdx.x];
  const uint4* s = reinterpret_cast<const uint4*>(stage + d.src);
  uint4* t = reinterpret_cast<uint4*>(d.dst);
  for (long long i = threadIdx.x; i < d.bytes / 16; i += blockDim.x) t[i] = s[i];
}

}  // namespace cassgpu

namespace {

int set_device(cass_ctx* c) {
  CASS_CUDA(cudaSetDevice(c->device));
  return CASS_OK;
}

int check_mol(cass_ctx* c, int im, int is) {
  if (is < 1 || is > c->nspecies) return set_error(CASS_EINVAL, "species index out of range");
  if (im < 1 || im > c->max_mol[is - 1]) return set_error(CASS_EINVAL, "molecule locate out of range");
  if (!c->sp[is - 1].defined) return set_error(CASS_ESTATE, "species not defined");
  return CASS_OK;
}

int mol_slot(cass_ctx* c, int im, int is) { return c->mol_base[is - 1] + im - 1; }

void invalidate(cass_ctx* c, int ibox) {
  if (ibox < 0 || ibox >= c->nboxes) return;
  c->box[ibox].energy_valid = false;
  c->box[ibox].frame_ready = false;
  c->box[ibox].pack_dirty = true;
  c->box[ibox].cell_dirty = true;
}

// live molecule slots of a box, species-major and in locate order
const std::vector<int>& members(cass_ctx* c, int ibox) {
  if (c->members_dirty) {
    for (auto& m : c->box_members) m.clear();
    c->box_members.resize(c->nboxes);
    for (int slot = 0; slot < c->nmol_slots; ++slot) {
      int b = c->mol_box[slot];
      if (b >= 0 && c->sp[c->slot_sp[slot]].defined) c->box_members[b].push_back(slot);
    }
    c->members_dirty = false;
  }
  return c->box_members[ibox];
}

void set_mol_box(cass_ctx* c, int slot, int ibox) {
  if (c->mol_box[slot] != ibox) c->members_dirty = true;
  c->mol_box[slot] = ibox;
}

// Bytes of pinned staging that packing box ibox needs.
size_t pack_bytes(cass_ctx* c, int ibox) {
  const std::vector<int>& mem = members(c, ibox);
  size_t na = 0;
  for (int slot : mem) na += (size_t)c->sp[c->slot_sp[slot]].natoms;
  const size_t n = std::max<size_t>(1, na), m = std::max<size_t>(1, mem.size());
  return (n * (sizeof(double4_32a) + sizeof(float4) + sizeof(int4)) + m * sizeof(int4) + 255) & ~(size_t)255;
}

// Packs the live molecules of a box (species-major, locate order) into pinned
// staging at `stage` (pack_bytes long) and queues the uploads (or, with
// `defer`, lists them for one upload of the whole staging area); the caller
// synchronizes before the staging is reused.
int pack_box_async(cass_ctx* c, int ibox, unsigned char* stage, std::vector<cassgpu::StageCopy>* defer = nullptr,
                   const unsigned char* base = nullptr) {
  BoxH& B = c->box[ibox];
  const std::vector<int>& mem = members(c, ibox);
  size_t na = 0;
  for (int slot : mem) na += (size_t)c->sp[c->slot_sp[slot]].natoms;
  const size_t nm = mem.size();
  const size_t n = std::max<size_t>(1, na), m = std::max<size_t>(1, nm);
  int rc = B.d_p64.reserve(n * sizeof(double4_32a));
  if (!rc) rc = B.d_p32.reserve(n * sizeof(float4));
  if (!rc) rc = B.d_meta.reserve(n * sizeof(int4));
  if (!rc) rc = B.d_molinfo.reserve(m * sizeof(int4));
  if (rc) return rc;
  double4_32a* p64 = reinterpret_cast<double4_32a*>(stage);
  float4* p32 = reinterpret_cast<float4*>(p64 + na);
  int4* meta = reinterpret_cast<int4*>(p32 + na);
  int4* molinfo = meta + na;
  B.pk_mol.clear();
  B.pk_mol_off.clear();
  int k = 0;
  for (int slot : mem) {
    const int is = c->slot_sp[slot], im = slot - c->mol_base[is];
    const SpeciesH& s = c->sp[is];
    c->pk_index[slot] = (int)B.pk_mol.size();
    molinfo[B.pk_mol.size()] = make_int4(slot, is, k, s.natoms);
    B.pk_mol.push_back(slot);
    B.pk_mol_off.push_back(k);
    const double* r = &s.pos[(size_t)im * 3 * s.natoms];
    for (int a = 0; a < s.natoms; ++a, ++k) {
      p64[k] = make_double4_32a(r[3 * a], r[3 * a + 1], r[3 * a + 2], s.q[a]);
      float tf;
      int ty = s.type[a];
      memcpy(&tf, &ty, sizeof(float));
      p32[k] = make_float4((float)r[3 * a], (float)r[3 * a + 1], (float)r[3 * a + 2], tf);
      meta[k] = make_int4(slot, s.type[a], is, a);
    }
  }
  B.npacked = (int)na;
  B.npacked_mols = (int)nm;
  if (B.comcut && na > 0) {
    // Get_COM and Compute_Max_Com_Distance (get_com.f90:45-105,220-295) per molecule
    std::vector<double4_32a> com(na);
    for (size_t q = 0; q < nm; ++q) {
      const int4 mi = molinfo[q];
      const SpeciesH& sp = c->sp[mi.y];
      double tm = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
      for (int a = 0; a < mi.w; ++a) {
        const double4_32a& p = p64[mi.z + a];
        tm = tm + sp.mass[a];
        cx = cx + sp.mass[a] * p.x;
        cy = cy + sp.mass[a] * p.y;
        cz = cz + sp.mass[a] * p.z;
      }
      cx = cx / tm;
      cy = cy / tm;
      cz = cz / tm;
      double dmax = 0.0;
      for (int a = 0; a < mi.w; ++a) {
        const double4_32a& p = p64[mi.z + a];
        const double dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
        dmax = std::max(dmax, dx * dx + dy * dy + dz * dz);
      }
      const double4_32a v = make_double4_32a(cx, cy, cz, std::sqrt(dmax));
      for (int a = 0; a < mi.w; ++a) com[mi.z + a] = v;
    }
    if ((rc = B.d_com.reserve(na * sizeof(double4_32a)))) return rc;
    CASS_CUDA(h2d(c, B.d_com.p, com.data(), na * sizeof(double4_32a)));
    CASS_CUDA(cudaStreamSynchronize(c->stream));  // the host vector goes out of scope
  }
  if (na > 0 && defer) {
    auto add = [&](const void* src, void* dst, size_t bytes) {
      defer->push_back(cassgpu::StageCopy{(long long)(static_cast<const unsigned char*>(src) - base), (long long)bytes, dst, 0});
    };
    add(p64, B.d_p64.p, na * sizeof(double4_32a));
    add(p32, B.d_p32.p, na * sizeof(float4));
    add(meta, B.d_meta.p, na * sizeof(int4));
    add(molinfo, B.d_molinfo.p, nm * sizeof(int4));
  } else if (na > 0) {
    CASS_CUDA(h2d(c, B.d_p64.p, p64, na * sizeof(double4_32a)));
    CASS_CUDA(h2d(c, B.d_p32.p, p32, na * sizeof(float4)));
    CASS_CUDA(h2d(c, B.d_meta.p, meta, na * sizeof(int4)));
    CASS_CUDA(h2d(c, B.d_molinfo.p, molinfo, nm * sizeof(int4)));
  }
  B.pack_dirty = false;
  return CASS_OK;
}

// Packs one box through the context's pinned staging buffer.
int pack_box(cass_ctx* c, int ibox) {
  if (!c->box[ibox].pack_dirty) return CASS_OK;
  int rc = c->h_pack.reserve(pack_bytes(c, ibox));
  if (!rc) rc = pack_box_async(c, ibox, static_cast<unsigned char*>(c->h_pack.p));
  if (rc) return rc;
  // the staging buffer is refilled by the next pack: wait for the copies
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  return CASS_OK;
}

int sync_result(cass_ctx* c, int n) {
  c->h_result.resize(n);
  CASS_CUDA(d2h(c, c->h_result.data(), c->d_result.p, n * sizeof(double)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  return CASS_OK;
}

int ensure_cos_mol(cass_ctx* c, int nv) {
  if (nv <= c->cos_mol_stride && c->d_cos_mol.p) return CASS_OK;
  // a quarter more k-vectors than needed, so that volume moves rarely regrow the rows
  int stride = std::max(nv + nv / 4, c->cos_mol_stride);
  if (c->d_cos_mol.p)  // the rows of every molecule are lost: boxes with an Ewald sum must be recomputed
    for (BoxH& B : c->box)
      if (B.desc.charge_style == CASS_CHARGE_COUL && B.desc.charge_sum_style == CASS_QQ_EWALD)
        B.energy_valid = B.frame_ready = false;
  size_t bytes = (size_t)std::max(1, c->nmol_slots) * stride * sizeof(double);
  int rc = c->d_cos_mol.reserve(bytes);
  if (!rc) rc = c->d_sin_mol.reserve(bytes);
  if (!rc) rc = c->d_cos_mol_old.reserve((size_t)stride * sizeof(double));
  if (!rc) rc = c->d_sin_mol_old.reserve((size_t)stride * sizeof(double));
  if (rc) return rc;
  CASS_CUDA(cudaMemsetAsync(c->d_cos_mol.p, 0, bytes, c->stream));
  CASS_CUDA(cudaMemsetAsync(c->d_sin_mol.p, 0, bytes, c->stream));
  c->cos_mol_stride = stride;
  return CASS_OK;
}

bool box_has_ewald(const BoxH& b) {
  return b.desc.charge_style == CASS_CHARGE_COUL && b.desc.charge_sum_style == CASS_QQ_EWALD;
}

// Compute_LR_Correction (energy_routines.f90:2956-3023), host FP64 (O(ntypes^2)).
double lr_correction(cass_ctx* c, const BoxH& B, const std::vector<double>& nb) {
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
        double eps = c->pt.eps[k], sig = std::sqrt(c->pt.sig2[k]), n = c->pt.mie_n[k], m = c->pt.mie_m[k];
        double sor = sig / B.desc.rcut_vdw;
        eij = eij + nb[ja] * c->pt.mie_c[k] * eps * std::pow(B.desc.rcut_vdw, 3.0) *
                        ((std::pow(sor, n) / (3.0 - n)) + (std::pow(sor, m) / (m - 3.0)));
      }
      e = e + nb[ia] * eij;
    }
    e = -2.0 * kPI * e / B.dev.volume;
  }
  return e;
}

std::vector<double> count_beads(cass_ctx* c, int ibox) {
  std::vector<double> nb(c->ntypes, 0.0);
  for (int slot : members(c, ibox)) {
    const SpeciesH& s = c->sp[c->slot_sp[slot]];
    for (int a = 0; a < s.natoms; ++a)
      if (s.type[a] >= 0) nb[s.type[a]] += 1.0;
  }
  return nb;
}

}  // namespace

namespace cassgpu {
int pack_box_ext(cass_ctx* c, int ibox) { return pack_box(c, ibox); }
void invalidate_ext(cass_ctx* c, int ibox) { invalidate(c, ibox); }
void set_mol_box_ext(cass_ctx* c, int slot, int ibox) { set_mol_box(c, slot, ibox); }
const std::vector<int>& members_ext(cass_ctx* c, int ibox) { return members(c, ibox); }

namespace {
// AtomPair_VdW_Energy_Vector (energy_routines.f90:1733-1829) at r^2 = rsq:
// the box's vdW pair energy without a cutoff test
double table_vdw(const cass_ctx_impl* c, const BoxDev& b, int it, int jt, double rsq) {
  const PairTable& t = c->pt;
  const int k = it * t.ntypes + jt;
  const double eps = t.eps[k];
  if (b.vdw_style == CASS_VDW_LJ) {
    const double s2 = t.sig2[k] / rsq, s6 = s2 * s2 * s2, s12 = s6 * s6;
    double e = 4.0 * eps * (s12 - s6);
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
      const double c2 = t.sig2[k] / b.rcut_vdwsq, c6 = c2 * c2 * c2, c12 = c6 * c6;
      e = e - 4.0 * eps * (c12 - c6);
    } else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) {
      if (rsq >= b.ron_switch_sq) {
        if (rsq > b.roff_switch_sq) {
          e = 0.0;
        } else {
          const double d = b.roff_switch_sq - rsq;
          e = d * d * (b.switch_factor2 + 2.0 * rsq) * b.switch_factor1 * e;
        }
      }
    } else if (b.vdw_sum_style == CASS_VDW_SUM_CHARMM) {
      e = eps * (s12 - 2.0 * s6);
    } else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT_FORCE) {
      const double c2 = t.sig2[k] / b.rcut_vdwsq, c6 = c2 * c2 * c2, c12 = c6 * c6;
      const double rc = std::sqrt(b.rcut_vdwsq);
      const double dedr = -24.0 * eps * (2.0 * c12 - c6) / rc;
      e = e - 4.0 * eps * (c12 - c6) - (std::sqrt(rsq) - rc) * dedr;
    }
    return e;
  }
  if (b.vdw_style == CASS_VDW_MIE) {
    const double sig = c->pt_sig[k], n = t.mie_n[k], m = t.mie_m[k], rc = std::sqrt(b.rcut_vdwsq);
    const double sr = sig / std::sqrt(rsq);
    double e = t.mie_c[k] * eps * (std::pow(sr, n) - std::pow(sr, m));
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
      const double sc = sig / rc;
      e = e - t.mie_c[k] * eps * (std::pow(sc, n) - std::pow(sc, m));
    }
    return e;
  }
  return 0.0;
}
}  // namespace

// The tables of the CBMC options: r_min^2 per type pair
// (create_nonbond_table.f90:219-220, 285-303, 396-418, with the charge range of
// each type of :144-153) and, per box, the atom-pair energy table
// (atompair_nrg_table_routines.f90:149-261; rsq_step and rsq_shifter of
// :163-168).  One device buffer: r_min^2 (FP64, FP32), then per box the vdW
// part [ntypes][ntypes][res] and the Coulomb kernel [res] in FP64 and FP32.
int ensure_cbmc(cass_ctx_impl* c) {
  const CassCBMCOptions& o = c->cbmc_opt;
  const bool on = o.energy_table_res > 0 || o.sector_overlap;
  if (!on) {
    for (BoxH& B : c->box) {
      B.dev.tab_res = 0;
      B.dev.sector = 0;
    }
    return CASS_OK;
  }
  if (!c->cbmc_dirty) return CASS_OK;
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  const int nt = c->ntypes, res = o.energy_table_res;
  double rlow = -1.0, max_cbmcsq = 0.0, min_beta = 0.0;
  int charge_style1 = CASS_CHARGE_NONE, nbox = 0;
  for (int ib = 0; ib < c->nboxes; ++ib) {
    const BoxH& B = c->box[ib];
    if (!B.defined) continue;
    if (nbox == 0) {
      rlow = B.dev.rcut_lowsq;
      min_beta = B.dev.beta;
    } else if (B.dev.rcut_lowsq != rlow) {
      return set_error(CASS_EUNSUPPORTED, "CBMC options need one rcut_low for all boxes");
    }
    if (ib == 0) charge_style1 = B.desc.charge_style;
    max_cbmcsq = std::max(max_cbmcsq, B.dev.rcut_cbmcsq);
    min_beta = std::min(min_beta, B.dev.beta);
    ++nbox;
  }
  if (nbox == 0) return set_error(CASS_ESTATE, "CBMC options need a box");
  std::vector<double> rmin((size_t)nt * nt, rlow);
  if (o.rmin_u_max > 0.0) {
    std::vector<double> qmin(nt, 0.0), qmax(nt, 0.0);
    std::vector<char> seen(nt, 0);
    for (const SpeciesH& sp : c->sp) {
      if (!sp.defined) continue;
      for (int a = 0; a < sp.natoms; ++a) {
        const int t = sp.type[a];
        if (t < 0) continue;
        qmin[t] = seen[t] ? std::min(qmin[t], sp.q[a]) : sp.q[a];
        qmax[t] = seen[t] ? std::max(qmax[t], sp.q[a]) : sp.q[a];
        seen[t] = 1;
      }
    }
    const double u_base = o.rmin_u_max / min_beta, rcut_low = std::sqrt(rlow);
    for (int i = 0; i < nt; ++i)
      for (int j = 0; j < nt; ++j) {
        const double eps = c->pt.eps[i * nt + j], sig = c->pt_sig[i * nt + j];
        if (!(eps > 0.0)) continue;
        double min_uq = 0.0;
        if (charge_style1 != CASS_CHARGE_NONE) {
          double qp = std::min(qmin[i] * qmax[j], qmax[i] * qmin[j]);
          if (qp <= 0.0) {
            min_uq = qp * kCHARGE_FACTOR / rcut_low;
          } else {
            qp = std::min(qmin[i] * qmin[j], qmax[i] * qmax[j]);
            min_uq = qp * kCHARGE_FACTOR / sig;
          }
        }
        const double umax = std::max(u_base - min_uq, 0.0);
        const double lambda = 0.5 * (1.0 + std::sqrt(1.0 + umax / eps));
        rmin[(size_t)i * nt + j] = sig * sig / std::pow(lambda, 1.0 / 3.0);
      }
  }
  if (o.sector_overlap)
    for (const BoxH& B : c->box)
      if (B.defined)
        for (double r2 : rmin)
          if (r2 > B.dev.rcut_cbmcsq) return set_error(CASS_EUNSUPPORTED, "r_min exceeds rcut_cbmc");
  // host image of the device buffer
  const size_t nn = (size_t)nt * nt;
  const size_t per_box = res > 0 ? (nn * res + res) * (sizeof(double) + sizeof(float)) : 0;
  const size_t head = ((nn * (sizeof(double) + sizeof(float)) + 255) & ~(size_t)255);
  const size_t box_stride = (per_box + 255) & ~(size_t)255;
  std::vector<unsigned char> img(head + box_stride * c->nboxes, 0);
  double* h_rmin = reinterpret_cast<double*>(img.data());
  float* h_rminf = reinterpret_cast<float*>(h_rmin + nn);
  for (size_t k = 0; k < nn; ++k) {
    h_rmin[k] = rmin[k];
    h_rminf[k] = (float)rmin[k];
  }
  std::vector<double> step(c->nboxes, 0.0), shift(c->nboxes, 0.0);
  if (res > 0)
    for (int ib = 0; ib < c->nboxes; ++ib) {
      const BoxH& B = c->box[ib];
      if (!B.defined) continue;
      const BoxDev& b = B.dev;
      double* v = reinterpret_cast<double*>(img.data() + head + box_stride * ib);
      double* f2 = v + nn * res;
      float* vf = reinterpret_cast<float*>(f2 + res);
      float* f2f = vf + nn * res;
      step[ib] = (max_cbmcsq - rlow) / res;
      shift[ib] = rlow - step[ib];
      for (int i = 1; i <= res; ++i) {
        const double mp = (shift[ib] + step[ib] * i) + 0.5 * step[ib];
        const double rij = std::sqrt(mp);
        double k2 = 0.0;
        if (b.charge_style == CASS_CHARGE_COUL) {
          if (b.charge_sum_style == CASS_QQ_EWALD) k2 = std::erfc(b.alpha * rij) / rij;
          else if (b.charge_sum_style == CASS_QQ_DSF)
            k2 = b.dsf_factor2 * (rij - b.rcut_coul) - b.dsf_factor1 + std::erfc(b.alpha_dsf * rij) / rij;
          else if (b.charge_sum_style == CASS_QQ_CUT) k2 = 1.0 / rij;
        }
        f2[i - 1] = k2;
        f2f[i - 1] = (float)k2;
        for (int ti = 0; ti < nt; ++ti)
          for (int tj = 0; tj < nt; ++tj) {
            const double e = table_vdw(c, b, ti, tj, mp);
            v[((size_t)ti * nt + tj) * res + (i - 1)] = e;
            vf[((size_t)ti * nt + tj) * res + (i - 1)] = (float)e;
          }
      }
    }
  CASS_CUDA(cudaSetDevice(c->device));
  if (int rc = c->d_cbmc_tab.reserve(img.size())) return rc;
  CASS_CUDA(h2d(c, c->d_cbmc_tab.p, img.data(), img.size()));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  unsigned char* base = static_cast<unsigned char*>(c->d_cbmc_tab.p);
  for (int ib = 0; ib < c->nboxes; ++ib) {
    BoxDev& b = c->box[ib].dev;
    b.sector = o.sector_overlap ? 1 : 0;
    b.rminsq = reinterpret_cast<const double*>(base);
    b.rminsqf = reinterpret_cast<const float*>(base + nn * sizeof(double));
    b.tab_res = (res > 0 && c->box[ib].defined) ? res : 0;
    b.tab_step = step[ib];
    b.tab_shift = shift[ib];
    const double* v = reinterpret_cast<const double*>(base + head + box_stride * ib);
    b.tab_v = v;
    b.tab_f2 = v + nn * res;
    b.tab_vf = reinterpret_cast<const float*>(b.tab_f2 + res);
    b.tab_f2f = b.tab_vf + nn * res;
  }
  c->cbmc_dirty = false;
  return CASS_OK;
}
}  // namespace cassgpu

// ===========================================================================
// exported entry points
extern "C" {

int cass_abi_version(void) { return CASS_ABI_VERSION; }
const char* cass_last_error(void) { return g_err.c_str(); }

int cass_ctx_create(const CassConfig* cfg, cass_ctx** out) {
  if (!cfg || !out || cfg->nspecies < 1 || cfg->ntypes < 1 || cfg->ntypes > kMaxTypes || cfg->nboxes < 1 ||
      !cfg->max_molecules)
    return set_error(CASS_EINVAL, "bad config (ntypes must be 1..8)");
  if (cfg->precision != CASS_PREC_FP64 && cfg->precision != CASS_PREC_MIXED)
    return set_error(CASS_EINVAL, "bad precision");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev < 1) return set_error(CASS_ECUDA, "no CUDA device available");
  if (cfg->device < 0 || cfg->device >= ndev) return set_error(CASS_EINVAL, "device ordinal out of range");
  cass_ctx* c = new cass_ctx();
  c->device = cfg->device;
  c->precision = cfg->precision;
  c->nspecies = cfg->nspecies;
  c->ntypes = cfg->ntypes;
  c->nboxes = cfg->nboxes;
  if (cfg->max_kvectors > 0) c->max_kvec = cfg->max_kvectors;
  c->max_mol.assign(cfg->max_molecules, cfg->max_molecules + cfg->nspecies);
  c->mol_base.resize(c->nspecies);
  int tot = 0;
  for (int i = 0; i < c->nspecies; ++i) {
    if (c->max_mol[i] < 0) {
      delete c;
      return set_error(CASS_EINVAL, "negative max_molecules");
    }
    c->mol_base[i] = tot;
    tot += c->max_mol[i];
  }
  c->nmol_slots = tot;
  c->mol_box.assign(tot, -1);
  c->pk_index.assign(tot, -1);
  c->slot_sp.resize(tot);
  for (int i = 0; i < c->nspecies; ++i)
    for (int m = 0; m < c->max_mol[i]; ++m) c->slot_sp[c->mol_base[i] + m] = i;
  c->sp.resize(c->nspecies);
  c->box.resize(c->nboxes);
  if (cudaSetDevice(c->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return set_error(CASS_ECUDA, "stream creation failed");
  }
  c->stream = c->own_stream;
  for (int k = 0; k < 4; ++k)
    if (cudaEventCreate(&c->ev[k]) != cudaSuccess) {
      delete c;
      return set_error(CASS_ECUDA, "event creation failed");
    }
  *out = c;
  return CASS_OK;
}

int cass_ctx_destroy(cass_ctx* c) {
  if (!c) return CASS_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& s : c->sp) {
    s.d_library.release();
    s.d_library_f.release();
  }
  c->box.clear();
  for (int k = 0; k < 4; ++k)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  cudaStreamDestroy(c->own_stream);
  delete c;
  return CASS_OK;
}

int cass_get_stats(cass_ctx* c, CassStats* out) {
  if (!c || !out) return set_error(CASS_EINVAL, "NULL argument");
  *out = c->stats;
  return CASS_OK;
}

int cass_set_count_pairs(cass_ctx* c, int32_t on) {
  if (!c) return set_error(CASS_EINVAL, "NULL context");
  c->count_pairs = on ? 1 : 0;
  return CASS_OK;
}

int cass_set_widom_autotune(cass_ctx* c, int32_t on) {
  if (!c) return set_error(CASS_EINVAL, "NULL context");
  c->widom_autotune = on != 0;
  return CASS_OK;
}

int cass_set_widom_cells(cass_ctx* c, double cells_per_cutoff) {
  if (!c || !(cells_per_cutoff >= 0.0 && cells_per_cutoff <= 8.0))
    return set_error(CASS_EINVAL, "cells_per_cutoff must be in [0, 8]");
  c->widom_cells = cells_per_cutoff;
  return CASS_OK;
}

int cass_set_widom_band(cass_ctx* c, double scale) {
  if (!c || !(scale >= 1.0 && scale <= 1.0e4)) return set_error(CASS_EINVAL, "scale must be in [1, 1e4]");
  c->widom_band = scale;
  return CASS_OK;
}

int cass_set_mc_cluster(cass_ctx* c, int32_t ctas) {
  if (!c || ctas < 0 || ctas > 8) return set_error(CASS_EINVAL, "ctas must be in [0, 8]");
  c->mc_cluster = ctas;
  return CASS_OK;
}

int cass_set_stream(cass_ctx* c, void* stream) {
  if (!c) return set_error(CASS_EINVAL, "NULL context");
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return CASS_OK;
}

int cass_set_nonbond_table(cass_ctx* c, int32_t nt, const double* eps, const double* sig, const double* mn,
                           const double* mm) {
  if (!c || nt != c->ntypes || !eps || !sig) return set_error(CASS_EINVAL, "bad nonbond table");
  PairTable& t = c->pt;
  memset(&t, 0, sizeof(t));
  t.ntypes = nt;
  for (int i = 0; i < nt * nt; ++i) {
    t.eps[i] = eps[i];
    t.sig2[i] = sig[i] * sig[i];
    t.mie_n[i] = mn ? mn[i] : 0.0;
    t.mie_m[i] = mm ? mm[i] : 0.0;
    double n = t.mie_n[i], m = t.mie_m[i];
    t.mie_c[i] = (n > m && m > 0) ? n / (n - m) * std::pow(n / m, m / (n - m)) : 0.0;
    t.epsf[i] = (float)t.eps[i];
    t.sig2f[i] = (float)t.sig2[i];
  }
  c->pt_set = true;
  c->pt_sig.assign(sig, sig + nt * nt);
  c->cbmc_dirty = true;
  for (int b = 0; b < c->nboxes; ++b) c->box[b].energy_valid = c->box[b].frame_ready = false;
  return CASS_OK;
}

int cass_set_species(cass_ctx* c, int32_t is, const CassSpeciesDesc* d) {
  if (!c || is < 1 || is > c->nspecies || !d || d->natoms < 1) return set_error(CASS_EINVAL, "bad species");
  if (!d->atom_type || !d->charge || !d->mass || !d->vdw_intra_scale || !d->charge_intra_scale || !d->bonded)
    return set_error(CASS_EINVAL, "species arrays missing");
  if (d->natoms > 64) return set_error(CASS_ECAPACITY, "species with more than 64 atoms");
  if (d->nfragments > 0 && (!d->frag_natoms || !d->frag_atoms || !d->frag_nconnect || !d->frag_nconfig))
    return set_error(CASS_EINVAL, "fragment arrays missing");
  {  // every 1-based index of the descriptor must name an atom / fragment of this species
    const int n = d->natoms;
    auto bad = [&](const int32_t* a, long cnt, int hi) {
      for (long k = 0; k < cnt; ++k)
        if (a[k] < 1 || a[k] > hi) return true;
      return false;
    };
    if ((d->nbonds > 0 && (!d->bond_atoms || bad(d->bond_atoms, 2L * d->nbonds, n))) ||
        (d->nangles > 0 && (!d->angle_atoms || bad(d->angle_atoms, 3L * d->nangles, n))) ||
        (d->ndihedrals > 0 && (!d->dihedral_atoms || bad(d->dihedral_atoms, 4L * d->ndihedrals, n))) ||
        (d->nimpropers > 0 && (!d->improper_atoms || bad(d->improper_atoms, 4L * d->nimpropers, n))))
      return set_error(CASS_EINVAL, "bonded atom index out of range");
    long nfa = 0, nfc = 0;
    for (int f = 0; f < d->nfragments; ++f) {
      if (d->frag_natoms[f] < 1 || d->frag_natoms[f] > n || d->frag_nconnect[f] < 0 || d->frag_nconfig[f] < 0)
        return set_error(CASS_EINVAL, "bad fragment sizes");
      nfa += d->frag_natoms[f];
      nfc += d->frag_nconnect[f];
    }
    if (bad(d->frag_atoms, nfa, n) || (nfc > 0 && (!d->frag_connect || bad(d->frag_connect, nfc, d->nfragments))))
      return set_error(CASS_EINVAL, "fragment atom / connection index out of range");
  }
  SpeciesH& s = c->sp[is - 1];
  int n = d->natoms;
  s.natoms = n;
  s.type.resize(n);
  for (int i = 0; i < n; ++i) {
    s.type[i] = d->atom_type[i] - 1;
    if (s.type[i] >= c->ntypes) return set_error(CASS_EINVAL, "atom type out of range");
  }
  s.q.assign(d->charge, d->charge + n);
  s.mass.assign(d->mass, d->mass + n);
  s.vscale.assign(d->vdw_intra_scale, d->vdw_intra_scale + n * n);
  s.qscale.assign(d->charge_intra_scale, d->charge_intra_scale + n * n);
  s.bonded.assign(d->bonded, d->bonded + n * n);
  s.bond_atoms.clear(); s.bond_kind.clear(); s.bond_param.clear();
  for (int k = 0; k < d->nbonds; ++k) {
    s.bond_atoms.push_back(d->bond_atoms[2 * k] - 1);
    s.bond_atoms.push_back(d->bond_atoms[2 * k + 1] - 1);
    s.bond_kind.push_back(d->bond_kind[k]);
    s.bond_param.push_back(d->bond_param[2 * k]);
    s.bond_param.push_back(d->bond_param[2 * k + 1]);
  }
  s.angle_atoms.clear(); s.angle_kind.clear(); s.angle_param.clear();
  for (int k = 0; k < d->nangles; ++k) {
    for (int j = 0; j < 3; ++j) s.angle_atoms.push_back(d->angle_atoms[3 * k + j] - 1);
    s.angle_kind.push_back(d->angle_kind[k]);
    s.angle_param.push_back(d->angle_param[2 * k]);
    s.angle_param.push_back(d->angle_param[2 * k + 1]);
  }
  s.dih_atoms.clear(); s.dih_rb.clear();
  for (int k = 0; k < d->ndihedrals; ++k) {
    for (int j = 0; j < 4; ++j) s.dih_atoms.push_back(d->dihedral_atoms[4 * k + j] - 1);
    for (int j = 0; j < 6; ++j) s.dih_rb.push_back(d->dihedral_rb[6 * k + j]);
  }
  s.imp_atoms.clear(); s.imp_param.clear();
  for (int k = 0; k < d->nimpropers; ++k) {
    for (int j = 0; j < 4; ++j) s.imp_atoms.push_back(d->improper_atoms[4 * k + j] - 1);
    s.imp_param.push_back(d->improper_param[2 * k]);
    s.imp_param.push_back(d->improper_param[2 * k + 1]);
  }
  s.nfrag = d->nfragments;
  s.frag_atoms.clear(); s.frag_connect.clear(); s.frag_nconfig.clear(); s.library.clear(); s.lib_off.clear();
  s.prob_ins.clear(); s.cum_prob_ins.clear();
  int off = 0, coff = 0, tot = 0;
  size_t loff = 0;
  for (int f = 0; f < s.nfrag; ++f) {
    std::vector<int> at;
    for (int j = 0; j < d->frag_natoms[f]; ++j) at.push_back(d->frag_atoms[off + j] - 1);
    off += d->frag_natoms[f];
    s.frag_atoms.push_back(at);
    std::vector<int> cn;
    for (int j = 0; j < d->frag_nconnect[f]; ++j) cn.push_back(d->frag_connect[coff + j] - 1);
    coff += d->frag_nconnect[f];
    s.frag_connect.push_back(cn);
    s.frag_nconfig.push_back(d->frag_nconfig[f]);
    size_t len = (size_t)d->frag_nconfig[f] * d->frag_natoms[f] * 3;
    s.lib_off.push_back((int)s.library.size());
    if (len && d->frag_library) s.library.insert(s.library.end(), d->frag_library + loff, d->frag_library + loff + len);
    loff += len;
    tot += d->frag_natoms[f];
  }
  int acc = 0;
  for (int f = 0; f < s.nfrag; ++f) {  // input_routines.f90:2844-2848
    s.prob_ins.push_back((double)d->frag_natoms[f] / (double)tot);
    acc += d->frag_natoms[f];
    s.cum_prob_ins.push_back(f == 0 ? s.prob_ins[0] : (double)acc / (double)tot);
  }
  s.l_coul_cbmc = d->l_coul_cbmc != 0;
  s.has_charge = false;
  for (int i = 0; i < n; ++i)
    if (s.q[i] != 0.0) s.has_charge = true;
  s.pos.assign((size_t)c->max_mol[is - 1] * 3 * n, 0.0);
  s.d_library.release();
  s.d_library_f.release();
  if (!s.library.empty()) {
    int rc = s.d_library.reserve(s.library.size() * sizeof(double));
    if (rc) return rc;
    CASS_CUDA(h2d(c, s.d_library.p, s.library.data(), s.library.size() * sizeof(double)));
    // FP32 copy read by the mixed-precision Widom kernel
    std::vector<float> lf(s.library.begin(), s.library.end());
    if ((rc = s.d_library_f.reserve(lf.size() * sizeof(float)))) return rc;
    CASS_CUDA(h2d(c, s.d_library_f.p, lf.data(), lf.size() * sizeof(float)));
  }
  s.defined = true;
  c->cbmc_dirty = true;
  c->members_dirty = true;
  c->pools_dirty = true;
  for (int b = 0; b < c->nboxes; ++b) invalidate(c, b);
  return CASS_OK;
}

int cass_set_box(cass_ctx* c, int32_t ibox, const CassBoxDesc* d) {
  if (!c || ibox < 1 || ibox > c->nboxes || !d) return set_error(CASS_EINVAL, "bad box");
  for (int k = 0; k < 3; ++k)
    if (!(d->length[k] > 0.0)) return set_error(CASS_EINVAL, "box length must be positive");
  BoxH& B = c->box[ibox - 1];
  B.desc = *d;
  BoxDev& v = B.dev;
  memset(&v, 0, sizeof(v));
  c->cbmc_dirty = true;
  for (int k = 0; k < 3; ++k) {
    v.L[k] = d->length[k];
    v.hL[k] = 0.5 * d->length[k];
    v.Lf[k] = (float)v.L[k];
    v.hLf[k] = (float)v.hL[k];
  }
  v.volume = v.L[0] * v.L[1] * v.L[2];
  v.vdw_style = d->vdw_style;
  v.vdw_sum_style = d->vdw_sum_style;
  v.charge_style = d->charge_style;
  v.charge_sum_style = d->charge_sum_style;
  double rcoul = d->charge_style == CASS_CHARGE_COUL ? d->rcut_coul : 0.0;
  v.rcut_vdw = d->rcut_vdw;
  v.rcut_coul = rcoul;
  v.rcut_vdwsq = d->rcut_vdw * d->rcut_vdw;
  v.rcut_coulsq = rcoul * rcoul;
  v.rcut_cbmcsq = d->rcut_cbmc * d->rcut_cbmc;
  v.rcut_lowsq = d->rcut_low * d->rcut_low;
  v.ron_switch_sq = d->ron_switch * d->ron_switch;
  v.roff_switch_sq = d->roff_switch * d->roff_switch;
  if (d->vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) {
    double d2 = v.roff_switch_sq - v.ron_switch_sq;
    v.switch_factor1 = 1.0 / (d2 * d2 * d2);
    v.switch_factor2 = v.roff_switch_sq - 3.0 * v.ron_switch_sq;
  }
  v.beta = 1.0 / (kKBOLTZ * d->temperature);
  B.rcut_max = std::max(d->rcut_vdw, rcoul);  // precalculate.f90:79-83
  B.comcut = d->vdw_sum_style != CASS_VDW_SUM_MINIMUM &&
             ((d->vdw_style == CASS_VDW_LJ && d->vdw_sum_style == CASS_VDW_SUM_CHARMM) ||
              (d->charge_style == CASS_CHARGE_COUL && d->charge_sum_style == CASS_QQ_MINIMUM));
  B.rcut3 = d->rcut_vdw * d->rcut_vdw * d->rcut_vdw;
  B.rcut9 = B.rcut3 * B.rcut3 * B.rcut3;
  B.kvec.clear();
  B.nvecs = 0;
  if (d->charge_style == CASS_CHARGE_COUL && d->charge_sum_style == CASS_QQ_EWALD) {
    if (!(d->ewald_tol > 0.0 && d->ewald_tol < 1.0)) return set_error(CASS_EINVAL, "ewald_tol must be in (0,1)");
    double p = -std::log(d->ewald_tol);  // input_routines.f90:711-716
    v.alpha = std::sqrt(p) / rcoul;
    double hcut = 2.0 * p / rcoul;
    // Ewald_Reciprocal_Lattice_Vector_Setup, orthorhombic branch (energy_routines.f90:2260-2311)
    double const_val = 1.0 / (4.0 * v.alpha * v.alpha), hcutsq = hcut * hcut;
    int kz = (int)((hcut * v.L[2]) / kTWOPI) + 1, ky = (int)((hcut * v.L[1]) / kTWOPI) + 1,
        kx = (int)((hcut * v.L[0]) / kTWOPI) + 1;
    for (int nz = -kz; nz <= kz; ++nz)
      for (int ny = -ky; ny <= ky; ++ny)
        for (int nx = 0; nx <= kx; ++nx) {
          if (nx == 0 && ny == 0 && nz == 0) continue;
          double hx = kTWOPI * (double)nx / v.L[0], hy = kTWOPI * (double)ny / v.L[1], hz = kTWOPI * (double)nz / v.L[2];
          double h2 = hx * hx + hy * hy + hz * hz;
          if (h2 < hcutsq) {
            if (B.nvecs >= c->max_kvec) return set_error(CASS_ECAPACITY, "Total number of k vectors exceeded");
            double cn = kTWOPI / v.volume * std::exp(-h2 * const_val) / h2;
            if (nx != 0) cn = 2.0 * kTWOPI / v.volume * std::exp(-h2 * const_val) / h2;
            B.kvec.insert(B.kvec.end(), {hx, hy, hz, cn});
            ++B.nvecs;
          }
        }
    v.nvecs = B.nvecs;
    size_t nb = std::max(1, B.nvecs) * sizeof(double);
    int rc = B.d_kvec.reserve(std::max(1, B.nvecs) * sizeof(double4_32a));
    if (!rc) rc = B.d_cos_sum.reserve(nb);
    if (!rc) rc = B.d_sin_sum.reserve(nb);
    if (!rc) rc = B.d_cos_old.reserve(nb);
    if (!rc) rc = B.d_sin_old.reserve(nb);
    if (rc) return rc;
    CASS_CUDA(h2d(c, B.d_kvec.p, B.kvec.data(), B.kvec.size() * sizeof(double)));
    B.krow.clear();
    for (int k = 0; k < B.nvecs; ++k) {
      const double* h = &B.kvec[4 * (size_t)k];
      const bool cont = k > 0 && h[1] == h[-3] && h[2] == h[-2] &&
                        std::fabs(h[0] - (h[-4] + kTWOPI / v.L[0])) <= 1e-9 * (kTWOPI / v.L[0]);
      if (cont) ++B.krow.back().y;
      else B.krow.push_back(make_int2(k, 1));
    }
    if ((rc = B.d_krow.reserve(std::max<size_t>(1, B.krow.size()) * sizeof(int2)))) return rc;
    CASS_CUDA(h2d(c, B.d_krow.p, B.krow.data(), B.krow.size() * sizeof(int2)));
    CASS_CUDA(cudaMemsetAsync(B.d_cos_sum.p, 0, nb, c->stream));
    CASS_CUDA(cudaMemsetAsync(B.d_sin_sum.p, 0, nb, c->stream));
    CASS_CUDA(cudaStreamSynchronize(c->stream));
  }
  if (d->charge_style == CASS_CHARGE_COUL && d->charge_sum_style == CASS_QQ_DSF) {
    double a = d->alpha_dsf;
    if (a <= 0.0) {  // input_routines.f90:742-747
      a = 0.425 - rcoul * 0.02;
      if (a < 0.0) a = 3.3930702 / rcoul;
    }
    v.alpha_dsf = a;
    v.dsf_factor1 = std::erfc(a * rcoul) / rcoul;
    v.dsf_factor2 = v.dsf_factor1 / rcoul + 2.0 * a * std::exp(-a * a * rcoul * rcoul) / (kROOTPI * rcoul);
  }
  B.defined = true;
  invalidate(c, ibox - 1);
  return CASS_OK;
}

int cass_set_molecules(cass_ctx* c, int32_t n, const int32_t* im, const int32_t* is, const int32_t* ibox,
                       const double* xyz) {
  if (!c || n < 0 || (n > 0 && (!im || !is || !ibox || !xyz))) return set_error(CASS_EINVAL, "bad molecule list");
  for (int k = 0; k < n; ++k) {
    int rc = check_mol(c, im[k], is[k]);
    if (rc) return rc;
    if (ibox[k] < 1 || ibox[k] > c->nboxes) return set_error(CASS_EINVAL, "box index out of range");
  }
  // molecules that stay in a packed box are patched in place by one scatter
  // launch; any other change repacks the boxes involved on their next use
  std::vector<int> patch_slots;
  size_t off = 0;
  for (int k = 0; k < n; ++k) {
    SpeciesH& s = c->sp[is[k] - 1];
    const int slot = mol_slot(c, im[k], is[k]);
    const int old = c->mol_box[slot], nb = ibox[k] - 1;
    memcpy(&s.pos[(size_t)(im[k] - 1) * 3 * s.natoms], xyz + off, 3 * s.natoms * sizeof(double));
    off += 3 * s.natoms;
    set_mol_box(c, slot, nb);
    if (old >= 0 && old != nb) invalidate(c, old);
    if (old == nb && !c->box[nb].pack_dirty && !c->box[nb].comcut) patch_slots.push_back(slot);
    else invalidate(c, nb);
  }
  c->h_patch.clear();
  for (int slot : patch_slots) {
    const int b = c->mol_box[slot];
    BoxH& B = c->box[b];
    if (B.pack_dirty) continue;  // repacked from the host copy instead
    const int sp = c->slot_sp[slot];
    const SpeciesH& s = c->sp[sp];
    const int first = B.pk_mol_off[c->pk_index[slot]];
    const double* r = &s.pos[(size_t)(slot - c->mol_base[sp]) * 3 * s.natoms];
    for (int a = 0; a < s.natoms; ++a) {
      PatchRec q;
      q.x = r[3 * a];
      q.y = r[3 * a + 1];
      q.z = r[3 * a + 2];
      q.box = b;
      q.atom = first + a;
      c->h_patch.push_back(q);
    }
    B.energy_valid = false;
    B.frame_ready = false;
    B.cell_dirty = true;
  }
  const int np = (int)c->h_patch.size();
  if (np > 0) {
    int rc = set_device(c);
    if (rc) return rc;
    std::vector<BoxPtrs> bp(c->nboxes);
    for (int b = 0; b < c->nboxes; ++b) {
      bp[b].p64 = c->box[b].d_p64.as<double4_32a>();
      bp[b].p32 = c->box[b].d_p32.as<float4>();
    }
    const size_t rec_bytes = (size_t)np * sizeof(PatchRec);
    if ((rc = c->d_patch.reserve(rec_bytes + bp.size() * sizeof(BoxPtrs)))) return rc;
    PatchRec* d_rec = c->d_patch.as<PatchRec>();
    BoxPtrs* d_bp = reinterpret_cast<BoxPtrs*>(d_rec + np);
    CASS_CUDA(h2d(c, d_rec, c->h_patch.data(), rec_bytes));
    CASS_CUDA(h2d(c, d_bp, bp.data(), bp.size() * sizeof(BoxPtrs)));
    k_patch_atoms<<<(np + kBlock - 1) / kBlock, kBlock, 0, c->stream>>>(d_rec, np, d_bp);
    CASS_CUDA(cudaGetLastError());
    count_launch(c);
    // the staging vectors are reused by the next call: wait for the copies
    CASS_CUDA(cudaStreamSynchronize(c->stream));
  }
  return CASS_OK;
}

int cass_remove_molecule(cass_ctx* c, int32_t im, int32_t is) {
  if (!c) return set_error(CASS_EINVAL, "NULL context");
  int rc = check_mol(c, im, is);
  if (rc) return rc;
  int slot = mol_slot(c, im, is);
  if (c->mol_box[slot] >= 0) invalidate(c, c->mol_box[slot]);
  set_mol_box(c, slot, -1);
  return CASS_OK;
}

int cass_get_molecule(cass_ctx* c, int32_t im, int32_t is, double* xyz) {
  if (!c || !xyz) return set_error(CASS_EINVAL, "NULL argument");
  int rc = check_mol(c, im, is);
  if (rc) return rc;
  const SpeciesH& s = c->sp[is - 1];
  memcpy(xyz, &s.pos[(size_t)(im - 1) * 3 * s.natoms], 3 * s.natoms * sizeof(double));
  return CASS_OK;
}

int cass_get_molecule_boxes(cass_ctx* c, int32_t is, int32_t n, int32_t* which_box) {
  if (!c || (!which_box && n > 0)) return set_error(CASS_EINVAL, "NULL argument");
  if (is < 1 || is > c->nspecies) return set_error(CASS_EINVAL, "species index out of range");
  if (n < 0 || n > c->max_mol[is - 1]) return set_error(CASS_EINVAL, "n out of range");
  for (int im = 1; im <= n; ++im) which_box[im - 1] = c->mol_box[mol_slot(c, im, is)] + 1;
  return CASS_OK;
}

// Volume_Change (move_volume.f90:24-679), cubic boxes, up to its acceptance
// test: every live molecule of the box keeps the fractional coordinates of
// its COM and moves rigidly (:296-336), the box gets the new edge and its
// k-vectors (:374) and the system energy is recomputed (:426).  The old state
// is kept for cass_volume_restore.
int cass_volume_scale(cass_ctx* c, int32_t ibox1, double new_length, CassEnergy* e_new, int32_t* overlap) {
  if (!c || ibox1 < 1 || ibox1 > c->nboxes || !e_new || !overlap || !(new_length > 0.0))
    return set_error(CASS_EINVAL, "bad volume move arguments");
  BoxH& B = c->box[ibox1 - 1];
  if (!B.defined) return set_error(CASS_ESTATE, "box not defined");
  if (!B.energy_valid) return set_error(CASS_ESTATE, "system energy of box not computed");
  const CassBoxDesc d0 = B.desc;
  if (d0.length[0] != d0.length[1] || d0.length[0] != d0.length[2])
    return set_error(CASS_EUNSUPPORTED, "volume moves need a cubic box");
  const double half = 0.5 * new_length;
  if (half < d0.rcut_vdw || (d0.charge_style == CASS_CHARGE_COUL && half < d0.rcut_coul) ||
      (d0.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH && half < d0.roff_switch))
    return set_error(CASS_EINVAL, "cutoff greater than half the new box length (move_volume.f90:283-292)");
  const double L0 = d0.length[0];
  B.vol_saved = true;
  B.vol_desc = d0;
  B.vol_energy = B.energy;
  B.vol_im.clear();
  B.vol_is.clear();
  B.vol_xyz.clear();
  std::vector<double> xyz_new;
  for (int slot : members(c, ibox1 - 1)) {
    const int sp = c->slot_sp[slot];
    const SpeciesH& s = c->sp[sp];
    const int im = slot - c->mol_base[sp] + 1;
    const double* x = &s.pos[(size_t)(im - 1) * 3 * s.natoms];
    double tm = 0.0, com[3] = {0.0, 0.0, 0.0};  // Get_COM (get_com.f90:45-105)
    for (int a = 0; a < s.natoms; ++a) {
      tm += s.mass[a];
      for (int k = 0; k < 3; ++k) com[k] += s.mass[a] * x[3 * a + k];
    }
    double sh[3];
    for (int k = 0; k < 3; ++k) {
      com[k] = com[k] / tm;
      sh[k] = new_length * (com[k] / L0) - com[k];  // fractional COM kept (:300-323)
    }
    B.vol_im.push_back(im);
    B.vol_is.push_back(sp + 1);
    for (int a = 0; a < 3 * s.natoms; ++a) {
      B.vol_xyz.push_back(x[a]);
      xyz_new.push_back(x[a] + sh[a % 3]);
    }
  }
  const int n = (int)B.vol_im.size();
  std::vector<int32_t> boxes(n, ibox1);
  int rc;
  if (n > 0 && (rc = cass_set_molecules(c, n, B.vol_im.data(), B.vol_is.data(), boxes.data(), xyz_new.data())))
    return rc;
  CassBoxDesc d1 = d0;
  d1.length[0] = d1.length[1] = d1.length[2] = new_length;
  if ((rc = cass_set_box(c, ibox1, &d1))) return rc;
  return cass_system_total_energy(c, ibox1, 1, e_new, overlap);
}

// Reset_Coords (move_volume.f90:555-677): the coordinates, box and energy
// saved by the last cass_volume_scale of the box.  The structure factors are
// recomputed from the restored coordinates; energy(ibox) is the saved value.
int cass_volume_restore(cass_ctx* c, int32_t ibox1) {
  if (!c || ibox1 < 1 || ibox1 > c->nboxes) return set_error(CASS_EINVAL, "bad box");
  BoxH& B = c->box[ibox1 - 1];
  if (!B.vol_saved) return set_error(CASS_ESTATE, "no volume move to restore");
  const int n = (int)B.vol_im.size();
  std::vector<int32_t> boxes(n, ibox1);
  int rc;
  if (n > 0 && (rc = cass_set_molecules(c, n, B.vol_im.data(), B.vol_is.data(), boxes.data(), B.vol_xyz.data())))
    return rc;
  const CassBoxDesc d0 = B.vol_desc;
  const CassEnergy e0 = B.vol_energy;
  if ((rc = cass_set_box(c, ibox1, &d0))) return rc;
  CassEnergy e;
  int32_t ov = 0;
  if ((rc = cass_system_total_energy(c, ibox1, 1, &e, &ov))) return rc;
  BoxH& B2 = c->box[ibox1 - 1];
  B2.energy = e0;
  B2.vol_saved = false;
  return CASS_OK;
}

int cass_set_cbmc_options(cass_ctx* c, const CassCBMCOptions* o) {
  if (!c || !o || o->energy_table_res < 0 || o->energy_table_res > (1 << 20) || !(o->rmin_u_max >= 0.0))
    return set_error(CASS_EINVAL, "bad CBMC options");
  c->cbmc_opt = *o;
  c->cbmc_dirty = true;
  return CASS_OK;
}

int cass_mol_inter_energy(cass_ctx* c, int32_t im, int32_t is, int32_t cbmc, double* ev, double* eq, int32_t* ov) {
  if (!c || !ev || !eq || !ov) return set_error(CASS_EINVAL, "NULL argument");
  int rc = check_mol(c, im, is);
  if (rc) return rc;
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  int slot = mol_slot(c, im, is);
  int ibox = c->mol_box[slot];
  if (ibox < 0) return set_error(CASS_ESTATE, "molecule not live");
  if ((rc = set_device(c)) || (rc = pack_box(c, ibox))) return rc;
  if (cbmc && (rc = ensure_cbmc(c))) return rc;
  BoxH& B = c->box[ibox];
  const int qoff = B.pk_mol_off[c->pk_index[slot]];
  const SpeciesH& s = c->sp[is - 1];
  if (s.natoms > kMaxAtoms * 4) return set_error(CASS_ECAPACITY, "query molecule too large");
  int nblk = std::max(1, std::min(148, (B.npacked + kBlock - 1) / kBlock));
  if ((rc = ensure_scratch(c, nblk, 2))) return rc;
  int rc2 = c->d_query.reserve(16);
  if (rc2) return rc2;
  CASS_CUDA(cudaMemsetAsync(c->d_query.p, 0, sizeof(int), c->stream));
  int want_qq = (cbmc && !s.l_coul_cbmc) ? 0 : 1;
  // Check_MoleculePair_Cutoff where a style has no atom cutoff (rcut_cbmc with the CBMC flag)
  const double4_32a* mcom = B.comcut ? B.d_com.as<double4_32a>() : nullptr;
  const double mrad = cbmc ? B.desc.rcut_cbmc : B.rcut_max;
  if (c->precision == CASS_PREC_MIXED)
    k_mol_inter<true><<<nblk, kBlock, 0, c->stream>>>(B.dev, c->pt, B.d_p64.as<double4_32a>(), B.d_p32.as<float4>(),
                                                      B.d_meta.as<int4>(), B.npacked, slot, qoff, s.natoms, cbmc,
                                                      want_qq, mcom, mrad, c->d_partial.as<double>(), c->d_counter.as<unsigned>(),
                                                      c->d_result.as<double>(), c->d_query.as<int>());
  else
    k_mol_inter<false><<<nblk, kBlock, 0, c->stream>>>(B.dev, c->pt, B.d_p64.as<double4_32a>(), B.d_p32.as<float4>(),
                                                       B.d_meta.as<int4>(), B.npacked, slot, qoff, s.natoms, cbmc,
                                                       want_qq, mcom, mrad, c->d_partial.as<double>(), c->d_counter.as<unsigned>(),
                                                       c->d_result.as<double>(), c->d_query.as<int>());
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  int hov = 0;
  CASS_CUDA(d2h(c, &hov, c->d_query.p, sizeof(int)));
  if ((rc = sync_result(c, 2))) return rc;
  *ov = hov ? 1 : 0;
  *ev = hov ? 0.0 : c->h_result[0];
  *eq = hov ? 0.0 : c->h_result[1];
  return CASS_OK;
}

int cass_atom_intra_energies(cass_ctx* c, int32_t ibox1, int32_t is, int32_t ia, int32_t ntrial, const double* xyz,
                             const int32_t* exist, int32_t cbmc, double* e, int32_t* overlap) {
  if (!c || ibox1 < 1 || ibox1 > c->nboxes || is < 1 || is > c->nspecies || ntrial < 0 ||
      (ntrial > 0 && (!xyz || !e || !overlap)))
    return set_error(CASS_EINVAL, "bad atom intra arguments");
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  const SpeciesH& s = c->sp[is - 1];
  if (!s.defined) return set_error(CASS_ESTATE, "species not defined");
  if (s.natoms > 32) return set_error(CASS_ECAPACITY, "at most 32 atoms per molecule");
  if (ia < 1 || ia > s.natoms) return set_error(CASS_EINVAL, "atom index out of range");
  if (ntrial == 0) return CASS_OK;
  unsigned mask = 0u;
  for (int a = 0; a < s.natoms; ++a)
    if (!exist || exist[a]) mask |= 1u << a;
  int rc;
  if ((rc = set_device(c)) || (rc = ensure_pools(c))) return rc;
  BoxH& B = c->box[ibox1 - 1];
  if (!B.defined) return set_error(CASS_ESTATE, "box not defined");
  const size_t nx = (size_t)ntrial * s.natoms * 3;
  if ((rc = c->d_trial.reserve(nx * sizeof(double) + (size_t)ntrial * (3 * sizeof(double) + sizeof(int)) + 64)))
    return rc;
  double* d_x = c->d_trial.as<double>();
  double* d_e = d_x + nx;
  int* d_ov = reinterpret_cast<int*>(d_e + 3 * (size_t)ntrial);
  CASS_CUDA(h2d(c, d_x, xyz, nx * sizeof(double)));
  k_atom_intra<<<(ntrial + kBlock - 1) / kBlock, kBlock, 0, c->stream>>>(B.dev, c->pt, c->pools, is - 1, ia - 1, d_x,
                                                                         s.natoms, mask, ntrial, cbmc, d_e, d_ov);
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  CASS_CUDA(d2h(c, e, d_e, 3 * (size_t)ntrial * sizeof(double)));
  CASS_CUDA(d2h(c, overlap, d_ov, (size_t)ntrial * sizeof(int)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  return CASS_OK;
}

int cass_cbmc_trial_energies(cass_ctx* c, int32_t ibox1, int32_t is, int32_t skip_im, int32_t nat,
                             const int32_t* atoms, int32_t ntrial, const double* xyz, int32_t cbmc, double* e,
                             int32_t* overlap) {
  if (!c || ibox1 < 1 || ibox1 > c->nboxes || is < 1 || is > c->nspecies || nat < 1 || !atoms || ntrial < 0 ||
      (ntrial > 0 && (!xyz || !e || !overlap)))
    return set_error(CASS_EINVAL, "bad trial arguments");
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  const SpeciesH& s = c->sp[is - 1];
  if (!s.defined) return set_error(CASS_ESTATE, "species not defined");
  if (nat > kTrialMaxAtoms) return set_error(CASS_ECAPACITY, "at most 64 atoms per trial");
  if (skip_im < 0 || skip_im > c->max_mol[is - 1]) return set_error(CASS_EINVAL, "molecule locate out of range");
  for (int a = 0; a < nat; ++a)
    if (atoms[a] < 1 || atoms[a] > s.natoms) return set_error(CASS_EINVAL, "trial atom index out of range");
  if (ntrial == 0) return CASS_OK;
  const int ib = ibox1 - 1;
  int rc;
  if ((rc = set_device(c)) || (rc = pack_box(c, ib))) return rc;
  if (cbmc && (rc = ensure_cbmc(c))) return rc;
  BoxH& B = c->box[ib];
  std::vector<double4_32a> tr((size_t)ntrial * nat);
  std::vector<int> tt(nat);
  for (int a = 0; a < nat; ++a) tt[a] = s.type[atoms[a] - 1];
  for (int k = 0; k < ntrial; ++k)
    for (int a = 0; a < nat; ++a) {
      const double* x = xyz + ((size_t)k * nat + a) * 3;
      tr[(size_t)k * nat + a] = make_double4_32a(x[0], x[1], x[2], s.q[atoms[a] - 1]);
    }
  // Check_MoleculePair_Cutoff where a style has no atom cutoff: the COM and
  // max_dcom of each trial's atoms (get_com.f90:45-105, 220-295)
  std::vector<double4_32a> tcom;
  if (B.comcut)
    for (int k = 0; k < ntrial; ++k) {
      double tm = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
      for (int a = 0; a < nat; ++a) {
        const double m = s.mass[atoms[a] - 1];
        const double4_32a& p = tr[(size_t)k * nat + a];
        tm = tm + m;
        cx = cx + m * p.x;
        cy = cy + m * p.y;
        cz = cz + m * p.z;
      }
      cx = cx / tm;
      cy = cy / tm;
      cz = cz / tm;
      double dmax = 0.0;
      for (int a = 0; a < nat; ++a) {
        const double4_32a& p = tr[(size_t)k * nat + a];
        const double dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
        dmax = std::max(dmax, dx * dx + dy * dy + dz * dz);
      }
      tcom.push_back(make_double4_32a(cx, cy, cz, std::sqrt(dmax)));
    }
  const size_t tb = tr.size() * sizeof(double4_32a);
  const size_t cb = tcom.size() * sizeof(double4_32a);
  if ((rc = c->d_trial.reserve(tb + cb + (size_t)nat * sizeof(int) + (size_t)ntrial * (sizeof(double) + sizeof(int)) + 64)))
    return rc;
  double4_32a* d_tr = c->d_trial.as<double4_32a>();
  double4_32a* d_tcom = B.comcut ? d_tr + tr.size() : nullptr;
  int* d_tt = reinterpret_cast<int*>(d_tr + tr.size() + tcom.size());
  double* d_e = reinterpret_cast<double*>(reinterpret_cast<char*>(d_tt) + (((size_t)nat * sizeof(int) + 7) & ~(size_t)7));
  int* d_ov = reinterpret_cast<int*>(d_e + ntrial);
  CASS_CUDA(h2d(c, d_tr, tr.data(), tb));
  if (B.comcut) CASS_CUDA(h2d(c, d_tcom, tcom.data(), cb));
  CASS_CUDA(h2d(c, d_tt, tt.data(), (size_t)nat * sizeof(int)));
  const double4_32a* d_com = B.comcut ? B.d_com.as<double4_32a>() : nullptr;
  const double rmax = cbmc ? B.desc.rcut_cbmc : B.rcut_max;
  const int skip_slot = skip_im > 0 ? mol_slot(c, skip_im, is) : -1;
  const int want_qq = (cbmc && !s.l_coul_cbmc) ? 0 : 1;  // Compute_MoleculePair_Energy, energy_routines.f90:1684-1686
  if (c->precision == CASS_PREC_MIXED)
    k_trial_energy<true><<<ntrial, kBlock, 0, c->stream>>>(B.dev, c->pt, B.d_p64.as<double4_32a>(), B.d_meta.as<int4>(),
                                                           B.npacked, skip_slot, d_tr, d_tt, nat, cbmc, want_qq, d_tcom,
                                                           d_com, rmax, d_e, d_ov);
  else
    k_trial_energy<false><<<ntrial, kBlock, 0, c->stream>>>(B.dev, c->pt, B.d_p64.as<double4_32a>(), B.d_meta.as<int4>(),
                                                            B.npacked, skip_slot, d_tr, d_tt, nat, cbmc, want_qq, d_tcom,
                                                            d_com, rmax, d_e, d_ov);
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  CASS_CUDA(d2h(c, e, d_e, (size_t)ntrial * sizeof(double)));
  CASS_CUDA(d2h(c, overlap, d_ov, (size_t)ntrial * sizeof(int)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  return CASS_OK;
}

int cass_mol_intra_energy(cass_ctx* c, int32_t im, int32_t is, int32_t cbmc, double* eiv, double* eiq, double* eoq,
                          int32_t* ov) {
  if (!c || !eiv || !eiq || !eoq || !ov) return set_error(CASS_EINVAL, "NULL argument");
  int rc = check_mol(c, im, is);
  if (rc) return rc;
  int slot = mol_slot(c, im, is);
  int ibox = c->mol_box[slot];
  if (ibox < 0) return set_error(CASS_ESTATE, "molecule not live");
  if ((rc = set_device(c)) || (rc = pack_box(c, ibox))) return rc;
  if ((rc = ensure_pools(c))) return rc;
  BoxH& B = c->box[ibox];
  const int q = c->pk_index[slot];
  if ((rc = ensure_scratch(c, 1, 7))) return rc;
  if ((rc = c->d_query.reserve(16))) return rc;
  CASS_CUDA(cudaMemsetAsync(c->d_query.p, 0, sizeof(int), c->stream));
  k_intra_total<<<1, kBlock, 0, c->stream>>>(B.dev, c->pt, c->pools, B.d_p64.as<double4_32a>(), B.d_molinfo.as<int4>() + q, 1,
                                             c->d_partial.as<double>(), c->d_counter.as<unsigned>(),
                                             c->d_result.as<double>(), c->d_query.as<int>(), cbmc ? 1 : 0);
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  int hov = 0;
  CASS_CUDA(d2h(c, &hov, c->d_query.p, sizeof(int)));
  if ((rc = sync_result(c, 7))) return rc;
  *ov = hov ? 1 : 0;
  *eiv = c->h_result[4];
  *eiq = c->h_result[5];
  *eoq = c->h_result[6];
  return CASS_OK;
}

// Compute_System_Ewald_Reciprocal_Energy (energy_routines.f90:4111-4231): every
// molecule's cos_mol/sin_mol row, the box's cos_sum/sin_sum and the reciprocal
// energy, on the device.
static int box_reciprocal(cass_ctx* c, int ibox, double* e_recip) {
  BoxH& B = c->box[ibox];
  int rc;
  int nv = B.nvecs;
  if ((rc = ensure_cos_mol(c, nv))) return rc;
  DevBuf& part = c->d_box_sums;
  int nchunks = std::max(1, (B.npacked_mols + kSfacMolChunk - 1) / kSfacMolChunk);
  if ((rc = part.reserve((size_t)nchunks * nv * sizeof(double2)))) return rc;
  std::vector<int> charged(c->nspecies);
  for (int is = 0; is < c->nspecies; ++is) charged[is] = c->sp[is].has_charge ? 1 : 0;
  DevBuf& dch = c->d_cell_count;  // small reuse: species charged flags
  if ((rc = dch.reserve(std::max(c->nspecies, 1) * sizeof(int) + 256))) return rc;
  CASS_CUDA(h2d(c, dch.p, charged.data(), c->nspecies * sizeof(int)));
  // FP64 contexts with small molecules: the row recurrence, then the sums
  // from the molecule rows
  int max_na = 0;
  for (int is = 0; is < c->nspecies; ++is)
    if (c->sp[is].defined && c->sp[is].has_charge) max_na = std::max(max_na, c->sp[is].natoms);
  if (c->precision != CASS_PREC_MIXED && !B.krow.empty() && max_na <= kSfacRowAtoms && B.npacked_mols > 0) {
    const int nrows = (int)B.krow.size();
    dim3 g((nrows + 127) / 128, std::min(B.npacked_mols, 65535));
    k_sfac_rows<<<g, 128, 0, c->stream>>>(B.d_kvec.as<double4_32a>(), B.d_krow.as<int2>(), nrows, kTWOPI / B.dev.L[0],
                                          B.d_p64.as<double4_32a>(), B.d_molinfo.as<int4>(), B.npacked_mols,
                                          dch.as<int>(), c->d_cos_mol.as<double>(), c->d_sin_mol.as<double>(),
                                          c->cos_mol_stride);
    CASS_CUDA(cudaGetLastError());
    count_launch(c);
    k_sfac_sum<<<dim3((nv + kBlock - 1) / kBlock, nchunks), kBlock, 0, c->stream>>>(
        nv, B.d_molinfo.as<int4>(), B.npacked_mols, dch.as<int>(), c->d_cos_mol.as<double>(),
        c->d_sin_mol.as<double>(), c->cos_mol_stride, part.as<double2>());
    CASS_CUDA(cudaGetLastError());
    count_launch(c);
  } else if (B.npacked_mols > 0) {
    dim3 g((nv + 127) / 128, nchunks);
    auto kern = c->precision == CASS_PREC_MIXED ? k_sfac<true> : k_sfac<false>;
    kern<<<g, 128, 0, c->stream>>>(B.d_kvec.as<double4_32a>(), nv, B.d_p64.as<double4_32a>(), B.d_molinfo.as<int4>(),
                                   B.npacked_mols, dch.as<int>(), c->d_cos_mol.as<double>(),
                                   c->d_sin_mol.as<double>(), c->cos_mol_stride, part.as<double2>());
    CASS_CUDA(cudaGetLastError());
  count_launch(c);
  } else {
    CASS_CUDA(cudaMemsetAsync(part.p, 0, (size_t)nv * sizeof(double2), c->stream));
  }
  int nblk = std::max(1, std::min(148, (nv + kBlock - 1) / kBlock));
  if ((rc = ensure_scratch(c, nblk, 1))) return rc;
  k_sfac_reduce<<<nblk, kBlock, 0, c->stream>>>(B.d_kvec.as<double4_32a>(), nv, part.as<double2>(), nchunks,
                                                B.d_cos_sum.as<double>(), B.d_sin_sum.as<double>(),
                                                c->d_partial.as<double>(), c->d_counter.as<unsigned>(),
                                                c->d_result.as<double>());
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  if ((rc = sync_result(c, 1))) return rc;
  *e_recip = c->h_result[0] * kCHARGE_FACTOR;
  return CASS_OK;
}

int cass_system_total_energy(cass_ctx* c, int32_t ibox1, int32_t intra_flag, CassEnergy* out, int32_t* overlap) {
  if (!c || ibox1 < 1 || ibox1 > c->nboxes || !out || !overlap) return set_error(CASS_EINVAL, "bad arguments");
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  int ibox = ibox1 - 1;
  BoxH& B = c->box[ibox];
  if (!B.defined) return set_error(CASS_ESTATE, "box not defined");
  int rc;
  if ((rc = set_device(c)) || (rc = pack_box(c, ibox))) return rc;
  if ((rc = ensure_pools(c))) return rc;
  CassEnergy E = B.energy;
  CassEnergy keep = E;
  E = CassEnergy{};
  *overlap = 0;
  if ((rc = c->d_query.reserve(16))) return rc;
  CASS_CUDA(cudaMemsetAsync(c->d_query.p, 0, sizeof(int), c->stream));
  int n = B.npacked;
  std::vector<double> res;
  if (intra_flag && B.npacked_mols > 0) {
    int nblk = std::max(1, std::min(296, (B.npacked_mols + kBlock - 1) / kBlock));
    if ((rc = ensure_scratch(c, nblk, 7))) return rc;
    k_intra_total<<<nblk, kBlock, 0, c->stream>>>(B.dev, c->pt, c->pools, B.d_p64.as<double4_32a>(), B.d_molinfo.as<int4>(),
                                                   B.npacked_mols, c->d_partial.as<double>(),
                                                   c->d_counter.as<unsigned>(), c->d_result.as<double>(),
                                                   c->d_query.as<int>());
    CASS_CUDA(cudaGetLastError());
  count_launch(c);
    if ((rc = sync_result(c, 7))) return rc;
    E.bond = c->h_result[0];
    E.angle = c->h_result[1];
    E.dihedral = c->h_result[2];
    E.improper = c->h_result[3];
    E.intra_vdw = c->h_result[4];
    E.intra_q = c->h_result[5];
    E.inter_q = c->h_result[6];
    E.intra = E.bond + E.angle + E.dihedral + E.improper + E.intra_q + E.intra_vdw;
  } else if (!intra_flag) {
    E.intra = keep.intra; E.bond = keep.bond; E.angle = keep.angle; E.dihedral = keep.dihedral;
    E.improper = keep.improper; E.intra_vdw = keep.intra_vdw; E.intra_q = keep.intra_q;
  }
  if (n > 1) {
    dim3 grid((n + kBlock - 1) / kBlock, (n + kTileJ - 1) / kTileJ);
    if ((rc = ensure_scratch(c, grid.x * grid.y, 2))) return rc;
    const bool fast = c->precision == CASS_PREC_MIXED && B.desc.vdw_style == CASS_VDW_LJ &&
                      (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT || B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) &&
                      (B.desc.charge_style == CASS_CHARGE_NONE || B.desc.charge_sum_style == CASS_QQ_EWALD);
    // the largest cutoff cutoff_mask applies outside CBMC (none for the minimum-image styles)
    double rmax2 = B.dev.rcut_lowsq;
    bool bounded = true;
    if (B.desc.vdw_style == CASS_VDW_LJ) {
      if (B.desc.vdw_sum_style == CASS_VDW_SUM_MINIMUM || B.desc.vdw_sum_style == CASS_VDW_SUM_CHARMM) bounded = false;
      else rmax2 = std::max(rmax2, B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH ? B.dev.roff_switch_sq : B.dev.rcut_vdwsq);
    } else if (B.desc.vdw_style == CASS_VDW_MIE) {
      rmax2 = std::max(rmax2, B.dev.rcut_vdwsq);
    }
    if (B.desc.charge_style == CASS_CHARGE_COUL) {
      if (B.desc.charge_sum_style == CASS_QQ_MINIMUM) bounded = false;
      else rmax2 = std::max(rmax2, B.dev.rcut_coulsq);
    }
    const float pre2 = bounded ? (float)(rmax2 * (1.0 + 1.0e-4) + 1.0e-3) : FLT_MAX;
    if (fast)
      k_pair_total<true><<<grid, kBlock, 0, c->stream>>>(B.dev, c->pt, B.d_p64.as<double4_32a>(), B.d_meta.as<int4>(), n,
                                                        pre2, nullptr, 0.0, c->d_partial.as<double>(),
                                                        c->d_counter.as<unsigned>(), c->d_result.as<double>(),
                                                        c->d_query.as<int>());
    else
      k_pair_total<false><<<grid, kBlock, 0, c->stream>>>(B.dev, c->pt, B.d_p64.as<double4_32a>(), B.d_meta.as<int4>(), n,
                                                         pre2, B.comcut ? B.d_com.as<double4_32a>() : nullptr,
                                                         B.rcut_max, c->d_partial.as<double>(),
                                                         c->d_counter.as<unsigned>(), c->d_result.as<double>(),
                                                         c->d_query.as<int>());
    CASS_CUDA(cudaGetLastError());
  count_launch(c);
    if ((rc = sync_result(c, 2))) return rc;
    E.inter_vdw += c->h_result[0];
    E.inter_q += c->h_result[1];
  }
  int hov = 0;
  CASS_CUDA(d2h(c, &hov, c->d_query.p, sizeof(int)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  if (hov) {
    *overlap = 1;
    B.energy_valid = false;
    B.frame_ready = false;
    return CASS_OK;
  }
  E.inter = E.inter_q + E.inter_vdw;
  if (B.desc.charge_style == CASS_CHARGE_COUL) {
    if (box_has_ewald(B) && B.nvecs > 0) {
      if ((rc = box_reciprocal(c, ibox, &E.reciprocal))) return rc;
      E.inter = E.inter + E.reciprocal;
    }
    // Compute_System_Self_Energy (energy_routines.f90:2553-2601), O(nmol) host sum of charges squared
    double es = 0.0;
    for (int slot : members(c, ibox)) {
      const SpeciesH& s = c->sp[c->slot_sp[slot]];
      for (int a = 0; a < s.natoms; ++a) es = es + s.q[a] * s.q[a];
    }
    if (B.desc.charge_sum_style == CASS_QQ_EWALD) E.self = -es * kCHARGE_FACTOR * B.dev.alpha / kROOTPI;
    else if (B.desc.charge_sum_style == CASS_QQ_DSF)
      E.self = -(es * (B.dev.alpha_dsf / kROOTPI + B.dev.dsf_factor1 / 2.0)) * kCHARGE_FACTOR;
    E.inter = E.inter + E.self;
  }
  if (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) {
    E.lrc = lr_correction(c, B, count_beads(c, ibox));
    E.inter = E.inter + E.lrc;
  }
  E.total = E.intra + E.inter;
  B.energy = E;
  B.energy_valid = true;
  B.frame_ready = true;
  *out = E;
  return CASS_OK;
}

int cass_ewald_update(cass_ctx* c, int32_t im, int32_t is, int32_t ibox1, int32_t move_flag, double* e_recip) {
  if (!c || !e_recip) return set_error(CASS_EINVAL, "NULL argument");
  int rc = check_mol(c, im, is);
  if (rc) return rc;
  if (ibox1 < 1 || ibox1 > c->nboxes) return set_error(CASS_EINVAL, "box index");
  if (move_flag < 0 || move_flag > 4) return set_error(CASS_EINVAL, "bad move_flag");
  BoxH& B = c->box[ibox1 - 1];
  if (!box_has_ewald(B)) return set_error(CASS_ESTATE, "box has no Ewald sum");
  if ((rc = set_device(c))) return rc;
  int nv = B.nvecs;
  if ((rc = ensure_cos_mol(c, nv))) return rc;
  int slot = mol_slot(c, im, is);
  const SpeciesH& s = c->sp[is - 1];
  size_t nb = (size_t)nv * sizeof(double);
  double* cm = c->d_cos_mol.as<double>() + (size_t)slot * c->cos_mol_stride;
  double* sm = c->d_sin_mol.as<double>() + (size_t)slot * c->cos_mol_stride;
  CASS_CUDA(cudaMemcpyAsync(B.d_cos_old.p, B.d_cos_sum.p, nb, cudaMemcpyDeviceToDevice, c->stream));
  CASS_CUDA(cudaMemcpyAsync(B.d_sin_old.p, B.d_sin_sum.p, nb, cudaMemcpyDeviceToDevice, c->stream));
  CASS_CUDA(cudaMemcpyAsync(c->d_cos_mol_old.p, cm, nb, cudaMemcpyDeviceToDevice, c->stream));
  CASS_CUDA(cudaMemcpyAsync(c->d_sin_mol_old.p, sm, nb, cudaMemcpyDeviceToDevice, c->stream));
  std::vector<double4_32a> qa(s.natoms);
  const double* r = &s.pos[(size_t)(im - 1) * 3 * s.natoms];
  for (int a = 0; a < s.natoms; ++a) qa[a] = make_double4_32a(r[3 * a], r[3 * a + 1], r[3 * a + 2], s.q[a]);
  if ((rc = c->d_query.reserve(std::max<size_t>(16, qa.size() * sizeof(double4_32a))))) return rc;
  CASS_CUDA(h2d(c, c->d_query.p, qa.data(), qa.size() * sizeof(double4_32a)));
  int nblk = std::max(1, std::min(148, (nv + kBlock - 1) / kBlock));
  if ((rc = ensure_scratch(c, nblk, 1))) return rc;
  k_ewald_update<<<nblk, kBlock, 0, c->stream>>>(B.d_kvec.as<double4_32a>(), nv, c->d_query.as<double4_32a>(), s.natoms,
                                                 move_flag, B.d_cos_sum.as<double>(), B.d_sin_sum.as<double>(), cm, sm,
                                                 c->d_partial.as<double>(), c->d_counter.as<unsigned>(),
                                                 c->d_result.as<double>());
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  if ((rc = sync_result(c, 1))) return rc;
  *e_recip = c->h_result[0] * kCHARGE_FACTOR;
  B.energy_valid = false;
  B.frame_ready = false;
  return CASS_OK;
}

int cass_ewald_restore(cass_ctx* c, int32_t im, int32_t is, int32_t ibox1) {
  if (!c) return set_error(CASS_EINVAL, "NULL context");
  int rc = check_mol(c, im, is);
  if (rc) return rc;
  if (ibox1 < 1 || ibox1 > c->nboxes) return set_error(CASS_EINVAL, "box index");
  BoxH& B = c->box[ibox1 - 1];
  if (!box_has_ewald(B) || !c->d_cos_mol.p) return set_error(CASS_ESTATE, "nothing to restore");
  if ((rc = set_device(c))) return rc;
  int slot = mol_slot(c, im, is);
  size_t nb = (size_t)B.nvecs * sizeof(double);
  double* cm = c->d_cos_mol.as<double>() + (size_t)slot * c->cos_mol_stride;
  double* sm = c->d_sin_mol.as<double>() + (size_t)slot * c->cos_mol_stride;
  CASS_CUDA(cudaMemcpyAsync(B.d_cos_sum.p, B.d_cos_old.p, nb, cudaMemcpyDeviceToDevice, c->stream));
  CASS_CUDA(cudaMemcpyAsync(B.d_sin_sum.p, B.d_sin_old.p, nb, cudaMemcpyDeviceToDevice, c->stream));
  CASS_CUDA(cudaMemcpyAsync(cm, c->d_cos_mol_old.p, nb, cudaMemcpyDeviceToDevice, c->stream));
  CASS_CUDA(cudaMemcpyAsync(sm, c->d_sin_mol_old.p, nb, cudaMemcpyDeviceToDevice, c->stream));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  return CASS_OK;
}

int cass_ewald_widom(cass_ctx* c, int32_t is, int32_t ibox1, int32_t n, const double* xyz, double* e) {
  if (!c || is < 1 || is > c->nspecies || ibox1 < 1 || ibox1 > c->nboxes || n < 0 || (n > 0 && (!xyz || !e)))
    return set_error(CASS_EINVAL, "bad arguments");
  BoxH& B = c->box[ibox1 - 1];
  if (!box_has_ewald(B)) return set_error(CASS_ESTATE, "box has no Ewald sum");
  if (n == 0) return CASS_OK;
  int rc;
  if ((rc = set_device(c))) return rc;
  const SpeciesH& s = c->sp[is - 1];
  size_t nx = (size_t)n * 3 * s.natoms;
  DevBuf& dx = c->d_widom_xyz;
  DevBuf& dout = c->d_widom_out;
  if ((rc = dx.reserve(nx * sizeof(double) + s.natoms * sizeof(double)))) return rc;
  if ((rc = dout.reserve((size_t)n * sizeof(double)))) return rc;
  CASS_CUDA(h2d(c, dx.p, xyz, nx * sizeof(double)));
  double* dq = dx.as<double>() + nx;
  CASS_CUDA(h2d(c, dq, s.q.data(), s.natoms * sizeof(double)));
  k_ewald_widom<<<n, kBlock, 0, c->stream>>>(B.d_kvec.as<double4_32a>(), B.nvecs, B.d_cos_sum.as<double>(),
                                             B.d_sin_sum.as<double>(), dx.as<double>(), dq, s.natoms, dout.as<double>());
  CASS_CUDA(cudaGetLastError());
  count_launch(c);
  CASS_CUDA(d2h(c, e, dout.p, n * sizeof(double)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  return CASS_OK;
}

}  // extern "C"

namespace cassgpu {
// The box set-up at the end of Set_Frame_Coords (load_next_frame.f90:290-301):
// the long-range correction (Compute_LR_Correction) and, for Ewald boxes, the
// structure factors and reciprocal energy (Compute_System_Ewald_Reciprocal_Energy).
// Enough for Widom insertions; the other energy components are left to
// cass_system_total_energy.
// Every box of the context; the molecule rows are sized for the largest k-vector
// count first, so that no box's rebuild reallocates (and so invalidates) the
// rows of a box set up before it.
int frame_setup_ext(cass_ctx* c) {
  int rc, nv = 0;
  for (BoxH& B : c->box)
    if (box_has_ewald(B)) nv = std::max(nv, B.nvecs);
  if (nv > 0 && (rc = ensure_cos_mol(c, nv))) return rc;
  // every dirty box packed into one pinned staging area, uploaded in one copy
  // with the list of its per-box arrays and scattered by one kernel (four
  // copies per box cost more in API calls than in bytes), one synchronization
  std::vector<size_t> off(c->nboxes + 1, 0);
  for (int ibox = 0; ibox < c->nboxes; ++ibox)
    off[ibox + 1] = off[ibox] + (c->box[ibox].pack_dirty ? pack_bytes(c, ibox) : 0);
  const size_t list_off = (off[c->nboxes] + 255) & ~(size_t)255;
  const size_t total = list_off + (size_t)4 * c->nboxes * sizeof(StageCopy);
  if ((rc = c->h_pack.reserve(std::max<size_t>(total, 256)))) return rc;
  unsigned char* hs = static_cast<unsigned char*>(c->h_pack.p);
  std::vector<StageCopy> cps;
  for (int ibox = 0; ibox < c->nboxes; ++ibox)
    if (c->box[ibox].pack_dirty && (rc = pack_box_async(c, ibox, hs + off[ibox], &cps, hs))) return rc;
  if (!cps.empty()) {
    memcpy(hs + list_off, cps.data(), cps.size() * sizeof(StageCopy));
    const size_t up = list_off + cps.size() * sizeof(StageCopy);
    if ((rc = c->d_stage.reserve(up))) return rc;
    CASS_CUDA(h2d(c, c->d_stage.p, hs, up));
    k_stage_scatter<<<(unsigned)cps.size(), 256, 0, c->stream>>>(
        c->d_stage.as<unsigned char>(), reinterpret_cast<const StageCopy*>(c->d_stage.as<unsigned char>() + list_off));
    CASS_CUDA(cudaGetLastError());
    count_launch(c);
  }
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  for (int ibox = 0; ibox < c->nboxes; ++ibox) {
    BoxH& B = c->box[ibox];
    if (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) B.energy.lrc = lr_correction(c, B, count_beads(c, ibox));
    if (box_has_ewald(B) && B.nvecs > 0 && (rc = box_reciprocal(c, ibox, &B.energy.reciprocal))) return rc;
    B.frame_ready = true;
  }
  return CASS_OK;
}
}  // namespace cassgpu

