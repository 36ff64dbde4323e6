// cass_noalloc.cu -- an energy entry point that allocates no device memory.
//
// Who needs it: a Monte Carlo driver calls the molecule-vs-box energy twice
// per translation or rotation move, millions of times per run.  Some such
// hosts cannot call cudaMalloc inside their move loop: the device memory is
// owned by another allocator (a framework's caching pool or a Fortran host that
// reserves everything at start-up and forbids later allocation), or an
// allocation would synchronize the device in the middle of a latency-bound
// loop.  cass_mol_box_energy_noalloc serves them: the caller passes device
// arrays for the inputs and the output, and the only scratch the kernel needs
// (per-block partial sums for a fixed-order reduction, a block counter and an
// overlap flag) lives in the file-scope array g_noalloc_scratch below, which
// every GPU that loads this library holds until the process exits.
//
// Limits and rules (repeated in the header):
//   - at most kNoAllocBlocks blocks of kNoAllocThreads threads, i.e. at most
//     262,144 box atoms per call; larger sizes are rejected with CASS_ECAPACITY;
//   - every call shares the one scratch array of its device: calls that
//     overlap on the GPU (different streams, or host threads racing) corrupt
//     each other's sums; serialize them;
//   - the first call on a device looks up the scratch array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture;
//   - the call is asynchronous: `out` is written on `stream`.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "cass_ctx.h"

namespace cassgpu {

constexpr int kNoAllocBlocks = 1024;
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxQuery = 64;
constexpr int kNoAllocMaxDevices = 64;

// [0]: block counter (first 4 bytes), [1]: overlap flag (first 4 bytes),
// [2 + 2*b], [3 + 2*b]: vdw and qq partial sums of block b.  16,400 bytes.
static __device__ __align__(256) double g_noalloc_scratch[2 + 2 * kNoAllocBlocks];

template <bool MIXED>
__global__ void __launch_bounds__(kNoAllocThreads)
    k_mol_box_noalloc(BoxDev b, PairTable t, const double* __restrict__ box_xyzq, const int* __restrict__ box_type,
                      const int* __restrict__ box_mol, int n, const double* __restrict__ q_xyzq,
                      const int* __restrict__ q_type, int nq, int skip_mol, int cbmc, int want_qq, double* scratch,
                      double* out) {
  __shared__ double qa[kNoAllocMaxQuery][4];
  __shared__ int qt[kNoAllocMaxQuery];
  __shared__ double sh[32];
  __shared__ bool last;
  for (int a = threadIdx.x; a < nq; a += blockDim.x) {
    for (int d = 0; d < 4; ++d) qa[a][d] = q_xyzq[4 * a + d];
    qt[a] = q_type[a] - 1;
  }
  __syncthreads();
  unsigned* counter = reinterpret_cast<unsigned*>(scratch);
  int* ovflag = reinterpret_cast<int*>(scratch + 1);
  double* partial = scratch + 2;
  double ev = 0.0, eq = 0.0;
  KahanF fv, fq;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n && box_mol[j] != skip_mol) {
    double xj = box_xyzq[4 * j], yj = box_xyzq[4 * j + 1], zj = box_xyzq[4 * j + 2], qj = box_xyzq[4 * j + 3];
    int tj = box_type[j] - 1;
    bool ov = false;
    for (int a = 0; a < nq; ++a) {
      double dx = fold(qa[a][0] - xj, b.hL[0], b.L[0]);
      double dy = fold(qa[a][1] - yj, b.hL[1], b.L[1]);
      double dz = fold(qa[a][2] - zj, b.hL[2], b.L[2]);
      double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < b.rcut_lowsq) {
        ov = true;
        continue;
      }
      int m = cutoff_mask(b, r2, cbmc != 0);
      if (!want_qq) m &= 1;
      if (m & 1) {
        if (MIXED && lj_plain_style(b) && qt[a] >= 0 && tj >= 0) {
          int k = pidx(qt[a], tj, t.ntypes);
          fv.add(lj_pair_f(t.epsf[k], t.sig2f[k], (float)r2));
        } else {
          ev += vdw_pair(t, b, qt[a], tj, r2, 1.0);
        }
      }
      if (m & 2) eq += qq_pair_inter(b, qa[a][3] * qj, r2);
    }
    if (ov) atomicOr(ovflag, 1);
  }
  // fixed-order reduction: block partials, then the last block sums them
  double v[2] = {ev + fv.value(), eq + fq.value()};
  for (int k = 0; k < 2; ++k) {
    double s = v[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += sh[w];
      partial[2 * blockIdx.x + k] = tot;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double sv = 0.0, sq = 0.0;
  for (unsigned bb = 0; bb < gridDim.x; ++bb) {
    sv += __ldcg(&partial[2 * bb]);
    sq += __ldcg(&partial[2 * bb + 1]);
  }
  int ov = __ldcg(ovflag);
  out[0] = ov ? 0.0 : sv;
  out[1] = ov ? 0.0 : sq;
  out[2] = ov ? 1.0 : 0.0;
}

}  // namespace cassgpu

using namespace cassgpu;

extern "C" int cass_mol_box_energy_noalloc(const CassBoxDesc* box, int32_t ntypes, const double* eps,
                                           const double* sig, const double* box_xyzq, const int32_t* box_type,
                                           const int32_t* box_mol, int32_t n, const double* query_xyzq,
                                           const int32_t* query_type, int32_t nq, int32_t skip_mol,
                                           int32_t cbmc_flag, int32_t l_coul_cbmc, int32_t precision, double* out,
                                           void* stream) {
  static std::mutex mu;
  static double* scratch_ptr[kNoAllocMaxDevices] = {};
  if (!box || !eps || !sig || !out || ntypes < 1 || ntypes > kMaxTypes)
    return set_error(CASS_EINVAL, "cass_mol_box_energy_noalloc: NULL argument or ntypes outside 1..8");
  if (n < 0 || n > kNoAllocBlocks * kNoAllocThreads)
    return set_error(CASS_ECAPACITY,
                     "cass_mol_box_energy_noalloc: n exceeds 262144 box atoms, the capacity of its static scratch "
                     "(1024 blocks x 256 threads)");
  if (nq < 1 || nq > kNoAllocMaxQuery)
    return set_error(CASS_ECAPACITY, "cass_mol_box_energy_noalloc: the query molecule must have 1..64 atoms");
  if ((n > 0 && (!box_xyzq || !box_type || !box_mol)) || !query_xyzq || !query_type)
    return set_error(CASS_EINVAL, "cass_mol_box_energy_noalloc: NULL device array");
  if (precision != CASS_PREC_FP64 && precision != CASS_PREC_MIXED)
    return set_error(CASS_EINVAL, "cass_mol_box_energy_noalloc: bad precision");
  if (box->vdw_style != CASS_VDW_LJ && box->vdw_style != CASS_VDW_NONE)
    return set_error(CASS_EUNSUPPORTED, "cass_mol_box_energy_noalloc: vdw style must be LJ or NONE");
  for (int k = 0; k < 3; ++k)
    if (!(box->length[k] > 0.0)) return set_error(CASS_EINVAL, "cass_mol_box_energy_noalloc: box length");
  if (box->vdw_sum_style != CASS_VDW_SUM_MINIMUM &&
      ((box->vdw_style == CASS_VDW_LJ && box->vdw_sum_style == CASS_VDW_SUM_CHARMM) ||
       (box->charge_style == CASS_CHARGE_COUL && box->charge_sum_style == CASS_QQ_MINIMUM)))
    return set_error(CASS_EUNSUPPORTED, "cass_mol_box_energy_noalloc: styles with a molecule-pair COM cutoff");
  int dev = 0;
  CASS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(CASS_EINVAL, "cass_mol_box_energy_noalloc: device");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!scratch_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
      scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = scratch_ptr[dev];
  }
  // per-call constants, passed by value to the kernel (no device copies)
  BoxDev b;
  memset(&b, 0, sizeof(b));
  for (int k = 0; k < 3; ++k) {
    b.L[k] = box->length[k];
    b.hL[k] = 0.5 * box->length[k];
    b.Lf[k] = (float)b.L[k];
    b.hLf[k] = (float)b.hL[k];
  }
  b.volume = b.L[0] * b.L[1] * b.L[2];
  b.vdw_style = box->vdw_style;
  b.vdw_sum_style = box->vdw_sum_style;
  b.charge_style = box->charge_style;
  b.charge_sum_style = box->charge_sum_style;
  double rcoul = box->charge_style == CASS_CHARGE_COUL ? box->rcut_coul : 0.0;
  b.rcut_vdw = box->rcut_vdw;
  b.rcut_coul = rcoul;
  b.rcut_vdwsq = box->rcut_vdw * box->rcut_vdw;
  b.rcut_coulsq = rcoul * rcoul;
  b.rcut_cbmcsq = box->rcut_cbmc * box->rcut_cbmc;
  b.rcut_lowsq = box->rcut_low * box->rcut_low;
  b.ron_switch_sq = box->ron_switch * box->ron_switch;
  b.roff_switch_sq = box->roff_switch * box->roff_switch;
  if (box->vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) {
    double d2 = b.roff_switch_sq - b.ron_switch_sq;
    b.switch_factor1 = 1.0 / (d2 * d2 * d2);
    b.switch_factor2 = b.roff_switch_sq - 3.0 * b.ron_switch_sq;
  }
  if (box->charge_style == CASS_CHARGE_COUL && box->charge_sum_style == CASS_QQ_EWALD) {
    if (!(box->ewald_tol > 0.0 && box->ewald_tol < 1.0))
      return set_error(CASS_EINVAL, "cass_mol_box_energy_noalloc: ewald_tol must be in (0,1)");
    b.alpha = std::sqrt(-std::log(box->ewald_tol)) / rcoul;
  }
  if (box->charge_style == CASS_CHARGE_COUL && box->charge_sum_style == CASS_QQ_DSF) {
    double a = box->alpha_dsf;
    if (a <= 0.0) {
      a = 0.425 - rcoul * 0.02;
      if (a < 0.0) a = 3.3930702 / rcoul;
    }
    b.alpha_dsf = a;
    b.dsf_factor1 = std::erfc(a * rcoul) / rcoul;
    b.dsf_factor2 = b.dsf_factor1 / rcoul + 2.0 * a * std::exp(-a * a * rcoul * rcoul) / (kROOTPI * rcoul);
  }
  PairTable t;
  memset(&t, 0, sizeof(t));
  t.ntypes = ntypes;
  for (int i = 0; i < ntypes * ntypes; ++i) {
    t.eps[i] = eps[i];
    t.sig2[i] = sig[i] * sig[i];
    t.epsf[i] = (float)t.eps[i];
    t.sig2f[i] = (float)t.sig2[i];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the counter and the overlap flag must start at zero; the partials are
  // overwritten by every block before the last block reads them
  CASS_CUDA(cudaMemsetAsync(scratch, 0, 2 * sizeof(double), st));
  int want_qq = (cbmc_flag && !l_coul_cbmc) ? 0 : 1;
  int nblk = n > 0 ? (n + kNoAllocThreads - 1) / kNoAllocThreads : 1;
  if (precision == CASS_PREC_MIXED)
    k_mol_box_noalloc<true><<<nblk, kNoAllocThreads, 0, st>>>(b, t, box_xyzq, box_type, box_mol, n, query_xyzq,
                                                              query_type, nq, skip_mol, cbmc_flag, want_qq, scratch,
                                                              out);
  else
    k_mol_box_noalloc<false><<<nblk, kNoAllocThreads, 0, st>>>(b, t, box_xyzq, box_type, box_mol, n, query_xyzq,
                                                               query_type, nq, skip_mol, cbmc_flag, want_qq, scratch,
                                                               out);
  CASS_CUDA(cudaGetLastError());
  return CASS_OK;
}
