// k_mc.cu -- NVT Monte Carlo sweeps on the device (translation / rotation).
//
// One CTA runs one box's Markov chain for the whole call: the box's atoms,
// charges, types and molecule table live in shared memory, thread 0 owns the
// lfsr258 stream and makes every random choice in the reference's order, and
// the block evaluates each move's energies cooperatively:
//   A  thread 0: move kind (nvtmc_driver.f90:107-134), species and molecule
//      (move_translate.f90:150-185), trial coordinates (:205-215 and Fold_Molecule,
//      or Rotate_Molecule_Axis / Rotate_Molecule_Eulerian, move_rotate.f90:362-536)
//   B  all threads: the moved molecule's old and trial energies against every
//      other atom in one pass (Compute_Molecule_Nonbond_Inter_Energy twice,
//      energy_routines.f90:1088-1206), block reduction
//   C  all threads, charged species in Ewald boxes: the molecule's new
//      cos/sin sums per k-vector and the new reciprocal energy
//      (Update_System_Ewald_Reciprocal_Energy, :2384-2431)
//   D  thread 0: accept_or_reject (accept_or_reject.f90:22-65), energy
//      bookkeeping, step-size adaptation (move_translate.f90:330-352,
//      move_rotate.f90:307-326)
//   E  on acceptance: coordinates, COM and structure factors are committed.
// FP64 kernel: the reference arithmetic.  Mixed kernel: FP32 positions for the
// pair loop, FP32 phases for the structure factors and the FP32 change of the
// reciprocal energy, Cn [dc (2 S_c + dc) + ds (2 S_s + ds)] summed per thread
// with compensation; the master coordinates, the running structure factors, the
// energy bookkeeping and the acceptance exponent stay FP64.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cass_cbmc_f.cuh"
#include "cass_ctx.h"

namespace cassgpu {

constexpr int kMcThreads = 128;
constexpr int kMcWarps = kMcThreads / 32;
constexpr int kMcThreadsG = 512;  // boxes in global memory: more lanes for their longer loops
constexpr int kMaxSpeciesMC = 8;
constexpr size_t kMcSmemLimit = 200 * 1024;

struct McSpecies {
  int natoms, linear, has_charge;
  double mass[kMaxAtoms];
};

// per-call constants
struct McArgs {
  int nspecies;
  McSpecies sp[kMaxSpeciesMC];
  long long nsweeps;
  int steps_per_sweep, nupdate;
  double prob_translate, target_accept;
  uint64_t seed;
  double* cos_mol;  // [slot][stride]
  double* sin_mol;
  int stride;
};

// per-box inputs and outputs
struct McBox {
  BoxDev b;
  double4_32a* p64;  // packed atoms x, y, z, q (updated at the end)
  float4* p32;       // x, y, z, type bits (updated at the end)
  const int4* meta;  // slot, type, species, atom index in species
  const int4* molinfo;  // slot, species, first atom, natoms
  int natoms, nmols, ibox1;
  int nmol_sp[kMaxSpeciesMC], first_sp[kMaxSpeciesMC];
  const double4_32a* kvec;  // hx, hy, hz, Cn
  double* cos_sum;
  double* sin_sum;
  double* new_cos;  // scratch [nvecs]
  double* new_sin;
  int nvecs, ewald;
  // Check_MoleculePair_Cutoff decides which molecule pairs interact (LJ CHARMM,
  // minimum-image charges): COM distance against rmax + both max_dcom
  int comcut;
  double rmax;
  double* max_disp;   // [nspecies] in/out
  double* max_rot;
  CassEnergy* energy;  // in/out
  CassMCResult* res;   // out
  int* status;         // out: 0 ok, 1 overlapping molecule before a move
  unsigned char* gbox; // the box layout in global memory (boxes too large for shared memory),
  size_t gbox_stride;  // one copy per CTA of the box's cluster, this many bytes apart
};

// the move thread 0 prepared for the block
struct McMove {
  int skip, stop, kind, is, pm, na, first, slot, accept, ewald;
  double old_r[3 * kMaxAtoms], trial[3 * kMaxAtoms], q[kMaxAtoms];
  int type[kMaxAtoms];
  float old_f[3 * kMaxAtoms], trial_f[3 * kMaxAtoms];
  double com_new[3];
};

__device__ __forceinline__ bool accept_or_reject_d(double ln_pacc, Lfsr& rng) {
  if (ln_pacc <= 0.0) return true;
  if (ln_pacc < kMAX_KBT) {
    const double u = rng.next();
    // exp(-ln_pacc) in FP32 first (FP64 issues at 1/64 of the FP32 rate): with
    // ln_pacc < 80 rounded to FP32 the value is within 6e-6 relative, so a
    // draw outside a band of 2e-5 about it is decided as in FP64
    if (ln_pacc < 80.0) {
      const float e = expf(-(float)ln_pacc), uf = (float)u;
      if (uf < e * 0.99998f) return true;
      if (uf > e * 1.00002f) return false;
    }
    return u <= exp(-ln_pacc);
  }
  return false;
}

// cumulative species fractions x_species of Translate / Rotate
// (move_translate.f90:150-165): species with a zero step do not move.  The
// adaptation keeps nonzero steps nonzero, so they are fixed for a call.
// Returns false when no species moves.
__device__ bool mc_species_cdf(const McBox& G, int nspecies, const double* step, double* x, int* last) {
  int ntot = 0;
  for (int is = 0; is < nspecies; ++is)
    if (step[is] > 0.0) ntot += G.nmol_sp[is];
  *last = 0;
  if (ntot == 0) return false;
  double c = 0.0;
  for (int is = 0; is < nspecies; ++is) {
    c = (step[is] > 0.0 ? (double)G.nmol_sp[is] / (double)ntot : 0.0) + (is > 0 ? c : 0.0);
    x[is] = c;
    if (step[is] > 0.0 && G.nmol_sp[is] > 0) *last = is;
  }
  return true;
}

// species choice: the first with rranf() <= x_species(is); the last movable
// species when rounding leaves u above the final sum
__device__ __forceinline__ int mc_pick_species(int nspecies, const double* x, int last, Lfsr& rng) {
  const double u = rng.next();
  for (int is = 0; is < nspecies; ++is)
    if (u <= x[is]) return is;
  return last;
}

// the mixed kernel's serial draws: the top 23 bits of the same lfsr258 numbers
// (draw_f), without the FP64 unit, which on this GPU holds a warp's FP64
// instruction for many cycles even when one lane issues it
__device__ __forceinline__ int mc_pick_species_f(int nspecies, const float* x, int last, Lfsr& rng) {
  const float u = draw_f(rng);
  for (int is = 0; is < nspecies; ++is)
    if (u <= x[is]) return is;
  return last;
}

template <bool MIXED>
__device__ __forceinline__ double mc_u(Lfsr& rng) {
  if constexpr (MIXED) return (double)draw_f(rng);
  else return rng.next();
}

// (s, c) += (s', c') for compensated FP32 sums: the rounding error of s + s'
// (TwoSum, exact in FP32) joins the correction terms
__device__ __forceinline__ void two_sum_add(float2& a, const float2 b) {
  const float t = a.x + b.x;
  const float bp = t - a.x;
  const float e = (a.x - (t - bp)) + (b.x - bp);
  a.x = t;
  a.y = (a.y + b.y) + e;
}

// warp sum of compensated FP32 pairs, butterfly order (lane 0's is fixed)
__device__ __forceinline__ float2 warp_sum2(float2 v) {
  for (int o = 16; o > 0; o >>= 1) {
    const float2 u = make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
    two_sum_add(v, u);
  }
  return v;
}

template <class V>
__device__ __forceinline__ V block_sum_mc(V v, V* red, int slot) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[(threadIdx.x >> 5) * 8 + slot] = v;
  return v;
}

// Sums over the CTAs of a box's cluster, in rank order, of the nd doubles and
// ni ints that thread 0 of every CTA placed in cd[buf] / ci[buf]; the results
// land in the same arrays of every CTA's thread 0 view.  Two buffers alternate,
// so a buffer is written again only after every CTA passed the barrier that
// followed its last read.  Thread 0 only reads; all threads take the barrier.
__device__ __forceinline__ void cluster_sum(int csize, double (*cd)[4], int (*ci)[2], int buf, int nd, int ni,
                                            double* od, int* oi) {
  namespace cgr = cooperative_groups;
  cgr::cluster_group cl = cgr::this_cluster();
  cl.sync();
  if (threadIdx.x == 0) {
    for (int k = 0; k < nd; ++k) {
      double v = 0.0;
      for (int r = 0; r < csize; ++r) v += *cl.map_shared_rank(&cd[buf][k], r);
      od[k] = v;
    }
    for (int k = 0; k < ni; ++k) {
      int v = 0;
      for (int r = 0; r < csize; ++r) v |= *cl.map_shared_rank(&ci[buf][k], r);
      oi[k] = v;
    }
  }
}

// GMEM: the box layout lives in a per-box global buffer (L2-resident) instead
// of shared memory, for boxes above the shared-memory limit; same code.
// csize > 1: a thread-block cluster of csize CTAs runs one box's chain (a box
// in global memory has one layout copy per CTA).  Every CTA holds the whole box and makes the same
// serial decisions from the same lfsr258 stream; the pair loop over the box
// atoms and the k-vector loop are split over the CTAs, whose partial sums are
// added in rank order through distributed shared memory, and each CTA commits
// the structure factors of its own k-vectors.
template <bool MIXED, bool GMEM>
__global__ void __launch_bounds__(GMEM ? kMcThreadsG : kMcThreads) k_mc_sweeps(McArgs A, McBox* boxes, PairTable T,
                                                                           int csize) {
  constexpr int NW = (GMEM ? kMcThreadsG : kMcThreads) / 32;
  const int nwarps = blockDim.x >> 5;  // <= NW
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ BoxDev b;
  __shared__ McMove mv;
  __shared__ double red[NW * 8];
  __shared__ float redf[NW * 4];  // mixed kernel: compensated FP32 pair sums per warp
  __shared__ int redi[NW * 2];
  __shared__ float2 ljp[kMaxTypes * kMaxTypes];
  __shared__ double cd[2][4];  // this CTA's partial sums for the cluster (alternating buffers)
  __shared__ int ci[2][2];
  __shared__ McBox G;  // the box descriptor, read by the serial steps of every move
  const int crank = (int)(blockIdx.x % (unsigned)csize);
  int cbuf = 0;
  if (threadIdx.x == 0) {
    G = boxes[blockIdx.x / csize];
    b = G.b;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kMaxTypes * kMaxTypes; i += blockDim.x) {
    const int a = i / kMaxTypes, c = i % kMaxTypes;
    const bool ok = a < T.ntypes && c < T.ntypes;
    ljp[i] = ok ? make_float2(T.epsf[a * T.ntypes + c], T.sig2f[a * T.ntypes + c]) : make_float2(0.f, 0.f);
  }
  const int N = G.natoms, M = G.nmols;
  unsigned char* smem = GMEM ? G.gbox + (size_t)crank * G.gbox_stride : dsmem;
  // shared layout: x y z q (double), type, mol (int), [x y z type (float4), q (float)], COM (double x3), first, nat
  double* sx = reinterpret_cast<double*>(smem);
  double* sy = sx + N;
  double* sz = sy + N;
  double* sq = sz + N;
  double* com = sq + N;  // [M][3]
  double* dcom = com + 3 * M;  // [M] max_dcom (Compute_Max_Com_Distance, get_com.f90:220-295)
  int* stype = reinterpret_cast<int*>(dcom + M);
  int* smol = stype + N;
  int* mfirst = smol + N;
  int* mnat = mfirst + M;
  int* mslot = mnat + M;  // molecule slot (the cos_mol / sin_mol row)
  float4* s32 = reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(smem) +
                                          ((((size_t)(mslot + M) - (size_t)smem) + 15) & ~(size_t)15));
  float* sq32 = reinterpret_cast<float*>(s32 + (MIXED ? N : 0));
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const double4_32a p = G.p64[j];
    sx[j] = p.x;
    sy[j] = p.y;
    sz[j] = p.z;
    sq[j] = p.w;
    stype[j] = G.meta[j].y;
    if (MIXED) {
      s32[j] = G.p32[j];
      sq32[j] = (float)p.w;
    }
  }
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const int4 mi = G.molinfo[m];
    mfirst[m] = mi.z;
    mnat[m] = mi.w;
    mslot[m] = mi.x;
    for (int a = 0; a < mi.w; ++a) smol[mi.z + a] = m;
  }
  __syncthreads();
  // Get_COM (get_com.f90:45-105) of every molecule
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const McSpecies& s = A.sp[G.molinfo[m].y];
    double tm = 0, x = 0, y = 0, z = 0;
    for (int a = 0; a < mnat[m]; ++a) {
      const int j = mfirst[m] + a;
      tm += s.mass[a];
      x += s.mass[a] * sx[j];
      y += s.mass[a] * sy[j];
      z += s.mass[a] * sz[j];
    }
    com[3 * m] = x / tm;
    com[3 * m + 1] = y / tm;
    com[3 * m + 2] = z / tm;
    double dmax = 0.0;  // rigid moves keep it
    for (int a = 0; a < mnat[m]; ++a) {
      const int j = mfirst[m] + a;
      const double dx = sx[j] - com[3 * m], dy = sy[j] - com[3 * m + 1], dz = sz[j] - com[3 * m + 2];
      dmax = fmax(dmax, dx * dx + dy * dy + dz * dz);
    }
    dcom[m] = sqrt(dmax);
  }
  // thread 0 state
  Lfsr rng;
  CassEnergy E;
  CassMCResult R;
  double md[kMaxSpeciesMC], mr[kMaxSpeciesMC], xd[kMaxSpeciesMC], xr[kMaxSpeciesMC];
  float mdf[kMaxSpeciesMC], xdf[kMaxSpeciesMC], xrf[kMaxSpeciesMC];  // mixed kernel: FP32 copies
  int nt_d[kMaxSpeciesMC], ns_d[kMaxSpeciesMC], nt_r[kMaxSpeciesMC], ns_r[kMaxSpeciesMC];
  int last_d = 0, last_r = 0;
  bool any_d = false, any_r = false;
  double dv = 0, dq = 0;
  // mixed kernel, one CTA and no k-space work: the move's energy change as
  // compensated FP32 pairs and its acceptance decided in FP32 (FP64 only for
  // the bookkeeping of an accepted move)
  float2 dv2 = make_float2(0.f, 0.f), dq2 = make_float2(0.f, 0.f);
  bool fast = false;
  float ptf = 1.0f, betaf = 0.0f;
  if (threadIdx.x == 0) {
    rng = seed_stream(A.seed, G.ibox1, 0);
    E = *G.energy;
    memset(&R, 0, sizeof(R));
    for (int is = 0; is < A.nspecies; ++is) {
      md[is] = G.max_disp[is];
      mr[is] = G.max_rot[is];
      nt_d[is] = ns_d[is] = nt_r[is] = ns_r[is] = 0;
    }
    any_d = mc_species_cdf(G, A.nspecies, md, xd, &last_d);
    any_r = mc_species_cdf(G, A.nspecies, mr, xr, &last_r);
    if (MIXED) {
      for (int is = 0; is < A.nspecies; ++is) {
        mdf[is] = (float)md[is];
        xdf[is] = (float)xd[is];
        xrf[is] = (float)xr[is];
      }
      ptf = (float)A.prob_translate;
      betaf = (float)b.beta;
    }
  }
  const long long steps = A.nsweeps * (long long)(A.steps_per_sweep > 0 ? A.steps_per_sweep : M);
  int status = 0;
  __syncthreads();
  for (long long step = 0; step < steps; ++step) {
    // ---- A: the move
    if (threadIdx.x == 0) {
      mv.skip = 0;
      mv.stop = 0;
      mv.accept = 0;
      const bool tr = MIXED ? draw_f(rng) <= ptf : rng.next() <= A.prob_translate;
      mv.kind = tr ? 0 : 1;
      int is = -1;
      if (tr ? any_d : any_r)
        is = MIXED ? mc_pick_species_f(A.nspecies, tr ? xdf : xrf, tr ? last_d : last_r, rng)
                   : mc_pick_species(A.nspecies, tr ? xd : xr, tr ? last_d : last_r, rng);
      if (is < 0) {
        mv.skip = 1;
      } else {
        // INT(rranf() * nmols) + 1, kept in range when rranf() rounds to 1.0
        const int im = MIXED ? min((int)(draw_f(rng) * (float)G.nmol_sp[is]) + 1, G.nmol_sp[is])
                             : min((int)(rng.next() * G.nmol_sp[is]) + 1, G.nmol_sp[is]);
        const int pm = G.first_sp[is] + im - 1;
        const McSpecies& s = A.sp[is];
        mv.is = is;
        mv.pm = pm;
        mv.na = mnat[pm];
        mv.first = mfirst[pm];
        mv.slot = mslot[pm];
        mv.ewald = G.ewald && s.has_charge;
        for (int a = 0; a < mv.na; ++a) {
          const int j = mv.first + a;
          mv.old_r[3 * a] = sx[j];
          mv.old_r[3 * a + 1] = sy[j];
          mv.old_r[3 * a + 2] = sz[j];
          if (MIXED) {  // (float) of the FP64 position, kept so at every commit
            const float4 f = s32[j];
            mv.old_f[3 * a] = f.x;
            mv.old_f[3 * a + 1] = f.y;
            mv.old_f[3 * a + 2] = f.z;
          }
          mv.q[a] = sq[j];
          mv.type[a] = stype[j];
        }
        const double c0 = com[3 * pm], c1 = com[3 * pm + 1], c2 = com[3 * pm + 2];
        if (tr) {
          ++R.n_translate;
          if (A.nupdate > 0) ++nt_d[is];
          double d[3];
          if (MIXED)
            for (int k = 0; k < 3; ++k) d[k] = (double)((2.0f * draw_f(rng) - 1.0f) * mdf[is]);
          else
            for (int k = 0; k < 3; ++k) d[k] = (2.0 * rng.next() - 1.0) * md[is];
          double cn[3] = {c0 + d[0], c1 + d[1], c2 + d[2]};
          double sh[3];
          for (int k = 0; k < 3; ++k) {  // Fold_Molecule
            sh[k] = cn[k] > b.hL[k] ? -b.L[k] : (cn[k] < -b.hL[k] ? b.L[k] : 0.0);
            cn[k] = cn[k] + sh[k];
          }
          for (int a = 0; a < mv.na; ++a)
            for (int k = 0; k < 3; ++k) {
              double v = mv.old_r[3 * a + k] + d[k];
              if (sh[k] != 0.0) v = v + sh[k];
              mv.trial[3 * a + k] = v;
            }
          for (int k = 0; k < 3; ++k) mv.com_new[k] = cn[k];
        } else {
          ++R.n_rotate;
          if (A.nupdate > 0) ++nt_r[is];
          double Rm[9];
          if (s.linear) {
            const double theta = acos(1.0 - 2.0 * mc_u<MIXED>(rng));
            const double phi = (1.0 - 2.0 * mc_u<MIXED>(rng)) * kPI;
            const double psi = (1.0 - 2.0 * mc_u<MIXED>(rng)) * kPI;
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
            double p1 = 0.0, p2 = 0.0, p3 = 0.0;
            const int axis = (int)(3.0 * mc_u<MIXED>(rng)) + 1;
            const double ang = (2.0 * mc_u<MIXED>(rng) - 1.0) * mr[is];
            if (axis == 1) p1 = ang;
            else if (axis == 2) p2 = ang;
            else p3 = ang;
            // DCOS / DSIN of the two zero angles are exactly 1 and 0
            double k1 = 1.0, k2 = 1.0, k3 = 1.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            if (axis == 1) sincos(p1, &s1, &k1);
            else if (axis == 2) sincos(p2, &s2, &k2);
            else sincos(p3, &s3, &k3);
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
          for (int a = 0; a < mv.na; ++a) {
            const double x = mv.old_r[3 * a] - c0, y = mv.old_r[3 * a + 1] - c1, z = mv.old_r[3 * a + 2] - c2;
            mv.trial[3 * a] = (Rm[0] * x + Rm[1] * y + Rm[2] * z) + c0;
            mv.trial[3 * a + 1] = (Rm[3] * x + Rm[4] * y + Rm[5] * z) + c1;
            mv.trial[3 * a + 2] = (Rm[6] * x + Rm[7] * y + Rm[8] * z) + c2;
          }
          mv.com_new[0] = c0;
          mv.com_new[1] = c1;
          mv.com_new[2] = c2;
        }
        if (MIXED)
          for (int i = 0; i < 3 * mv.na; ++i) mv.trial_f[i] = (float)mv.trial[i];
      }
    }
    __syncthreads();
    if (mv.skip) {  // uniform: no species can make this kind of move
      __syncthreads();
      continue;
    }
    // ---- B: old and trial energies of the molecule against the other atoms
    const int pm = mv.pm, na = mv.na;
    double pdv = 0, pdq = 0;  // this thread's share of E_new - E_old
    float2 pv2 = make_float2(0.f, 0.f), pq2 = make_float2(0.f, 0.f);  // the same, mixed kernel
    int po = 0, pn = 0;
    const int j0 = threadIdx.x + crank * blockDim.x, jstep = blockDim.x * csize;
    if (MIXED) {
      KahanF kv, kq;
      const float rv2 = (float)b.rcut_vdwsq, rq2 = (float)b.rcut_coulsq, low2 = (float)b.rcut_lowsq;
      const float alpha = (float)b.alpha;
      const bool qq_on = b.charge_style == CASS_CHARGE_COUL;
      for (int j = j0; j < N; j += jstep) {
        if (smol[j] == pm) continue;
        const float4 pj = s32[j];
        const int tj = __float_as_int(pj.w);
        const float qj = sq32[j];
        for (int a = 0; a < na; ++a) {
          const int ta = mv.type[a];
          const float2 es = (ta >= 0 && tj >= 0) ? ljp[ta * kMaxTypes + tj] : make_float2(0.f, 0.f);
          const float qq = (float)mv.q[a] * qj;
          float ev[2] = {0.0f, 0.0f}, eq[2] = {0.0f, 0.0f};
#pragma unroll
          for (int w = 0; w < 2; ++w) {
            const float* r = w ? mv.trial_f : mv.old_f;
            const float dx = fold(r[3 * a] - pj.x, b.hLf[0], b.Lf[0]);
            const float dy = fold(r[3 * a + 1] - pj.y, b.hLf[1], b.Lf[1]);
            const float dz = fold(r[3 * a + 2] - pj.z, b.hLf[2], b.Lf[2]);
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (r2 < low2) {
              if (w) pn = 1;
              else po = 1;
              continue;
            }
            if (r2 <= rv2 && es.x != 0.0f) ev[w] = lj_pair_f(es.x, es.y, r2);
            if (qq_on && r2 <= rq2 && qq != 0.0f) eq[w] = qq_ewald_inter_f(alpha, qq, r2);
          }
          kv.add(ev[1] - ev[0]);
          kq.add(eq[1] - eq[0]);
        }
      }
      pv2 = make_float2(kv.s, kv.c);
      pq2 = make_float2(kq.s, kq.c);
    } else {
      for (int j = j0; j < N; j += jstep) {
        const int mj = smol[j];
        if (mj == pm) continue;
        const double xj = sx[j], yj = sy[j], zj = sz[j], qj = sq[j];
        const int tj = stype[j];
        bool in[2] = {true, true};
        if (G.comcut)  // Check_MoleculePair_Cutoff (energy_routines.f90:3027-3088), old and trial COM
#pragma unroll
          for (int w = 0; w < 2; ++w) {
            const double* cw = w ? mv.com_new : com + 3 * pm;
            const double dx = fold(cw[0] - com[3 * mj], b.hL[0], b.L[0]);
            const double dy = fold(cw[1] - com[3 * mj + 1], b.hL[1], b.L[1]);
            const double dz = fold(cw[2] - com[3 * mj + 2], b.hL[2], b.L[2]);
            in[w] = !(sqrt(dx * dx + dy * dy + dz * dz) > G.rmax + dcom[pm] + dcom[mj]);
          }
        for (int a = 0; a < na; ++a) {
#pragma unroll
          for (int w = 0; w < 2; ++w) {
            if (!in[w]) continue;
            const double* r = w ? mv.trial : mv.old_r;
            const double dx = fold(r[3 * a] - xj, b.hL[0], b.L[0]);
            const double dy = fold(r[3 * a + 1] - yj, b.hL[1], b.L[1]);
            const double dz = fold(r[3 * a + 2] - zj, b.hL[2], b.L[2]);
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < b.rcut_lowsq) {
              if (w) pn = 1;
              else po = 1;
              continue;
            }
            const int m = cutoff_mask(b, r2, false);
            const double sg = w ? 1.0 : -1.0;
            if (m & 1) pdv += sg * vdw_pair(T, b, mv.type[a], tj, r2, 1.0);
            if (m & 2) pdq += sg * qq_pair_inter(b, mv.q[a] * qj, r2);
          }
        }
      }
    }
    if (MIXED) {  // compensated FP32 warp sums (no FP64 instructions in any warp)
      pv2 = warp_sum2(pv2);
      pq2 = warp_sum2(pq2);
      if ((threadIdx.x & 31) == 0) {
        const int w = threadIdx.x >> 5;
        redf[4 * w] = pv2.x;
        redf[4 * w + 1] = pv2.y;
        redf[4 * w + 2] = pq2.x;
        redf[4 * w + 3] = pq2.y;
      }
    } else {
      block_sum_mc(pdv, red, 0);
      block_sum_mc(pdq, red, 1);
    }
    {
      const int o = __any_sync(0xffffffffu, po), n = __any_sync(0xffffffffu, pn);
      if ((threadIdx.x & 31) == 0) {
        redi[(threadIdx.x >> 5) * 2] = o;
        redi[(threadIdx.x >> 5) * 2 + 1] = n;
      }
    }
    __syncthreads();
    int o = 0, n = 0;
    if (threadIdx.x == 0) {
      if (MIXED) {
        dv2 = dq2 = make_float2(0.f, 0.f);
        for (int w = 0; w < nwarps; ++w) {
          two_sum_add(dv2, make_float2(redf[4 * w], redf[4 * w + 1]));
          two_sum_add(dq2, make_float2(redf[4 * w + 2], redf[4 * w + 3]));
          o |= redi[2 * w];
          n |= redi[2 * w + 1];
        }
        fast = csize == 1 && !mv.ewald;
        if (!fast) {
          dv = (double)dv2.x + (double)dv2.y;
          dq = (double)dq2.x + (double)dq2.y;
        }
      } else {
        dv = dq = 0.0;
        for (int w = 0; w < nwarps; ++w) {
          dv += red[w * 8];
          dq += red[w * 8 + 1];
          o |= redi[2 * w];
          n |= redi[2 * w + 1];
        }
      }
      if (csize > 1) {
        cd[cbuf][0] = dv;
        cd[cbuf][1] = dq;
        ci[cbuf][0] = o;
        ci[cbuf][1] = n;
      }
    }
    if (csize > 1) {
      double sums[2];
      int flags[2];
      cluster_sum(csize, cd, ci, cbuf, 2, 2, sums, flags);
      cbuf ^= 1;
      if (threadIdx.x == 0) {
        dv = sums[0];
        dq = sums[1];
        o = flags[0];
        n = flags[1];
      }
    }
    if (threadIdx.x == 0) {
      if (o) {
        mv.stop = 1;
        status = 1;
      } else if (n) {
        ++R.n_overlap;
        mv.ewald = 0;
      }
      mv.accept = (!o && !n) ? 1 : 0;  // provisional: energies valid
    }
    __syncthreads();
    if (mv.stop) break;
    // ---- C: reciprocal-space energy after the move
    double e_recip = 0.0;
    if (mv.ewald) {
      const double* cm = A.cos_mol + (size_t)mv.slot * A.stride;
      const double* smv = A.sin_mol + (size_t)mv.slot * A.stride;
      double part = 0.0;
      KahanF partf;
      for (int k = threadIdx.x + crank * blockDim.x; k < G.nvecs; k += blockDim.x * csize) {
        const double4_32a h = G.kvec[k];
        double cn = 0.0, sn = 0.0;
        if (MIXED) {
          float cf = 0.0f, sf = 0.0f;
          const float hx = (float)h.x, hy = (float)h.y, hz = (float)h.z;
          for (int a = 0; a < na; ++a) {
            float s_, c_;
            sincosf(hx * mv.trial_f[3 * a] + hy * mv.trial_f[3 * a + 1] + hz * mv.trial_f[3 * a + 2], &s_, &c_);
            cf += (float)mv.q[a] * c_;
            sf += (float)mv.q[a] * s_;
          }
          cn = (double)cf;
          sn = (double)sf;
        } else {
          for (int a = 0; a < na; ++a) {
            const double hdotr = h.x * mv.trial[3 * a] + h.y * mv.trial[3 * a + 1] + h.z * mv.trial[3 * a + 2];
            cn = cn + mv.q[a] * cos(hdotr);
            sn = sn + mv.q[a] * sin(hdotr);
          }
        }
        if (MIXED) {
          // the change of Cn (S_c^2 + S_s^2) in FP32: dc (2 S_c + dc) + ds (2 S_s + ds)
          const float dc = (float)cn - (float)cm[k], ds = (float)sn - (float)smv[k];
          const float sc = (float)G.cos_sum[k], ss = (float)G.sin_sum[k];
          partf.add((float)h.w * (dc * (2.0f * sc + dc) + ds * (2.0f * ss + ds)));
        } else {
          const double c = G.cos_sum[k] + (cn - cm[k]);
          const double s = G.sin_sum[k] + (sn - smv[k]);
          part += h.w * (c * c + s * s);
        }
        G.new_cos[k] = cn;
        G.new_sin[k] = sn;
      }
      if (MIXED) part = partf.value();
      block_sum_mc(part, red, 4);
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int w = 0; w < nwarps; ++w) e_recip += red[w * 8 + 4];
        if (csize > 1) cd[cbuf][0] = e_recip;
      }
      if (csize > 1) {
        double sums[1];
        cluster_sum(csize, cd, ci, cbuf, 1, 0, sums, nullptr);
        cbuf ^= 1;
        if (threadIdx.x == 0) e_recip = sums[0];
      }
      if (threadIdx.x == 0)  // mixed: the previous reciprocal energy plus the FP32 change (FP64 sum)
        e_recip = MIXED ? E.reciprocal + e_recip * kCHARGE_FACTOR : e_recip * kCHARGE_FACTOR;
    }
    // ---- D: acceptance
    if (threadIdx.x == 0) {
      bool acc = false;
      if (mv.accept && MIXED && fast) {
        // accept_or_reject in FP32 (the rule of accept_or_reject.f90:22-65 with
        // a 23-bit draw); the bookkeeping of an accepted move in FP64
        const float lnf = betaf * ((dv2.x + dq2.x) + (dv2.y + dq2.y));
        acc = lnf <= 0.0f || (lnf < (float)kMAX_KBT && draw_f(rng) <= expf(-lnf));
        if (acc) {
          dv = (double)dv2.x + (double)dv2.y;
          dq = (double)dq2.x + (double)dq2.y;
          const double dE = dv + dq;
          E.total = E.total + dE;
          E.inter = E.inter + dE;
          E.inter_vdw = E.inter_vdw + dv;
          E.inter_q = E.inter_q + dq;
        }
      } else if (mv.accept) {
        double dE = 0.0;
        if (mv.ewald) dE = e_recip - E.reciprocal;
        dE = dE + dv + dq;
        acc = accept_or_reject_d(b.beta * dE, rng);
        if (acc) {
          E.total = E.total + dE;
          E.inter = E.inter + dE;
          E.inter_vdw = E.inter_vdw + dv;
          E.inter_q = E.inter_q + dq;
          if (mv.ewald) E.reciprocal = e_recip;
        }
      }
      mv.accept = acc ? 1 : 0;
      const int is = mv.is;
      if (mv.kind == 0) {
        if (acc) {
          ++R.n_translate_accepted;
          ++ns_d[is];
        }
        if (A.nupdate > 0 && nt_d[is] == A.nupdate) {  // every nupdate trials of the species
          nt_d[is] = 0;
          const double ratio = (double)ns_d[is] / (double)A.nupdate;
          ns_d[is] = 0;
          // rcut_small of move_translate.f90:341-346
          const double rsmall = (A.sp[is].has_charge && b.charge_style != CASS_CHARGE_NONE)
                                    ? fmin(b.rcut_vdw, b.rcut_coul) : b.rcut_vdw;
          if (ratio < 0.00005) md[is] = 0.1 * md[is];
          else md[is] = fmin(rsmall, ratio / A.target_accept * md[is]);
          if (MIXED) mdf[is] = (float)md[is];
        }
      } else {
        if (acc) {
          ++R.n_rotate_accepted;
          ++ns_r[is];
        }
        if (A.nupdate > 0 && nt_r[is] == A.nupdate) {
          nt_r[is] = 0;
          const double ratio = (double)ns_r[is] / (double)A.nupdate;
          ns_r[is] = 0;
          if (ratio < 0.5) mr[is] = fmax(0.01, 0.95 * mr[is]);
          else mr[is] = fmin(kPI, 1.05 * mr[is]);
        }
      }
      if (acc) {  // commit the coordinates and the COM
        for (int a = 0; a < na; ++a) {
          const int j = mv.first + a;
          sx[j] = mv.trial[3 * a];
          sy[j] = mv.trial[3 * a + 1];
          sz[j] = mv.trial[3 * a + 2];
          if (MIXED) s32[j] = make_float4(mv.trial_f[3 * a], mv.trial_f[3 * a + 1], mv.trial_f[3 * a + 2], s32[j].w);
        }
        if (mv.kind == 0) {
          for (int k = 0; k < 3; ++k) com[3 * pm + k] = mv.com_new[k];
        } else {  // Get_COM on acceptance of a rotation
          const McSpecies& s = A.sp[is];
          double tm = 0, x = 0, y = 0, z = 0;
          for (int a = 0; a < na; ++a) {
            tm += s.mass[a];
            x += s.mass[a] * mv.trial[3 * a];
            y += s.mass[a] * mv.trial[3 * a + 1];
            z += s.mass[a] * mv.trial[3 * a + 2];
          }
          com[3 * pm] = x / tm;
          com[3 * pm + 1] = y / tm;
          com[3 * pm + 2] = z / tm;
        }
      }
    }
    __syncthreads();
    // ---- E: commit the structure factors
    if (mv.accept && mv.ewald) {
      double* cm = A.cos_mol + (size_t)mv.slot * A.stride;
      double* smv = A.sin_mol + (size_t)mv.slot * A.stride;
      for (int k = threadIdx.x + crank * blockDim.x; k < G.nvecs; k += blockDim.x * csize) {
        const double cn = G.new_cos[k], sn = G.new_sin[k];
        G.cos_sum[k] = G.cos_sum[k] + (cn - cm[k]);
        G.sin_sum[k] = G.sin_sum[k] + (sn - smv[k]);
        cm[k] = cn;
        smv[k] = sn;
      }
    }
    // the next move's thread-0 phase reads committed shared data only
    __syncthreads();
  }
  __syncthreads();
  if (csize > 1) cooperative_groups::this_cluster().sync();  // no CTA leaves while its shared memory may be read
  if (crank != 0) return;  // every CTA of the cluster holds the same state
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    G.p64[j] = make_double4_32a(sx[j], sy[j], sz[j], sq[j]);
    float4 f = G.p32[j];
    G.p32[j] = make_float4((float)sx[j], (float)sy[j], (float)sz[j], f.w);
  }
  if (threadIdx.x == 0) {
    R.energy = E;
    *G.res = R;
    *G.energy = E;
    *G.status = status;
    for (int is = 0; is < A.nspecies; ++is) {
      G.max_disp[is] = md[is];
      G.max_rot[is] = mr[is];
    }
  }
}

size_t mc_smem_bytes(int natoms, int nmols, bool mixed) {
  size_t s = (size_t)natoms * (4 * sizeof(double) + 2 * sizeof(int)) + (size_t)nmols * (4 * sizeof(double) + 3 * sizeof(int));
  s = (s + 15) & ~(size_t)15;
  if (mixed) s += (size_t)natoms * (sizeof(float4) + sizeof(float));
  return s;
}

int pack_box_ext(cass_ctx* c, int ibox);
const std::vector<int>& members_ext(cass_ctx* c, int ibox);
int ensure_pools(cass_ctx* c);

}  // namespace cassgpu

using namespace cassgpu;

extern "C" int cass_mc_sweeps(cass_ctx* c, int32_t nboxes, const int32_t* iboxes, const CassMCParams* p,
                              double* max_disp, double* max_rot, uint64_t seed, CassMCResult* out) {
  if (!c || nboxes < 1 || !iboxes || !p || !max_disp || !max_rot || !out || p->nsweeps < 0 ||
      p->steps_per_sweep < 0 || p->nupdate < 0 || !(p->target_accept > 0.0))
    return set_error(CASS_EINVAL, "bad mc arguments");
  if (c->nspecies > kMaxSpeciesMC) return set_error(CASS_ECAPACITY, "mc sweeps support at most 8 species");
  if (!c->pt_set) return set_error(CASS_ESTATE, "nonbond table not set");
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    if (ib < 0 || ib >= c->nboxes) return set_error(CASS_EINVAL, "box index out of range");
    for (int j = 0; j < k; ++j)
      if (iboxes[j] == iboxes[k]) return set_error(CASS_EINVAL, "box listed twice");
    if (!c->box[ib].energy_valid) return set_error(CASS_ESTATE, "system energy of box not computed");
  }
  int rc;
  CASS_CUDA(cudaSetDevice(c->device));
  McArgs A;
  memset(&A, 0, sizeof(A));
  A.nspecies = c->nspecies;
  for (int is = 0; is < c->nspecies; ++is) {
    const SpeciesH& s = c->sp[is];
    McSpecies& m = A.sp[is];
    m.natoms = s.natoms;
    m.has_charge = s.has_charge ? 1 : 0;
    bool lin = true;  // species_list%linear (input_routines.f90:1955-1967)
    for (size_t k = 0; k < s.angle_kind.size(); ++k)
      if (s.angle_kind[k] != CASS_BONDED_FIXED || s.angle_param[2 * k] != 180.0) lin = false;
    m.linear = lin ? 1 : 0;
    for (int a = 0; a < s.natoms && a < kMaxAtoms; ++a) m.mass[a] = s.mass[a];
  }
  A.nsweeps = p->nsweeps;
  A.steps_per_sweep = p->steps_per_sweep;
  A.nupdate = p->nupdate;
  A.prob_translate = p->prob_translate;
  A.target_accept = p->target_accept;
  A.seed = seed;
  bool mixed = c->precision == CASS_PREC_MIXED && c->pt.ntypes <= kMaxTypes;
  size_t smem = 0;
  int max_nv = 0;
  bool any_ewald = false;
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    if ((rc = pack_box_ext(c, ib))) return rc;
    BoxH& B = c->box[ib];
    for (int slot : members_ext(c, ib)) {
      const SpeciesH& s = c->sp[c->slot_sp[slot]];
      if (s.natoms > kMaxAtoms) return set_error(CASS_ECAPACITY, "mc sweeps move molecules of at most 16 atoms");
    }
    mixed = mixed && B.desc.vdw_style == CASS_VDW_LJ &&
            (B.desc.vdw_sum_style == CASS_VDW_SUM_CUT || B.desc.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) &&
            (B.desc.charge_style == CASS_CHARGE_NONE || B.desc.charge_sum_style == CASS_QQ_EWALD);
    smem = std::max(smem, mc_smem_bytes(B.npacked, B.npacked_mols, true));
    if (B.desc.charge_style == CASS_CHARGE_COUL && B.desc.charge_sum_style == CASS_QQ_EWALD && B.nvecs > 0) {
      any_ewald = true;
      max_nv = std::max(max_nv, B.nvecs);
    }
  }
  // boxes above the shared-memory limit run with their layout in global memory
  const bool gmem = smem > kMcSmemLimit;
  if (any_ewald && !c->d_cos_mol.p) return set_error(CASS_ESTATE, "structure factors not computed");
  A.cos_mol = c->d_cos_mol.as<double>();
  A.sin_mol = c->d_sin_mol.as<double>();
  A.stride = c->cos_mol_stride;
  // per-box descriptors and outputs in one device buffer
  const size_t nsp = (size_t)c->nspecies;
  const size_t bytes = nboxes * sizeof(McBox) + nboxes * sizeof(CassEnergy) + nboxes * sizeof(CassMCResult) +
                       2 * nboxes * nsp * sizeof(double) + nboxes * sizeof(int) + 2 * (size_t)nboxes * max_nv * sizeof(double) + 256;
  if ((rc = c->d_mc.reserve(bytes))) return rc;
  McBox* d_box = c->d_mc.as<McBox>();
  CassEnergy* d_E = reinterpret_cast<CassEnergy*>(d_box + nboxes);
  CassMCResult* d_res = reinterpret_cast<CassMCResult*>(d_E + nboxes);
  double* d_md = reinterpret_cast<double*>(d_res + nboxes);
  double* d_mr = d_md + nboxes * nsp;
  double* d_scr = d_mr + nboxes * nsp;
  int* d_status = reinterpret_cast<int*>(d_scr + 2 * (size_t)nboxes * max_nv);
  std::vector<McBox> hb(nboxes);
  std::vector<CassEnergy> hE(nboxes);
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    BoxH& B = c->box[ib];
    McBox& g = hb[k];
    memset(&g, 0, sizeof(g));
    g.b = B.dev;
    g.p64 = B.d_p64.as<double4_32a>();
    g.p32 = B.d_p32.as<float4>();
    g.meta = B.d_meta.as<int4>();
    g.molinfo = B.d_molinfo.as<int4>();
    g.natoms = B.npacked;
    g.nmols = B.npacked_mols;
    g.ibox1 = iboxes[k];
    int first = 0;
    for (int is = 0; is < c->nspecies; ++is) {
      int n = 0;
      for (int slot : members_ext(c, ib))
        if (c->slot_sp[slot] == is) ++n;
      g.nmol_sp[is] = n;
      g.first_sp[is] = first;
      first += n;
    }
    g.comcut = B.comcut ? 1 : 0;
    g.rmax = B.rcut_max;
    g.ewald = B.desc.charge_style == CASS_CHARGE_COUL && B.desc.charge_sum_style == CASS_QQ_EWALD && B.nvecs > 0;
    g.nvecs = g.ewald ? B.nvecs : 0;
    g.kvec = B.d_kvec.as<double4_32a>();
    g.cos_sum = B.d_cos_sum.as<double>();
    g.sin_sum = B.d_sin_sum.as<double>();
    g.new_cos = d_scr + 2 * (size_t)k * max_nv;
    g.new_sin = g.new_cos + max_nv;
    g.max_disp = d_md + k * nsp;
    g.max_rot = d_mr + k * nsp;
    g.energy = d_E + k;
    g.res = d_res + k;
    g.status = d_status + k;
    hE[k] = B.energy;
  }

  CASS_CUDA(h2d(c, d_E, hE.data(), nboxes * sizeof(CassEnergy)));
  CASS_CUDA(h2d(c, d_md, max_disp, nboxes * nsp * sizeof(double)));
  CASS_CUDA(h2d(c, d_mr, max_rot, nboxes * nsp * sizeof(double)));
  size_t dyn = 0;
  for (int k = 0; k < nboxes; ++k) dyn = std::max(dyn, mc_smem_bytes(hb[k].natoms, hb[k].nmols, mixed));
  auto kern = gmem ? (mixed ? k_mc_sweeps<true, true> : k_mc_sweeps<false, true>)
                   : (mixed ? k_mc_sweeps<true, false> : k_mc_sweeps<false, false>);
  if (gmem) dyn = 0;
  CASS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  const int threads = gmem ? kMcThreadsG : kMcThreads;
  // CTAs per chain: a cluster splits the pair and k-vector loops of a move when
  // SMs would otherwise stay idle (few chains); every cluster must be resident.
  // Measured on single chains (sweeps/s, 1 -> best cluster): FP64 LJ-500
  // 117 -> 218 at 4 CTAs, FP64 water-256 with Ewald 20 -> 100 at 8, mixed
  // water-256 143 -> 288 at 8, while mixed LJ-500 (FP32 pairs, no k-space) is
  // bound by the serial steps of a move and loses a little (307 -> 278-292).
  int csize = 1;
  {
    int sms = 0, nmax = 1;
    CASS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    for (const McBox& g : hb) nmax = std::max(nmax, g.natoms);
    int want = c->mc_cluster > 0 ? c->mc_cluster : std::min(8, std::max(1, sms / nboxes));
    if (c->mc_cluster <= 0) want = std::min(want, any_ewald ? 8 : (mixed ? 1 : std::max(1, (nmax + 127) / 128)));
    for (int cs = std::min(8, want); cs >= 2; --cs) {
      cudaLaunchConfig_t q = {};
      cudaLaunchAttribute qa[1];
      qa[0].id = cudaLaunchAttributeClusterDimension;
      qa[0].val.clusterDim.x = cs;
      qa[0].val.clusterDim.y = 1;
      qa[0].val.clusterDim.z = 1;
      q.gridDim = dim3(nboxes * cs);
      q.blockDim = dim3(threads);
      q.dynamicSmemBytes = dyn;
      q.attrs = qa;
      q.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &q) == cudaSuccess && nclusters >= nboxes) {
        csize = cs;
        break;
      }
      (void)cudaGetLastError();
    }
  }
  c->stats.gcmc_cluster = csize;
  if (gmem) {  // one layout per CTA of each box's cluster
    std::vector<size_t> off(nboxes), stride(nboxes);
    size_t tot = 0;
    for (int k = 0; k < nboxes; ++k) {
      off[k] = tot;
      stride[k] = (mc_smem_bytes(hb[k].natoms, hb[k].nmols, mixed) + 255) & ~(size_t)255;
      tot += stride[k] * csize;
    }
    if ((rc = c->d_mc_box.reserve(std::max<size_t>(tot, 256)))) return rc;
    for (int k = 0; k < nboxes; ++k) {
      hb[k].gbox = static_cast<unsigned char*>(c->d_mc_box.p) + off[k];
      hb[k].gbox_stride = stride[k];
    }
  }
  CASS_CUDA(h2d(c, d_box, hb.data(), nboxes * sizeof(McBox)));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(nboxes * csize);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = c->stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CASS_CUDA(cudaEventRecord(c->ev[0], c->stream));
  CASS_CUDA(cudaLaunchKernelEx(&cfg, kern, A, d_box, c->pt, csize));
  CASS_CUDA(cudaGetLastError());
  CASS_CUDA(cudaEventRecord(c->ev[1], c->stream));
  count_launch(c);
  std::vector<CassMCResult> hr(nboxes);
  std::vector<int> hs(nboxes);
  CASS_CUDA(d2h(c, hr.data(), d_res, nboxes * sizeof(CassMCResult)));
  CASS_CUDA(d2h(c, hs.data(), d_status, nboxes * sizeof(int)));
  CASS_CUDA(d2h(c, max_disp, d_md, nboxes * nsp * sizeof(double)));
  CASS_CUDA(d2h(c, max_rot, d_mr, nboxes * nsp * sizeof(double)));
  // the host copy of the coordinates follows the device
  std::vector<std::vector<double4_32a>> pos(nboxes);
  for (int k = 0; k < nboxes; ++k) {
    const BoxH& B = c->box[iboxes[k] - 1];
    pos[k].resize(B.npacked);
    if (B.npacked) CASS_CUDA(d2h(c, pos[k].data(), B.d_p64.p, B.npacked * sizeof(double4_32a)));
  }
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  float ms = 0.0f;
  CASS_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->stats.mc_ms = ms;
  long long moves = 0;
  for (int k = 0; k < nboxes; ++k) {
    BoxH& B = c->box[iboxes[k] - 1];
    for (size_t q = 0; q < B.pk_mol.size(); ++q) {
      const int slot = B.pk_mol[q], is = c->slot_sp[slot];
      SpeciesH& s = c->sp[is];
      double* r = &s.pos[(size_t)(slot - c->mol_base[is]) * 3 * s.natoms];
      for (int a = 0; a < s.natoms; ++a) {
        const double4_32a& v = pos[k][B.pk_mol_off[q] + a];
        r[3 * a] = v.x;
        r[3 * a + 1] = v.y;
        r[3 * a + 2] = v.z;
      }
    }
    B.energy = hr[k].energy;
    B.cell_dirty = true;
    out[k] = hr[k];
    moves += p->nsweeps * (long long)(p->steps_per_sweep > 0 ? p->steps_per_sweep : B.npacked_mols);
  }
  c->stats.mc_moves = moves;
  for (int k = 0; k < nboxes; ++k)
    if (hs[k]) {
      c->box[iboxes[k] - 1].energy_valid = c->box[iboxes[k] - 1].frame_ready = false;
      return set_error(CASS_ESTATE, "a molecule overlapped another before its move (energy too high)");
    }
  return CASS_OK;
}
