// cass_cbmc_f.cuh -- FP32 test-molecule tables and geometry of the mixed
// kernels (Widom and grand-canonical): species and box constants as FP32,
// get_com.f90, Get_Aligner_Hanger (fragment_growth.f90:2135-2185), the RB
// dihedral energy, the intramolecular pair energies and the Boltzmann trial
// choice.  GB300 issues FP64 at 1/64 of its FP32 rate, so the serial parts of
// a CBMC step run in FP32 here.
#pragma once

#include "cass_cbmc.cuh"

namespace cassgpu {

// FP32 copy of the test species' tables (kernel parameter)
struct SpeciesF {
  int natoms, nbonds, nangles, ndih, nimp;
  float q[kMaxAtoms], mass[kMaxAtoms];
  int type[kMaxAtoms];
  float vs[kMaxAtoms * kMaxAtoms], qs[kMaxAtoms * kMaxAtoms];
  unsigned bonded[kMaxAtoms];  // bit j of bonded[i]: i-j is a 1-2 pair
  signed char bond_atoms[kMaxBonded][2], angle_atoms[kMaxBonded][3], dih_atoms[kMaxBonded][4],
      imp_atoms[kMaxBonded][4];
  unsigned char bond_harm[kMaxBonded], angle_harm[kMaxBonded];
  float bond_k[kMaxBonded], bond_l0[kMaxBonded], angle_k[kMaxBonded], angle_t0[kMaxBonded];
  float rb[kMaxBonded][6], imp_k[kMaxBonded], imp_p0[kMaxBonded];
  float cum_prob_ins[kMaxFrags];
  // floor(cum_prob_ins * 2^32): the fragment choice decided on the top 32 bits of a draw
  unsigned long long cumthr[kMaxFrags];
};

// FP32 constants of the CTA's box
struct BoxF {
  float L[3], hL[3], cinv[3];
  float Llo[3];  // L - (float)L: the box edge as a two-term FP32 value (Widom centres of mass)
  float ch[3];  // cell edge L / nc (Widom stencils)
  int nc[3];
  float rcb2, rv2, rq2, low2, rc_cbmc, rc_full, beta, kmaxE, alpha;
  int charge_on;
  // CBMC options: the FP32 atom-pair energy table and the r_min^2 test
  int tab_res, sector, ntypes;
  float tab_shift, tab_rcs, tab_step, tab_inv_step;  // tab_rcs = rcut_cbmc^2 - tab_shift
  const float* tab_v;
  const float* tab_f2;
  float rmin2[kMaxTypes * kMaxTypes];  // row stride kMaxTypes
  // Widom full-cutoff pass: FP64 box edges and squared cutoffs, and the half
  // widths (A^2) of the bands about rv2, rq2 and low2 inside which an FP32 r^2
  // can fall on the other side of a cutoff than the FP64 r^2
  double L64[3], hL64[3];
  double rv2d, rq2d, low2d;
  float band_v, band_q, band_low;
};

// the CBMC-option fields of f from the box's BoxDev; thread 0 then all threads
__device__ inline void boxf_options(BoxF& f, const BoxDev& b, int ntypes) {
  if (threadIdx.x == 0) {
    f.tab_res = b.tab_res;
    f.sector = b.sector;
    f.ntypes = ntypes;
    f.tab_shift = (float)b.tab_shift;
    f.tab_rcs = (float)(b.rcut_cbmcsq - b.tab_shift);
    f.tab_step = (float)b.tab_step;
    f.tab_inv_step = b.tab_res > 0 ? (float)(1.0 / b.tab_step) : 0.0f;
    f.tab_v = b.tab_vf;
    f.tab_f2 = b.tab_f2f;
  }
  for (int i = threadIdx.x; i < kMaxTypes * kMaxTypes; i += blockDim.x) {
    const int ta = i / kMaxTypes, tb = i % kMaxTypes;
    f.rmin2[i] = (b.sector && ta < ntypes && tb < ntypes) ? b.rminsqf[ta * ntypes + tb] : (float)b.rcut_lowsq;
  }
}

// uniform in [0, 1) from an lfsr258 draw without the FP64 unit: the reference
// value x*2^-64 + 0.5 (x signed) equals (x ^ 2^63) / 2^64; keep its top 23 bits
__device__ __forceinline__ float draw_f(Lfsr& g) {
  g.next_bits();
  unsigned v = (unsigned)(((g.s1 ^ g.s2 ^ g.s3 ^ g.s4 ^ g.s5) ^ 0x8000000000000000ull) >> 41);
  return (__int_as_float(0x4B000000 | v) - 8388608.0f) * 1.1920928955078125e-7f;
}

// The Widom kernel's draws keep the top 32 bits v of the reference's uniform
// u = x 2^-64 + 0.5 (v = (x ^ 2^63) >> 32), so that
//   * uniforms that enter the geometry carry 24 significant bits (rounded toward zero);
//   * int(u * n) (library conformations) is exact in integer arithmetic unless
//     u * n lies within n 2^-32 of an integer (a 2^-32 n chance per draw);
//   * a centre-of-mass coordinate (0.5 - u) L is formed in two-term FP32 and
//     rounded once, so it carries only the FP32 rounding of its own value.
__device__ __forceinline__ unsigned draw_u32(Lfsr& g) {
  g.next_bits();
  return (unsigned)(((g.s1 ^ g.s2 ^ g.s3 ^ g.s4 ^ g.s5) ^ 0x8000000000000000ull) >> 32);
}

__device__ __forceinline__ float unit_of(unsigned v) { return __uint2float_rz(v) * 2.3283064365386963e-10f; }

__device__ __forceinline__ int index_of(unsigned v, int n) {
  const int k = (int)(((unsigned long long)v * (unsigned)n) >> 32);
  return k < n ? k : n - 1;
}

// (0.5 - u) L = (2^31 - v) L 2^-32 with L = Lh + Ll
__device__ __forceinline__ float centre_of(unsigned v, float Lh, float Ll) {
  const long long m = 2147483648LL - (long long)v;
  const long long mhi = m & ~0xFFLL;
  const float mh = (float)mhi, ml = (float)(m - mhi);
  const float p = mh * Lh;
  const float e = fmaf(mh, Lh, -p);
  const float rest = fmaf(mh, Ll, fmaf(ml, Lh, e));
  return (p + rest) * 2.3283064365386963e-10f;
}

__device__ __forceinline__ void get_com_f(const SpeciesF& S, const float* r, unsigned exist, float com[3]) {
  float tm = 0, x = 0, y = 0, z = 0;
  for (int k = 0; k < S.natoms; ++k) {
    if (!((exist >> k) & 1u)) continue;
    float m = S.mass[k];
    tm += m;
    x += m * r[3 * k];
    y += m * r[3 * k + 1];
    z += m * r[3 * k + 2];
  }
  float inv = 1.0f / tm;
  com[0] = x * inv;
  com[1] = y * inv;
  com[2] = z * inv;
}

__device__ inline void aligner_hanger_f(float v1[3], float v2[3], float al[9], float hg[9]) {
  float n1 = rsqrtf(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  for (int i = 0; i < 3; ++i) v1[i] *= n1;
  float n2 = rsqrtf(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  for (int i = 0; i < 3; ++i) v2[i] *= n2;
  float p1[3] = {v1[1] * v2[2] - v1[2] * v2[1], -v1[0] * v2[2] + v1[2] * v2[0], v1[0] * v2[1] - v1[1] * v2[0]};
  float np1 = rsqrtf(p1[0] * p1[0] + p1[1] * p1[1] + p1[2] * p1[2]);
  for (int i = 0; i < 3; ++i) p1[i] *= np1;
  float p2[3] = {v1[1] * p1[2] - v1[2] * p1[1], -v1[0] * p1[2] + v1[2] * p1[0], v1[0] * p1[1] - v1[1] * p1[0]};
  float np2 = rsqrtf(p2[0] * p2[0] + p2[1] * p2[1] + p2[2] * p2[2]);
  for (int i = 0; i < 3; ++i) p2[i] *= np2;
  for (int i = 0; i < 3; ++i) {
    al[i] = v1[i];
    al[3 + i] = p2[i];
    al[6 + i] = p1[i];
    hg[i * 3 + 0] = v1[i];
    hg[i * 3 + 1] = p2[i];
    hg[i * 3 + 2] = p1[i];
  }
}


__device__ __forceinline__ float lj_or_zero(const float2* ljp, int ti, int tj, float scale, float r2) {
  if (ti < 0 || tj < 0) return 0.0f;
  float2 es = ljp[ti * kMaxTypes + tj];
  return lj_pair_f(es.x * scale, es.y, r2);
}

// Compute_Molecule_Dihedral_Energy (RB form) over dihedrals whose atoms all exist
__device__ inline float dihedral_f(const SpeciesF& S, const float* r, unsigned exist) {
  float e = 0.0f;
  for (int k = 0; k < S.ndih; ++k) {
    const signed char* a = S.dih_atoms[k];
    unsigned m = (1u << a[0]) | (1u << a[1]) | (1u << a[2]) | (1u << a[3]);
    if ((exist & m) != m) continue;
    float rx12 = r[3 * a[0]] - r[3 * a[1]], ry12 = r[3 * a[0] + 1] - r[3 * a[1] + 1], rz12 = r[3 * a[0] + 2] - r[3 * a[1] + 2];
    float rx32 = r[3 * a[2]] - r[3 * a[1]], ry32 = r[3 * a[2] + 1] - r[3 * a[1] + 1], rz32 = r[3 * a[2] + 2] - r[3 * a[1] + 2];
    float rx34 = r[3 * a[2]] - r[3 * a[3]], ry34 = r[3 * a[2] + 1] - r[3 * a[3] + 1], rz34 = r[3 * a[2] + 2] - r[3 * a[3] + 2];
    float mx = ry12 * rz32 - ry32 * rz12, my = -rx12 * rz32 + rz12 * rx32, mz = rx12 * ry32 - ry12 * rx32;
    float nx = ry32 * rz34 - rz32 * ry34, ny = -rx32 * rz34 + rz32 * rx34, nz = rx32 * ry34 - ry32 * rx34;
    float c = (mx * nx + my * ny + mz * nz) * rsqrtf((mx * mx + my * my + mz * mz) * (nx * nx + ny * ny + nz * nz));
    const float* cb = S.rb[k];
    e += cb[0] + c * (cb[1] + c * (cb[2] + c * (cb[3] + c * (cb[4] + c * cb[5]))));
  }
  return e;
}

// intramolecular pair energy with the species scales (LJ + Ewald real space)
__device__ __forceinline__ void intra_pair_f(const SpeciesF& S, const BoxF& f, const float2* ljp, int ia, int ja,
                                             float r2, bool vdw, bool qq, float& eiv, float& eiq, float& eoq) {
  const int n = S.natoms;
  if (vdw) eiv += lj_or_zero(ljp, S.type[ia], S.type[ja], S.vs[ia * n + ja], r2);
  if (qq) {
    float rinv = rsqrtf(r2);
    float eij = S.q[ia] * S.q[ja] * rinv * (float)kCHARGE_FACTOR;
    float erf_val = 1.0f - erfc_asf(f.alpha * r2 * rinv);
    eiq += S.qs[ia * n + ja] * eij;
    eoq += -erf_val * eij;
  }
}

// Compute_Atom_Nonbond_Intra_Energy (energy_routines.f90:691-737), CBMC cutoff
__device__ inline bool atom_intra_f(const SpeciesF& S, const BoxF& f, const float2* ljp, int ia, const float* r,
                             unsigned exist, float& eiv, float& eiq, float& eoq) {
  eiv = eiq = eoq = 0.0f;
  const int n = S.natoms;
  for (int ja = 0; ja < n; ++ja) {
    if (ja == ia || !((exist >> ja) & 1u)) continue;
    const bool nzv = S.vs[ia * n + ja] > 0.0f, nzq = S.qs[ia * n + ja] > 0.0f;
    if (!(nzv || nzq)) continue;
    float dx = r[3 * ja] - r[3 * ia], dy = r[3 * ja + 1] - r[3 * ia + 1], dz = r[3 * ja + 2] - r[3 * ia + 2];
    float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < f.low2 && nzv) return true;
    const bool in = r2 <= f.rcb2;
    intra_pair_f(S, f, ljp, ja, ia, r2, in && nzv, in && nzq && f.charge_on, eiv, eiq, eoq);
  }
  return false;
}

struct IntraF {
  float bond, angle, dih, imp, ivdw, iqq, pqq;
  bool overlap;
};

// bonded + Compute_Molecule_Nonbond_Intra_Energy (full cutoffs), FP32
__device__ inline IntraF molecule_intra_f(const SpeciesF& S, const BoxF& f, const float2* ljp, const float* r) {
  IntraF o{0, 0, 0, 0, 0, 0, 0, false};
  for (int k = 0; k < S.nbonds; ++k) {
    if (!S.bond_harm[k]) continue;
    int a = S.bond_atoms[k][0], c = S.bond_atoms[k][1];
    float dx = r[3 * a] - r[3 * c], dy = r[3 * a + 1] - r[3 * c + 1], dz = r[3 * a + 2] - r[3 * c + 2];
    float l = sqrtf(dx * dx + dy * dy + dz * dz);
    o.bond += S.bond_k[k] * (l - S.bond_l0[k]) * (l - S.bond_l0[k]);
  }
  for (int k = 0; k < S.nangles; ++k) {
    if (!S.angle_harm[k]) continue;
    int a1 = S.angle_atoms[k][0], a2 = S.angle_atoms[k][1], a3 = S.angle_atoms[k][2];
    float rx21 = r[3 * a2] - r[3 * a1], ry21 = r[3 * a2 + 1] - r[3 * a1 + 1], rz21 = r[3 * a2 + 2] - r[3 * a1 + 2];
    float rx32 = r[3 * a3] - r[3 * a2], ry32 = r[3 * a3 + 1] - r[3 * a2 + 1], rz32 = r[3 * a3 + 2] - r[3 * a2 + 2];
    float C23 = rx21 * rx32 + ry21 * ry32 + rz21 * rz32, C22 = rx21 * rx21 + ry21 * ry21 + rz21 * rz21,
          C33 = rx32 * rx32 + ry32 * ry32 + rz32 * rz32;
    float ct = fmaxf(fminf(C23 * rsqrtf(C33 * C22), 0.999999f), -0.999999f);
    float th = (float)kPI - acosf(ct);
    o.angle += S.angle_k[k] * (th - S.angle_t0[k]) * (th - S.angle_t0[k]);
  }
  o.dih = dihedral_f(S, r, 0xffffffffu);
  for (int k = 0; k < S.nimp; ++k) {
    const signed char* a = S.imp_atoms[k];
    float rx12 = r[3 * a[0]] - r[3 * a[1]], ry12 = r[3 * a[0] + 1] - r[3 * a[1] + 1], rz12 = r[3 * a[0] + 2] - r[3 * a[1] + 2];
    float rx32 = r[3 * a[2]] - r[3 * a[1]], ry32 = r[3 * a[2] + 1] - r[3 * a[1] + 1], rz32 = r[3 * a[2] + 2] - r[3 * a[1] + 2];
    float rx34 = r[3 * a[2]] - r[3 * a[3]], ry34 = r[3 * a[2] + 1] - r[3 * a[3] + 1], rz34 = r[3 * a[2] + 2] - r[3 * a[3] + 2];
    float mx = ry12 * rz32 - ry32 * rz12, my = -rx12 * rz32 + rz12 * rx32, mz = rx12 * ry32 - ry12 * rx32;
    float nx = ry32 * rz34 - rz32 * ry34, ny = -rx32 * rz34 + rz32 * rx34, nz = rx32 * ry34 - ry32 * rx34;
    float cp = (mx * nx + my * ny + mz * nz) * rsqrtf((mx * mx + my * my + mz * mz) * (nx * nx + ny * ny + nz * nz));
    cp = fminf(1.0f, fmaxf(-1.0f, cp));
    float phi = copysignf(acosf(cp), rx12 * nx + ry12 * ny + rz12 * nz);
    o.imp += S.imp_k[k] * (phi - S.imp_p0[k]) * (phi - S.imp_p0[k]);
  }
  const int n = S.natoms;
  for (int ia = 0; ia < n; ++ia)
    for (int ja = ia + 1; ja < n; ++ja) {
      float dx = r[3 * ia] - r[3 * ja], dy = r[3 * ia + 1] - r[3 * ja + 1], dz = r[3 * ia + 2] - r[3 * ja + 2];
      float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 <= f.low2 && !((S.bonded[ia] >> ja) & 1u)) {
        o.overlap = true;
        return o;
      }
      intra_pair_f(S, f, ljp, ia, ja, r2, r2 <= f.rv2, f.charge_on && r2 <= f.rq2, o.ivdw, o.iqq, o.pqq);
    }
  return o;
}

// Boltzmann choice among k trials (fragment_growth.f90:569-620, 1994-2046):
// weights exp(-beta (U - U_min)) and the rule "rand * sum < cumulative sum";
// returns the trial or -1 and sets *lnw = ln sum_t exp(-beta U_t)
__device__ __forceinline__ int select_trial_f(int k, const float* u, unsigned ovm, float beta, float pick, float* lnw) {
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
  const float x = pick * cum;
  int sel = 0;
  while (sel < k && !(x < w[sel])) ++sel;
  if (sel == k) return -1;
  *lnw = -beta * umin + logf(cum);
  return sel;
}

struct SpeciesH;
bool species_f(const SpeciesH& s, SpeciesF& F);

}  // namespace cassgpu
