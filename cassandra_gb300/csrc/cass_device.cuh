// cass_device.cuh -- device-side building blocks of the energy hot path.
//
// Plain-old-data structs shared by the host launcher and the kernels, and
// __device__ restatements of the per-pair arithmetic of Cassandra's
// energy_routines.f90 in two precisions:
//   FP64  : every operation in double, the reference arithmetic;
//   mixed : FP32 minimum image, r^2, LJ and A&S erfc, with compensated FP32
//           sums promoted to double.  Cutoff and overlap decisions are taken on
//           the FP32 r^2, so a pair within about 1e-5 A^2 of a cutoff can fall
//           on the other side than in FP64 (changing the energy by that pair's
//           energy at the cutoff).
#pragma once

#include <cstdint>

#include "../../include/cassandra_gb300.h"

namespace cassgpu {

// global_variables.f90:182-232 (truncated pi on purpose)
constexpr double kPI = 3.1415926536;
constexpr double kTWOPI = 6.2831853072;
constexpr double kROOTPI = 1.7724538509;
constexpr double kKBOLTZ = 0.8314472;
constexpr double kCHARGE_FACTOR = 138935.4558;
constexpr double kMAX_KBT = 708.0;

constexpr int kMaxTypes = 8;       // nonbond atom types per context
constexpr int kMaxAtoms = 16;      // atoms of a CBMC / Widom test species
constexpr int kMaxFrags = 8;       // CBMC fragments of a test species
constexpr int kMaxKappa = 32;      // kappa_ins, kappa_dih
constexpr int kMaxBonded = 24;     // angles / dihedrals of a test species

// Nonbond pair table (vdw_param1..4_table after mixing).
struct PairTable {
  int ntypes;
  double eps[kMaxTypes * kMaxTypes];
  double sig2[kMaxTypes * kMaxTypes];
  double mie_n[kMaxTypes * kMaxTypes];
  double mie_m[kMaxTypes * kMaxTypes];
  double mie_c[kMaxTypes * kMaxTypes];  // n/(n-m) (n/m)^(m/(n-m))
  float epsf[kMaxTypes * kMaxTypes];
  float sig2f[kMaxTypes * kMaxTypes];
};

// Per-box constants a kernel needs (Box_Class + cutoffs + styles).
struct BoxDev {
  double L[3], hL[3], volume;
  float Lf[3], hLf[3];
  int vdw_style, vdw_sum_style, charge_style, charge_sum_style;
  double rcut_vdwsq, rcut_coulsq, rcut_cbmcsq, rcut_lowsq, rcut_coul, rcut_vdw;
  double ron_switch_sq, roff_switch_sq, switch_factor1, switch_factor2;
  double alpha, alpha_dsf, dsf_factor1, dsf_factor2;
  double beta;
  // cell grid of the packed, cell-sorted atoms (Widom path)
  int nc[3];
  double cell_inv[3];  // nc / L
  int atom_off, natoms, cell_off;  // offsets into the concatenated sorted arrays
  // Ewald
  int nvecs, kvec_off;
  // Widom per-box constants
  double e_inter_constant, prefactor;
  // CBMC options (cass_set_cbmc_options): the atom-pair energy table (0 bins:
  // off) and the r_min^2 overlap test of Widom growth (sector != 0)
  int tab_res, sector;
  double tab_step, tab_shift;
  const double* tab_v;   // [ntypes][ntypes][tab_res] vdW part
  const double* tab_f2;  // [tab_res] Coulomb kernel, times (q_i cf) q_j
  const float* tab_vf;   // FP32 copies
  const float* tab_f2f;
  const double* rminsq;  // [ntypes][ntypes]
  const float* rminsqf;
  // Check_MoleculePair_Cutoff boxes (LJ CHARMM, minimum-image charges; Widom
  // path): per packed atom its molecule's COM and max_dcom, and rcut_max
  const double4_32a* mcom;
  double rcut_max;
};

__host__ __device__ inline int pidx(int i, int j, int nt) { return i * nt + j; }

// ---------------------------------------------------------------------------
// lfsr258 (random_generators.f90:95-122) and the per-insertion stream seeding.
struct Lfsr {
  uint64_t s1, s2, s3, s4, s5;
  // advances the five components (the state update of rranf)
  __host__ __device__ inline void next_bits() {
    uint64_t b;
    b = ((s1 << 1) ^ s1) >> 53;
    s1 = ((s1 & 0xFFFFFFFFFFFFFFFEull) << 10) ^ b;
    b = ((s2 << 24) ^ s2) >> 50;
    s2 = ((s2 & 0xFFFFFFFFFFFFFE00ull) << 5) ^ b;
    b = ((s3 << 3) ^ s3) >> 23;
    s3 = ((s3 & 0xFFFFFFFFFFFFF000ull) << 29) ^ b;
    b = ((s4 << 5) ^ s4) >> 24;
    s4 = ((s4 & 0xFFFFFFFFFFFE0000ull) << 23) ^ b;
    b = ((s5 << 3) ^ s5) >> 33;
    s5 = ((s5 & 0xFFFFFFFFFF800000ull) << 8) ^ b;
  }
  __host__ __device__ inline double next() {
    uint64_t b;
    b = ((s1 << 1) ^ s1) >> 53;
    s1 = ((s1 & 0xFFFFFFFFFFFFFFFEull) << 10) ^ b;
    b = ((s2 << 24) ^ s2) >> 50;
    s2 = ((s2 & 0xFFFFFFFFFFFFFE00ull) << 5) ^ b;
    b = ((s3 << 3) ^ s3) >> 23;
    s3 = ((s3 & 0xFFFFFFFFFFFFF000ull) << 29) ^ b;
    b = ((s4 << 5) ^ s4) >> 24;
    s4 = ((s4 & 0xFFFFFFFFFFFE0000ull) << 23) ^ b;
    b = ((s5 << 3) ^ s5) >> 33;
    s5 = ((s5 & 0xFFFFFFFFFF800000ull) << 8) ^ b;
    long long x = (long long)(s1 ^ s2 ^ s3 ^ s4 ^ s5);
    return (double)x * 5.4210108624275221E-20 + 0.5;
  }
};

__host__ __device__ inline uint64_t splitmix64(uint64_t& st) {
  uint64_t z = (st += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Stream of insertion `ins` (0-based) in box `ibox` (1-based): five splitmix64
// words, each forced above the component's minimum state.
__host__ __device__ inline Lfsr seed_stream(uint64_t seed, long long ibox, long long ins) {
  uint64_t st = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(ibox + 1)) ^ (0x8CB92BA72F3D8DD7ull * (uint64_t)(ins + 1));
  const uint64_t mins[5] = {1ull, 511ull, 4095ull, 131071ull, 8388607ull};
  uint64_t v[5];
  for (int k = 0; k < 5; ++k) {
    uint64_t w = splitmix64(st);
    if ((w & ~mins[k]) == 0) w |= (mins[k] + 1);
    v[k] = w;
  }
  Lfsr r;
  r.s1 = v[0]; r.s2 = v[1]; r.s3 = v[2]; r.s4 = v[3]; r.s5 = v[4];
  return r;
}

// ---------------------------------------------------------------------------
// Minimum_Image_Separation, orthorhombic branch (minimum_image_separation.f90:60-82)
template <class T>
__device__ __forceinline__ T fold(T d, T hl, T l) {
  return d > hl ? d - l : (d < -hl ? d + l : d);
}

// A&S 7.1.26 erfc (energy_routines.f90:2143-2163)
__device__ __forceinline__ double erfc_as(double x) {
  const double A1 = 0.254829592, A2 = -0.284496736, A3 = 1.421413741, A4 = -1.453152027, A5 = 1.061405429,
               P = 0.3275911;
  double T = 1.0 / (1.0 + P * x);
  double TP = T * (A1 + T * (A2 + T * (A3 + T * (A4 + T * A5))));
  return TP * exp(-x * x);
}
__device__ __forceinline__ float erfc_asf(float x) {
  const float A1 = 0.254829592f, A2 = -0.284496736f, A3 = 1.421413741f, A4 = -1.453152027f, A5 = 1.061405429f,
              P = 0.3275911f;
  float T = __frcp_rn(1.0f + P * x);
  float TP = T * (A1 + T * (A2 + T * (A3 + T * (A4 + T * A5))));
  return TP * __expf(-x * x);
}

// Which interactions a pair at r2 contributes (Check_AtomPair_Cutoff,
// energy_routines.f90:3092-3195), as a bit mask: 1 = vdw, 2 = qq.
__device__ __forceinline__ int cutoff_mask(const BoxDev& b, double r2, bool cbmc) {
  int m = 0;
  if (b.vdw_style == CASS_VDW_LJ) {
    if (cbmc) m |= (r2 <= b.rcut_cbmcsq);
    else if (b.vdw_sum_style == CASS_VDW_SUM_MINIMUM || b.vdw_sum_style == CASS_VDW_SUM_CHARMM) m |= 1;
    else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) m |= (r2 <= b.roff_switch_sq);
    else m |= (r2 <= b.rcut_vdwsq);
  } else if (b.vdw_style == CASS_VDW_MIE) {
    if (cbmc) m |= (r2 <= b.rcut_cbmcsq);
    else if (b.vdw_sum_style == CASS_VDW_SUM_CUT || b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT ||
             b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL)
      m |= (r2 <= b.rcut_vdwsq);
  }
  if (b.charge_style == CASS_CHARGE_COUL) {
    if (b.charge_sum_style == CASS_QQ_MINIMUM) m |= 2;
    else if (cbmc ? (r2 <= b.rcut_cbmcsq) : (r2 <= b.rcut_coulsq)) m |= 2;
  }
  return m;
}

// Compute_AtomPair_Energy vdw part (energy_routines.f90:1907-2000), FP64.
// `scale` is vdw_intra_scale for intramolecular pairs, 1 otherwise.
__device__ __forceinline__ double vdw_pair(const PairTable& t, const BoxDev& b, int it, int jt, double r2,
                                           double scale) {
  if (it < 0 || jt < 0) return 0.0;
  int k = pidx(it, jt, t.ntypes);
  double eps = t.eps[k] * scale;
  if (b.vdw_style == CASS_VDW_LJ) {
    double s2 = t.sig2[k] / r2;
    double s6 = s2 * s2 * s2;
    double s12 = s6 * s6;
    double e = 4.0 * eps * (s12 - s6);
    switch (b.vdw_sum_style) {
      case CASS_VDW_SUM_CUT_SHIFT: {
        double sc2 = t.sig2[k] / b.rcut_vdwsq, sc6 = sc2 * sc2 * sc2, sc12 = sc6 * sc6;
        e = e - 4.0 * eps * (sc12 - sc6);
        break;
      }
      case CASS_VDW_SUM_CUT_SWITCH:
        if (r2 >= b.ron_switch_sq) {
          if (r2 <= b.roff_switch_sq) {
            double d = b.roff_switch_sq - r2;
            e = d * d * (b.switch_factor2 + 2.0 * r2) * b.switch_factor1 * e;
          } else {
            e = 0.0;
          }
        }
        break;
      case CASS_VDW_SUM_CHARMM:
        e = eps * (s12 - 2.0 * s6);
        break;
      case CASS_VDW_SUM_CUT_SHIFT_FORCE: {
        double sc2 = t.sig2[k] / b.rcut_vdwsq, sc6 = sc2 * sc2 * sc2, sc12 = sc6 * sc6;
        e = e - 4.0 * eps * (sc12 - sc6);
        double rij = sqrt(r2), rc = b.rcut_vdw;
        double de = -24.0 * eps * (2.0 * sc12 / rc - sc6 / rc);
        e = e - (rij - rc) * de;
        break;
      }
      default:
        break;
    }
    return e;
  }
  if (b.vdw_style == CASS_VDW_MIE) {
    double rij = sqrt(r2);
    double s = sqrt(t.sig2[k]) / rij;
    double e = t.mie_c[k] * eps * (pow(s, t.mie_n[k]) - pow(s, t.mie_m[k]));
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
      double sc = sqrt(t.sig2[k]) / b.rcut_vdw;
      e = e - t.mie_c[k] * eps * (pow(sc, t.mie_n[k]) - pow(sc, t.mie_m[k]));
    }
    return e;
  }
  return 0.0;
}

// Real-space charge-charge part of Compute_AtomPair_Energy for an
// intermolecular pair (energy_routines.f90:2014-2049, 2088-2166), FP64.
__device__ __forceinline__ double qq_pair_inter(const BoxDev& b, double qiqj, double r2) {
  if (b.charge_sum_style == CASS_QQ_EWALD) {
    double rij = sqrt(r2);
    double erf_val = 1.0 - erfc_as(b.alpha * rij);
    double Eij = qiqj / rij * kCHARGE_FACTOR;
    return Eij - erf_val * Eij;
  }
  if (b.charge_sum_style == CASS_QQ_DSF) {
    double rij = sqrt(r2);
    double Eij = b.dsf_factor2 * (rij - b.rcut_coul) - b.dsf_factor1 + erfc(b.alpha_dsf * rij) / rij;
    return Eij * qiqj * kCHARGE_FACTOR;
  }
  return kCHARGE_FACTOR * qiqj / sqrt(r2);
}

// Intramolecular pair: returns the scaled minimum-image part (E_intra_qq) and
// adds the periodic part (E_inter_qq) to *periodic.
__device__ __forceinline__ double qq_pair_intra(const BoxDev& b, double qiqj, double r2, double qscale,
                                                double* periodic) {
  if (b.charge_sum_style == CASS_QQ_EWALD) {
    double rij = sqrt(r2);
    double erf_val = 1.0 - erfc_as(b.alpha * rij);
    double Eij = qiqj / rij * kCHARGE_FACTOR;
    *periodic += 0.0 - erf_val * Eij;
    return qscale * Eij;
  }
  if (b.charge_sum_style == CASS_QQ_DSF) {
    double rij = sqrt(r2);
    double cfqq = qiqj * kCHARGE_FACTOR;
    double Eij = (b.dsf_factor2 * (rij - b.rcut_coul) - b.dsf_factor1 + erfc(b.alpha_dsf * rij) / rij) * cfqq;
    return Eij - (1.0 - qscale) * (cfqq / rij);
  }
  return qscale * kCHARGE_FACTOR * qiqj / sqrt(r2);
}

// Estimate_MoleculePair_Energy for one atom pair (energy_routines.f90:
// 1563-1583): the table bin of r^2 - rsq_shifter.  Returns 0 beyond
// rcut_cbmc, 2 on overlap (below rcut_low), else 1 with the entry added to e.
__device__ __forceinline__ int table_pair(const BoxDev& b, int nt, double r2, int ti, int tj, double qi, double qj,
                                          double& e) {
  const double rs = r2 - b.tab_shift;
  if (rs >= b.rcut_cbmcsq - b.tab_shift) return 0;
  if (rs < b.tab_step) return 2;
  int bin = (int)(rs / b.tab_step);  // 1-based; res at most, except within rounding of the cutoff
  if (bin > b.tab_res) bin = b.tab_res;
  const double ev = (ti >= 0 && tj >= 0) ? b.tab_v[((size_t)ti * nt + tj) * b.tab_res + (bin - 1)] : 0.0;
  e += ev + b.tab_f2[bin - 1] * ((qi * kCHARGE_FACTOR) * qj);
  return 1;
}

// the same in FP32 from the FP32 table (mixed kernels); rcs = rcut_cbmc^2 - shift;
// the term is returned in e
__device__ __forceinline__ int table_pair_f(const float* v, const float* f2, int res, float shift, float rcs,
                                            float step, float inv_step, int nt, float r2, int ti, int tj, float qicf,
                                            float qj, float& e) {
  const float rs = r2 - shift;
  if (rs >= rcs) return 0;
  if (rs < step) return 2;
  int bin = (int)(rs * inv_step);
  bin = min(max(bin, 1), res);
  const float ev = (ti >= 0 && tj >= 0) ? __ldg(&v[(ti * nt + tj) * res + (bin - 1)]) : 0.0f;
  e = ev + __ldg(&f2[bin - 1]) * (qicf * qj);
  return 1;
}

// r_min^2 of check_overlap (sector_routines.f90:160-233) for a type pair
__device__ __forceinline__ double rmin2_pair(const BoxDev& b, int nt, int ti, int tj) {
  return (ti >= 0 && tj >= 0) ? b.rminsq[ti * nt + tj] : b.rcut_lowsq;
}

// True where the mixed kernels may take the FP32 form lj_pair_f: LJ with the
// cut, cut_tail or minimum-image sum, whose pair energy is the plain
// 4 eps (s^12 - s^6).  The shift, switch, shifted-force and CHARMM forms
// (energy_routines.f90:1927-1970) apply whatever the CBMC flag is, so those
// styles keep the FP64 vdw_pair in every precision.
__host__ __device__ inline bool lj_plain_style(const BoxDev& b) {
  return b.vdw_style == CASS_VDW_LJ &&
         (b.vdw_sum_style == CASS_VDW_SUM_CUT || b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL ||
          b.vdw_sum_style == CASS_VDW_SUM_MINIMUM);
}

// FP32 LJ without shift or switch terms, for the styles of lj_plain_style
__device__ __forceinline__ float lj_pair_f(float eps, float sig2, float r2) {
  float s2 = sig2 * __frcp_rn(r2);
  float s6 = s2 * s2 * s2;
  return 4.0f * eps * (s6 * s6 - s6);
}

__device__ __forceinline__ float qq_ewald_inter_f(float alpha, float qiqj, float r2) {
  float rinv = rsqrtf(r2);
  float rij = r2 * rinv;
  return qiqj * (float)kCHARGE_FACTOR * rinv * erfc_asf(alpha * rij);
}

// Compensated (Neumaier) FP32 accumulator.
struct KahanF {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    float t = s + x;
    c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

}  // namespace cassgpu
