// cass_oracle.cpp -- CPU FP64 oracle for the Cassandra molecular-energy hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++ and FP64, the
// reference Fortran routines that the GPU library replaces, so that the GPU
// results can be checked against them.  It is imported only by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg; the product
// library (libcassgpu.so) never links or calls it.
//
// Parity is pinned by the reference's own golden values (NIST SRSW LJ and
// SPC/E energies, the analytic LJ/Mie/Ewald checks and the per-frame energies
// of the pregen Widom fixtures); see tests/test_oracle_golden.py.
//
// Every function cites the reference routine it follows (paths relative to the
// Cassandra source tree).  Exported symbols carry an orc_ prefix and mirror the
// signatures of include/cassandra_gb300.h.

#include "../include/cassandra_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Constants of global_variables.f90:182-232, with the truncated pi values.
constexpr double PI = 3.1415926536;
constexpr double TWOPI = 6.2831853072;
constexpr double ROOTPI = 1.7724538509;
constexpr double KBOLTZ = 0.8314472;
constexpr double CHARGE_FACTOR = 138935.4558;
constexpr double MAX_KBT = 708.0;
constexpr double H_PLANK = 39.9031268605;
constexpr double ATOMIC_TO_KJMOL = 0.01;

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

struct Species {
  int natoms = 0;
  std::vector<int> type;  // 0-based, -1 = no vdW
  std::vector<double> q, mass, vdw_scale, qq_scale;
  std::vector<int> bonded;
  std::vector<int> bond_atoms, bond_kind;
  std::vector<double> bond_param;
  std::vector<int> angle_atoms, angle_kind;
  std::vector<double> angle_param;
  std::vector<int> dih_atoms;
  std::vector<double> dih_rb;
  std::vector<int> imp_atoms;
  std::vector<double> imp_param;
  int nfrag = 0;
  std::vector<std::vector<int>> frag_atoms;     // 0-based atom ids, [0] = anchor
  std::vector<std::vector<int>> frag_connect;   // 0-based fragment ids
  std::vector<int> frag_nconfig;
  std::vector<std::vector<double>> frag_lib;    // [nconfig][natoms_f][3]
  std::vector<double> prob_ins, cum_prob_ins;
  bool l_coul_cbmc = false;
  bool has_charge = false;
  bool defined = false;
};

struct Box {
  bool defined = false;
  CassBoxDesc desc{};
  double L[3] = {0, 0, 0}, hL[3] = {0, 0, 0}, volume = 0;
  int vdw_style = 0, vdw_sum_style = 0, charge_style = 0, charge_sum_style = 0;
  double rcut_vdw = 0, rcut_coul = 0, rcut_cbmc = 0, rcut_low = 0, rcut_max = 0;
  double rcut_vdwsq = 0, rcut_coulsq = 0, rcut_cbmcsq = 0, rcut_lowsq = 0;
  double ron_switch_sq = 0, roff_switch_sq = 0, switch_factor1 = 0, switch_factor2 = 0;
  double rcut3 = 0, rcut9 = 0;
  double alpha_ewald = 0, h_ewald_cut = 0;
  double alpha_dsf = 0, dsf_factor1 = 0, dsf_factor2 = 0;
  double beta = 0;
  // Ewald k-space
  std::vector<double> hx, hy, hz, hsq, Cn;
  std::vector<double> cos_sum, sin_sum, cos_sum_old, sin_sum_old;
  CassEnergy energy{};
  bool energy_valid = false;
};

struct Mol {
  int is = -1, ibox = -1;
  bool live = false;
  std::vector<double> r;       // [natoms][3]
  std::vector<char> exist;
  double com[3] = {0, 0, 0};
  double max_dcom = 0;
  std::vector<double> cos_mol, sin_mol, cos_mol_old, sin_mol_old;
};

// CBMC atom-pair energy table of one box (Create_Atompair_Nrg_table,
// atompair_nrg_table_routines.f90:149-261): bin i (1-based) holds the pair
// energy at the midpoint of [rcut_low^2 + (i-1) step, rcut_low^2 + i step).
struct CbmcTab {
  int res = 0;
  double step = 0, shift = 0;   // rsq_step, rsq_shifter
  std::vector<double> v;        // [ntypes][ntypes][res] vdW part
  std::vector<double> f2;       // [res] Coulomb kernel, times (q_i cf) q_j
};

}  // namespace

struct orc_ctx {
  int nspecies = 0, ntypes = 0, nboxes = 0;
  int max_kvec = 100000;
  std::vector<int> max_mol, mol_base;
  std::vector<double> eps, sig, mie_n, mie_m;  // [ntypes*ntypes]
  std::vector<Species> sp;
  std::vector<Box> box;
  std::vector<Mol> mol;  // slot = mol_base[is] + im
  // live slots of each box in slot order (species-major, locate order), the
  // counterpart of the reference's locate(:, is, ibox) arrays; sp_off[ibox][is]
  // is the first member of species is
  std::vector<std::vector<int>> members, sp_off;
  bool members_dirty = true;
  // CBMC options (cass_set_cbmc_options) and what they derive
  CassCBMCOptions opt{};
  bool cbmc_dirty = true;
  std::vector<CbmcTab> tab;     // per box, when opt.energy_table_res > 0
  std::vector<double> rminsq;   // [ntypes][ntypes] r_min^2 of check_overlap
  double rlowsq = 0.0;          // rcut_low^2 shared by the boxes
  // the state orc_volume_scale keeps for orc_volume_restore, per box
  struct VolSave {
    bool saved = false;
    CassBoxDesc desc{};
    CassEnergy energy{};
    std::vector<int> im, is;
    std::vector<double> xyz;
  };
  std::vector<VolSave> vol;
};

namespace {

inline Mol& mol_of(orc_ctx* c, int is, int im) { return c->mol[c->mol_base[is] + im]; }

void refresh_members(orc_ctx* c) {
  if (!c->members_dirty) return;
  c->members.assign(c->nboxes, {});
  c->sp_off.assign(c->nboxes, std::vector<int>(c->nspecies + 1, 0));
  for (size_t slot = 0; slot < c->mol.size(); ++slot) {
    const Mol& m = c->mol[slot];
    if (m.live && m.ibox >= 0 && m.ibox < c->nboxes) c->members[m.ibox].push_back((int)slot);
  }
  for (int b = 0; b < c->nboxes; ++b) {
    const std::vector<int>& mem = c->members[b];
    size_t k = 0;
    for (int is = 0; is <= c->nspecies; ++is) {
      const int lim = is < c->nspecies ? c->mol_base[is] : INT32_MAX;
      while (k < mem.size() && mem[k] < lim) ++k;
      c->sp_off[b][is] = (int)k;
    }
  }
  c->members_dirty = false;
}

// ---------------------------------------------------------------------------
// lfsr258 generator, random_generators.f90:95-122 (rranf), plus the
// per-insertion seeding used by the batched Widom path (see seed_stream).
struct Rng {
  int64_t s[5];
  double next() {
    uint64_t s1 = (uint64_t)s[0], s2 = (uint64_t)s[1], s3 = (uint64_t)s[2], s4 = (uint64_t)s[3],
             s5 = (uint64_t)s[4], b;
    // ISHFT with a negative count is a logical right shift
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
    s[0] = (int64_t)s1; s[1] = (int64_t)s2; s[2] = (int64_t)s3; s[3] = (int64_t)s4; s[4] = (int64_t)s5;
    int64_t x = (int64_t)(s1 ^ s2 ^ s3 ^ s4 ^ s5);
    return (double)x * 5.4210108624275221E-20 + 0.5;
  }
};

inline uint64_t splitmix64(uint64_t& st) {
  uint64_t z = (st += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One independent lfsr258 stream per (seed, box, insertion): five splitmix64
// outputs, each forced above the component's minimum state (the same rule as
// init_seeds, random_generators.f90:51-91).
Rng seed_stream(uint64_t seed, int64_t ibox, int64_t ins) {
  uint64_t st = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(ibox + 1)) ^
                (0x8CB92BA72F3D8DD7ull * (uint64_t)(ins + 1));
  Rng r;
  const uint64_t mins[5] = {1ull, 511ull, 4095ull, 131071ull, 8388607ull};
  for (int k = 0; k < 5; ++k) {
    uint64_t v = splitmix64(st);
    if ((v & ~mins[k]) == 0) v |= (mins[k] + 1);
    r.s[k] = (int64_t)v;
  }
  return r;
}

// ---------------------------------------------------------------------------
// Minimum_Image_Separation, cubic/orthorhombic branch
// (minimum_image_separation.f90:60-82).
inline void min_image(const Box& b, double& dx, double& dy, double& dz) {
  if (dx > b.hL[0]) dx -= b.L[0]; else if (dx < -b.hL[0]) dx += b.L[0];
  if (dy > b.hL[1]) dy -= b.L[1]; else if (dy < -b.hL[1]) dy += b.L[1];
  if (dz > b.hL[2]) dz -= b.L[2]; else if (dz < -b.hL[2]) dz += b.L[2];
}

// Check_AtomPair_Cutoff (energy_routines.f90:3092-3195)
inline void check_atompair_cutoff(const Box& b, double r2, bool cbmc, bool& get_vdw, bool& get_qq) {
  get_vdw = false;
  get_qq = false;
  if (b.vdw_style == CASS_VDW_LJ) {
    if (cbmc) get_vdw = r2 <= b.rcut_cbmcsq;
    else if (b.vdw_sum_style == CASS_VDW_SUM_CUT || b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT ||
             b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL || b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT_FORCE)
      get_vdw = r2 <= b.rcut_vdwsq;
    else if (b.vdw_sum_style == CASS_VDW_SUM_MINIMUM || b.vdw_sum_style == CASS_VDW_SUM_CHARMM)
      get_vdw = true;
    else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH)
      get_vdw = r2 <= b.roff_switch_sq;
  } else if (b.vdw_style == CASS_VDW_MIE) {
    if (cbmc) get_vdw = r2 <= b.rcut_cbmcsq;
    else if (b.vdw_sum_style == CASS_VDW_SUM_CUT || b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT ||
             b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL)
      get_vdw = r2 <= b.rcut_vdwsq;
  }
  if (b.charge_style == CASS_CHARGE_COUL) {
    if (b.charge_sum_style == CASS_QQ_CUT || b.charge_sum_style == CASS_QQ_EWALD ||
        b.charge_sum_style == CASS_QQ_DSF)
      get_qq = cbmc ? (r2 <= b.rcut_cbmcsq) : (r2 <= b.rcut_coulsq);
    else if (b.charge_sum_style == CASS_QQ_MINIMUM)
      get_qq = true;
  }
}

// Abramowitz-Stegun 7.1.26 erfc of Compute_AtomPair_Ewald_Real
// (energy_routines.f90:2143-2163).
inline double erfc_as(double x) {
  const double A1 = 0.254829592, A2 = -0.284496736, A3 = 1.421413741, A4 = -1.453152027,
               A5 = 1.061405429, P = 0.3275911;
  double T = 1.0 / (1.0 + P * x);
  double xsq = x * x;
  double TP = T * (A1 + T * (A2 + T * (A3 + T * (A4 + T * A5))));
  return TP * std::exp(-xsq);
}

struct PairE {
  double intra_vdw = 0, intra_qq = 0, inter_vdw = 0, inter_qq = 0;
};

// Compute_AtomPair_Energy (energy_routines.f90:1831-2053) with
// Compute_AtomPair_Ewald_Real (:2088-2166) and Compute_AtomPair_DSF_Energy
// (:2056-2082).  Existence checks are done by the callers.
PairE atompair_energy(const orc_ctx* c, const Box& b, double r2, int is, int ia, int js, int ja,
                      bool same_mol, bool get_vdw, bool get_qq) {
  PairE e;
  const Species& si = c->sp[is];
  const Species& sj = c->sp[js];
  int it = si.type[ia], jt = sj.type[ja];
  if (get_vdw && it >= 0 && jt >= 0) {
    double Eij = 0.0;
    int k = it * c->ntypes + jt;
    if (b.vdw_style == CASS_VDW_LJ) {
      double eps = c->eps[k], sig = c->sig[k];
      if (same_mol) eps = eps * si.vdw_scale[ia * si.natoms + ja];
      double SigByR2 = (sig * sig) / r2;
      double SigByR6 = SigByR2 * SigByR2 * SigByR2;
      double SigByR12 = SigByR6 * SigByR6;
      Eij = 4.0 * eps * (SigByR12 - SigByR6);
      if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
        double s2 = sig * sig / b.rcut_vdwsq;
        double s6 = s2 * s2 * s2, s12 = s6 * s6;
        Eij = Eij - 4.0 * eps * (s12 - s6);
      } else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) {
        if (r2 < b.ron_switch_sq) {
        } else if (r2 <= b.roff_switch_sq) {
          double d = b.roff_switch_sq - r2;
          double fscale = d * d * (b.switch_factor2 + 2.0 * r2) * b.switch_factor1;
          Eij = fscale * Eij;
        } else {
          Eij = 0.0;
        }
      } else if (b.vdw_sum_style == CASS_VDW_SUM_CHARMM) {
        Eij = eps * (SigByR12 - 2.0 * SigByR6);
      } else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT_FORCE) {
        double s2 = sig * sig / b.rcut_vdwsq;
        double s6 = s2 * s2 * s2, s12 = s6 * s6;
        Eij = Eij - 4.0 * eps * (s12 - s6);
        double rij = std::sqrt(r2), rc = std::sqrt(b.rcut_vdwsq);
        double dE = -24.0 * eps * (2.0 * s12 / rc - s6 / rc);
        Eij = Eij - (rij - rc) * dE;
      }
    } else if (b.vdw_style == CASS_VDW_MIE) {
      double eps = c->eps[k], sig = c->sig[k], n = c->mie_n[k], m = c->mie_m[k];
      if (same_mol) eps = eps * si.vdw_scale[ia * si.natoms + ja];
      double rij = std::sqrt(r2), rc = std::sqrt(b.rcut_vdwsq);
      double coeff = n / (n - m) * std::pow(n / m, m / (n - m));
      double s = sig / rij;
      Eij = coeff * eps * (std::pow(s, n) - std::pow(s, m));
      if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
        double sc = sig / rc;
        Eij = Eij - coeff * eps * (std::pow(sc, n) - std::pow(sc, m));
      }
    }
    if (same_mol) e.intra_vdw = Eij; else e.inter_vdw = Eij;
  }
  if (get_qq) {
    double qi = si.q[ia], qj = sj.q[ja];
    if (b.charge_sum_style == CASS_QQ_EWALD) {
      double rij = std::sqrt(r2);
      double erf_val = 1.0 - erfc_as(b.alpha_ewald * rij);
      double Eij = qi * qj / rij * CHARGE_FACTOR;
      if (same_mol) {
        e.intra_qq = si.qq_scale[ia * si.natoms + ja] * Eij;
        e.inter_qq = 0.0;
      } else {
        e.intra_qq = 0.0;
        e.inter_qq = Eij;
      }
      e.inter_qq = e.inter_qq - erf_val * Eij;
    } else if (b.charge_sum_style == CASS_QQ_DSF) {
      double rij = std::sqrt(r2);
      double cfqq = qi * qj * CHARGE_FACTOR;
      double Eij = b.dsf_factor2 * (rij - b.rcut_coul) - b.dsf_factor1 + std::erfc(b.alpha_dsf * rij) / rij;
      Eij = Eij * cfqq;
      if (same_mol) {
        double qsc = si.qq_scale[ia * si.natoms + ja];
        e.intra_qq = Eij - (1.0 - qsc) * (cfqq / rij);
      } else {
        e.inter_qq = Eij;
      }
    } else {
      double Eij = CHARGE_FACTOR * (qi * qj) / std::sqrt(r2);
      if (same_mol) e.intra_qq += si.qq_scale[ia * si.natoms + ja] * Eij;
      else e.inter_qq += Eij;
    }
  }
  return e;
}

// Atoms of a molecule-like object: coordinates, existence, COM, max_dcom.
struct MolView {
  int is;
  const double* r;
  const char* exist;
  const double* com;
  double max_dcom;
};

// Check_MoleculePair_Cutoff (energy_routines.f90:3027-3088)
inline bool check_molpair_cutoff(const Box& b, const MolView& a, const MolView& m, bool cbmc) {
  if (b.vdw_sum_style == CASS_VDW_SUM_MINIMUM) return true;
  double dx = a.com[0] - m.com[0], dy = a.com[1] - m.com[1], dz = a.com[2] - m.com[2];
  min_image(b, dx, dy, dz);
  double rcom = std::sqrt(dx * dx + dy * dy + dz * dz);
  double rint = (cbmc ? b.rcut_cbmc : b.rcut_max) + a.max_dcom + m.max_dcom;
  return !(rcom > rint);
}

// Compute_MoleculePair_Energy (energy_routines.f90:1589-1730): molecule a
// (the query) against molecule m; early return on core overlap.
bool molpair_energy(const orc_ctx* c, const Box& b, const MolView& a, const MolView& m, bool cbmc,
                    double& vlj, double& vqq, double* eabs = nullptr) {
  vlj = 0.0;
  vqq = 0.0;
  const Species& sa = c->sp[a.is];
  const Species& sm = c->sp[m.is];
  for (int ia = 0; ia < sa.natoms; ++ia) {
    if (!a.exist[ia]) continue;
    for (int ja = 0; ja < sm.natoms; ++ja) {
      if (!m.exist[ja]) continue;
      double dx = a.r[3 * ia] - m.r[3 * ja], dy = a.r[3 * ia + 1] - m.r[3 * ja + 1],
             dz = a.r[3 * ia + 2] - m.r[3 * ja + 2];
      min_image(b, dx, dy, dz);
      double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < b.rcut_lowsq) return true;
      bool gv, gq;
      check_atompair_cutoff(b, r2, cbmc, gv, gq);
      if (cbmc && !sa.l_coul_cbmc) gq = false;
      if (gv || gq) {
        PairE e = atompair_energy(c, b, r2, a.is, ia, m.is, ja, false, gv, gq);
        vlj += e.inter_vdw;
        vqq += e.inter_qq;
        if (eabs) *eabs += std::fabs(e.inter_vdw) + std::fabs(e.inter_qq);
      }
    }
  }
  return false;
}

// AtomPair_VdW_Energy_Vector (energy_routines.f90:1733-1829) at one r^2:
// the vdW pair energy of the box's style with no cutoff test
double vdw_vector_entry(const orc_ctx* c, const Box& b, int it, int jt, double rsq) {
  if (it < 0 || jt < 0) return 0.0;
  const int k = it * c->ntypes + jt;
  const double eps = c->eps[k], sig = c->sig[k];
  if (b.vdw_style == CASS_VDW_LJ) {
    const double s2 = (sig * sig) / rsq, s6 = s2 * s2 * s2, s12 = s6 * s6;
    double e = 4.0 * eps * (s12 - s6);
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
      const double c2 = sig * sig / b.rcut_vdwsq, c6 = c2 * c2 * c2, c12 = c6 * c6;
      e = e - 4.0 * eps * (c12 - c6);
    } else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) {
      if (rsq < b.ron_switch_sq) {
      } else if (rsq > b.roff_switch_sq) {
        e = 0.0;
      } else {
        const double d = b.roff_switch_sq - rsq;
        e = d * d * (b.switch_factor2 + 2.0 * rsq) * b.switch_factor1 * e;
      }
    } else if (b.vdw_sum_style == CASS_VDW_SUM_CHARMM) {
      e = eps * (s12 - 2.0 * s6);
    } else if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT_FORCE) {
      const double c2 = sig * sig / b.rcut_vdwsq, c6 = c2 * c2 * c2, c12 = c6 * c6;
      const double rc = std::sqrt(b.rcut_vdwsq);
      const double dedr = -24.0 * eps * (2.0 * c12 - c6) / rc;
      e = e - 4.0 * eps * (c12 - c6) - (std::sqrt(rsq) - rc) * dedr;
    }
    return e;
  }
  if (b.vdw_style == CASS_VDW_MIE) {
    const double n = c->mie_n[k], m = c->mie_m[k];
    const double rc = std::sqrt(b.rcut_vdwsq);
    const double coeff = n / (n - m) * std::pow(n / m, m / (n - m));
    const double sr = sig / std::sqrt(rsq);
    double e = coeff * eps * (std::pow(sr, n) - std::pow(sr, m));
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
      const double sc = sig / rc;
      e = e - coeff * eps * (std::pow(sc, n) - std::pow(sc, m));
    }
    return e;
  }
  return 0.0;
}

// The tables the CBMC options derive: the energy table per box
// (atompair_nrg_table_routines.f90:149-261, with rsq_step and rsq_shifter of
// :163-168) and r_min^2 per type pair (create_nonbond_table.f90:219-220,
// 285-303, 396-418 with the type charge ranges of :144-153)
int build_cbmc(orc_ctx* c) {
  if (!c->cbmc_dirty) return CASS_OK;
  const int nt = c->ntypes;
  double rlow = -1.0, max_cbmcsq = 0.0, min_beta = 0.0;
  int charge_style1 = CASS_CHARGE_NONE;
  bool first = true;
  for (int ib = 0; ib < c->nboxes; ++ib) {
    const Box& b = c->box[ib];
    if (!b.defined) continue;
    if (first) {
      rlow = b.rcut_lowsq;
      min_beta = b.beta;
      first = false;
    } else if (b.rcut_lowsq != rlow) {
      return fail(CASS_EUNSUPPORTED, "CBMC options need one rcut_low for all boxes");
    }
    if (ib == 0) charge_style1 = b.charge_style;
    max_cbmcsq = std::max(max_cbmcsq, b.rcut_cbmcsq);
    min_beta = std::min(min_beta, b.beta);
  }
  if (first) return fail(CASS_ESTATE, "CBMC options need a box");
  c->rlowsq = rlow;
  // r_min^2 per type pair
  c->rminsq.assign((size_t)nt * nt, rlow);
  if (c->opt.rmin_u_max > 0.0) {
    std::vector<double> qmin(nt, 0.0), qmax(nt, 0.0);
    std::vector<char> seen(nt, 0);
    for (const Species& sp : c->sp) {
      if (!sp.defined) continue;
      for (int a = 0; a < sp.natoms; ++a) {
        const int t = sp.type[a];
        if (t < 0) continue;
        if (seen[t]) {
          qmin[t] = std::min(qmin[t], sp.q[a]);
          qmax[t] = std::max(qmax[t], sp.q[a]);
        } else {
          qmin[t] = qmax[t] = sp.q[a];
          seen[t] = 1;
        }
      }
    }
    const double u_base = c->opt.rmin_u_max / min_beta;
    const double rcut_low = std::sqrt(rlow);
    for (int i = 0; i < nt; ++i)
      for (int j = 0; j < nt; ++j) {
        const double eps = c->eps[i * nt + j], sig = c->sig[i * nt + j];
        if (!(eps > 0.0)) continue;
        double min_uq = 0.0;
        if (charge_style1 != CASS_CHARGE_NONE) {
          double qp = std::min(qmin[i] * qmax[j], qmax[i] * qmin[j]);
          if (qp <= 0.0) {
            min_uq = qp * CHARGE_FACTOR / rcut_low;
          } else {
            qp = std::min(qmin[i] * qmin[j], qmax[i] * qmax[j]);
            min_uq = qp * CHARGE_FACTOR / sig;
          }
        }
        const double umax = std::max(u_base - min_uq, 0.0);
        const double lambda = 0.5 * (1.0 + std::sqrt(1.0 + umax / eps));
        c->rminsq[i * nt + j] = sig * sig / std::pow(lambda, 1.0 / 3.0);
      }
  }
  if (c->opt.sector_overlap)
    for (int ib = 0; ib < c->nboxes; ++ib) {
      const Box& b = c->box[ib];
      if (!b.defined) continue;
      for (double r2 : c->rminsq)
        if (r2 > b.rcut_cbmcsq) return fail(CASS_EUNSUPPORTED, "r_min exceeds rcut_cbmc");
    }
  // energy tables
  c->tab.assign(c->nboxes, CbmcTab{});
  const int res = c->opt.energy_table_res;
  if (res > 0)
    for (int ib = 0; ib < c->nboxes; ++ib) {
      const Box& b = c->box[ib];
      if (!b.defined) continue;
      CbmcTab& T = c->tab[ib];
      T.res = res;
      T.step = (max_cbmcsq - rlow) / res;
      T.shift = rlow - T.step;
      T.v.assign((size_t)nt * nt * res, 0.0);
      T.f2.assign(res, 0.0);
      for (int i = 1; i <= res; ++i) {
        const double lb = T.shift + T.step * i;
        const double mp = lb + 0.5 * T.step;
        const double rij = std::sqrt(mp);
        double f2 = 0.0;
        if (b.charge_style == CASS_CHARGE_COUL) {
          if (b.charge_sum_style == CASS_QQ_EWALD) f2 = std::erfc(b.alpha_ewald * rij) / rij;
          else if (b.charge_sum_style == CASS_QQ_DSF)
            f2 = b.dsf_factor2 * (rij - b.rcut_coul) - b.dsf_factor1 + std::erfc(b.alpha_dsf * rij) / rij;
          else if (b.charge_sum_style == CASS_QQ_CUT) f2 = 1.0 / rij;
        }
        T.f2[i - 1] = f2;
        for (int ti = 0; ti < nt; ++ti)
          for (int tj = 0; tj < nt; ++tj) T.v[((size_t)ti * nt + tj) * res + (i - 1)] = vdw_vector_entry(c, b, ti, tj, mp);
      }
    }
  c->cbmc_dirty = false;
  return CASS_OK;
}

// Estimate_MoleculePair_Energy (energy_routines.f90:1528-1587): the combined
// vdW + Coulomb energy of molecule a (the solute) with m (the solvent) from
// the box's table; true on overlap (a pair below rcut_low inside rcut_cbmc)
bool molpair_estimate(const orc_ctx* c, int ibox, const MolView& a, const MolView& m, double& e) {
  const Box& b = c->box[ibox];
  const CbmcTab& T = c->tab[ibox];
  const Species& sa = c->sp[a.is];
  const Species& sm = c->sp[m.is];
  const int nt = c->ntypes;
  const double rcs = b.rcut_cbmcsq - T.shift;
  e = 0.0;
  for (int ia = 0; ia < sa.natoms; ++ia) {
    if (!a.exist[ia]) continue;
    for (int ja = 0; ja < sm.natoms; ++ja) {
      if (!m.exist[ja]) continue;
      double dx = a.r[3 * ia] - m.r[3 * ja], dy = a.r[3 * ia + 1] - m.r[3 * ja + 1], dz = a.r[3 * ia + 2] - m.r[3 * ja + 2];
      min_image(b, dx, dy, dz);
      const double rs = dx * dx + dy * dy + dz * dz - T.shift;
      if (rs >= rcs) continue;
      if (rs < T.step) return true;
      int bin = (int)(rs / T.step);  // 1-based; at most res except within rounding of the cutoff
      if (bin > T.res) bin = T.res;
      const int ta = sa.type[ia], tj = sm.type[ja];
      const double ev = (ta >= 0 && tj >= 0) ? T.v[((size_t)ta * nt + tj) * T.res + (bin - 1)] : 0.0;
      e += ev + T.f2[bin - 1] * ((sa.q[ia] * CHARGE_FACTOR) * sm.q[ja]);
    }
  }
  return false;
}

// check_overlap (sector_routines.f90:160-233) for atom ia of species is at
// p: true if a box atom lies closer than r_min(type pair)
bool check_overlap_atom(const orc_ctx* c, int ibox, int is, int ia, const double* p) {
  const Box& b = c->box[ibox];
  const int nt = c->ntypes, ta = c->sp[is].type[ia];
  for (int slot : c->members[ibox]) {
    const Mol& m = c->mol[slot];
    const Species& sm = c->sp[m.is];
    for (int ja = 0; ja < sm.natoms; ++ja) {
      if (!m.exist[ja]) continue;
      double dx = m.r[3 * ja] - p[0], dy = m.r[3 * ja + 1] - p[1], dz = m.r[3 * ja + 2] - p[2];
      min_image(b, dx, dy, dz);
      const int tj = sm.type[ja];
      const double rmin2 = (ta >= 0 && tj >= 0) ? c->rminsq[(size_t)ta * nt + tj] : c->rlowsq;
      if (dx * dx + dy * dy + dz * dz < rmin2) return true;
    }
  }
  return false;
}

MolView view_of(const Mol& m) { return MolView{m.is, m.r.data(), m.exist.data(), m.com, m.max_dcom}; }

// Get_COM (get_com.f90:45-105)
void get_com(const orc_ctx* c, int is, const double* r, const char* exist, double* com) {
  const Species& s = c->sp[is];
  double tm = 0, x = 0, y = 0, z = 0;
  for (int k = 0; k < s.natoms; ++k) {
    if (!exist[k]) continue;
    double m = s.mass[k];
    tm += m;
    x += m * r[3 * k];
    y += m * r[3 * k + 1];
    z += m * r[3 * k + 2];
  }
  com[0] = x / tm;
  com[1] = y / tm;
  com[2] = z / tm;
}

// Compute_Max_Com_Distance (get_com.f90:220-295)
double max_com_distance(const orc_ctx* c, int is, const double* r, const char* exist, const double* com) {
  double dmax = 0.0;
  for (int k = 0; k < c->sp[is].natoms; ++k) {
    if (!exist[k]) continue;
    double dx = r[3 * k] - com[0], dy = r[3 * k + 1] - com[1], dz = r[3 * k + 2] - com[2];
    dmax = std::max(dmax, dx * dx + dy * dy + dz * dz);
  }
  return std::sqrt(dmax);
}

void refresh_com(orc_ctx* c, Mol& m) {
  get_com(c, m.is, m.r.data(), m.exist.data(), m.com);
  m.max_dcom = max_com_distance(c, m.is, m.r.data(), m.exist.data(), m.com);
}

// Molecule loop of Compute_Molecule_Nonbond_Inter_Energy (energy_routines.f90:
// 1088-1206) and of its _Widom variant (:1266-1297): query a against every
// live molecule of box b except slot `skip` (-1 = none).  Returns overlap.
bool mol_inter_energy(const orc_ctx* c, int ibox, const MolView& a, int skip, bool cbmc, double& evdw,
                      double& eqq, double* eabs = nullptr) {
  const Box& b = c->box[ibox];
  evdw = 0.0;
  eqq = 0.0;
  for (int slot : c->members[ibox]) {
    if (slot == skip) continue;
    const Mol& m = c->mol[slot];
    MolView mv = view_of(m);
    if (!check_molpair_cutoff(b, a, mv, cbmc)) continue;
    double vlj, vqq;
    if (cbmc && c->opt.energy_table_res > 0) {
      // the estimate is the combined vdW + Coulomb energy (energy_routines.f90:1182-1191)
      if (molpair_estimate(c, ibox, a, mv, vlj)) return true;
      vqq = 0.0;
    } else if (molpair_energy(c, b, a, mv, cbmc, vlj, vqq, eabs)) {
      return true;
    }
    evdw += vlj;
    eqq += vqq;
  }
  return false;
}

// Compute_Molecule_Nonbond_Intra_Energy (energy_routines.f90:980-1085)
bool mol_intra_energy(const orc_ctx* c, const Box& b, int is, const double* r, const char* exist, bool cbmc,
                      double& eivdw, double& eiqq, double& eoqq) {
  const Species& s = c->sp[is];
  eivdw = eiqq = eoqq = 0.0;
  for (int ia = 0; ia < s.natoms; ++ia) {
    if (!exist[ia]) continue;
    for (int ja = ia + 1; ja < s.natoms; ++ja) {
      if (!exist[ja]) continue;
      double dx = r[3 * ia] - r[3 * ja], dy = r[3 * ia + 1] - r[3 * ja + 1], dz = r[3 * ia + 2] - r[3 * ja + 2];
      double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 <= b.rcut_lowsq && !s.bonded[ia * s.natoms + ja]) return true;
      bool gv, gq;
      check_atompair_cutoff(b, r2, cbmc, gv, gq);
      if (cbmc && s.l_coul_cbmc) gq = false;
      if (gv || gq) {
        PairE e = atompair_energy(c, b, r2, is, ia, is, ja, true, gv, gq);
        eivdw += e.intra_vdw;
        eiqq += e.intra_qq;
        eoqq += e.inter_qq;
      }
    }
  }
  return false;
}

// Compute_Atom_Nonbond_Intra_Energy (energy_routines.f90:691-737)
bool atom_intra_energy(const orc_ctx* c, const Box& b, int is, int ia, const double* r, const char* exist,
                       bool cbmc, double& eivdw, double& eiqq, double& eoqq) {
  const Species& s = c->sp[is];
  eivdw = eiqq = eoqq = 0.0;
  for (int ja = 0; ja < s.natoms; ++ja) {
    if (ja == ia || !exist[ja]) continue;
    bool nzv = s.vdw_scale[ia * s.natoms + ja] > 0.0;
    bool nzq = s.qq_scale[ia * s.natoms + ja] > 0.0;
    if (!(nzv || nzq)) continue;
    double dx = r[3 * ja] - r[3 * ia], dy = r[3 * ja + 1] - r[3 * ia + 1], dz = r[3 * ja + 2] - r[3 * ia + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < b.rcut_lowsq && nzv) return true;
    bool gv, gq;
    check_atompair_cutoff(b, r2, cbmc, gv, gq);
    gv = gv && nzv;
    gq = gq && nzq;
    if (gv || gq) {
      PairE e = atompair_energy(c, b, r2, is, ja, is, ia, true, gv, gq);
      eivdw += e.intra_vdw;
      eiqq += e.intra_qq;
      eoqq += e.inter_qq;
    }
  }
  return false;
}

// Bonded energies (energy_routines.f90:197-496) with Get_Bond_Angle and
// Get_Dihedral_Angle_COS (internal_coordinate_routines.f90:188-410).
double bond_energy(const Species& s, const double* r) {
  double e = 0;
  for (size_t k = 0; k < s.bond_kind.size(); ++k) {
    if (s.bond_kind[k] != CASS_BONDED_HARMONIC) continue;
    int a = s.bond_atoms[2 * k], b = s.bond_atoms[2 * k + 1];
    double dx = r[3 * a] - r[3 * b], dy = r[3 * a + 1] - r[3 * b + 1], dz = r[3 * a + 2] - r[3 * b + 2];
    double l = std::sqrt(dx * dx + dy * dy + dz * dz);
    double kk = s.bond_param[2 * k], l0 = s.bond_param[2 * k + 1];
    e += kk * (l - l0) * (l - l0);
  }
  return e;
}

double bond_angle(const double* r, int a1, int a2, int a3) {
  double rx21 = r[3 * a2] - r[3 * a1], ry21 = r[3 * a2 + 1] - r[3 * a1 + 1], rz21 = r[3 * a2 + 2] - r[3 * a1 + 2];
  double rx32 = r[3 * a3] - r[3 * a2], ry32 = r[3 * a3 + 1] - r[3 * a2 + 1], rz32 = r[3 * a3 + 2] - r[3 * a2 + 2];
  double C23 = rx21 * rx32 + ry21 * ry32 + rz21 * rz32;
  double C22 = rx21 * rx21 + ry21 * ry21 + rz21 * rz21;
  double C33 = rx32 * rx32 + ry32 * ry32 + rz32 * rz32;
  double inv = 1.0 / std::sqrt(C33 * C22);
  double ct = C23 * inv;
  ct = std::min(ct, 0.999999);
  ct = std::max(ct, -0.999999);
  return PI - std::acos(ct);
}

double angle_energy(const Species& s, const double* r, const char* exist) {
  double e = 0;
  for (size_t k = 0; k < s.angle_kind.size(); ++k) {
    if (s.angle_kind[k] != CASS_BONDED_HARMONIC) continue;
    int a1 = s.angle_atoms[3 * k], a2 = s.angle_atoms[3 * k + 1], a3 = s.angle_atoms[3 * k + 2];
    (void)exist;
    double th = bond_angle(r, a1, a2, a3);
    double kk = s.angle_param[2 * k], t0 = s.angle_param[2 * k + 1];
    e += kk * (th - t0) * (th - t0);
  }
  return e;
}

double dihedral_cos(const double* r, int a1, int a2, int a3, int a4) {
  double rx12 = r[3 * a1] - r[3 * a2], ry12 = r[3 * a1 + 1] - r[3 * a2 + 1], rz12 = r[3 * a1 + 2] - r[3 * a2 + 2];
  double rx32 = r[3 * a3] - r[3 * a2], ry32 = r[3 * a3 + 1] - r[3 * a2 + 1], rz32 = r[3 * a3 + 2] - r[3 * a2 + 2];
  double rx34 = r[3 * a3] - r[3 * a4], ry34 = r[3 * a3 + 1] - r[3 * a4 + 1], rz34 = r[3 * a3 + 2] - r[3 * a4 + 2];
  double mx = ry12 * rz32 - ry32 * rz12;
  double my = -rx12 * rz32 + rz12 * rx32;
  double mz = rx12 * ry32 - ry12 * rx32;
  double nx = ry32 * rz34 - rz32 * ry34;
  double ny = -rx32 * rz34 + rz32 * rx34;
  double nz = rx32 * ry34 - ry32 * rx34;
  double msq = mx * mx + my * my + mz * mz;
  double nsq = nx * nx + ny * ny + nz * nz;
  double mdn = mx * nx + my * ny + mz * nz;
  return mdn / std::sqrt(msq * nsq);
}

// Compute_Molecule_Dihedral_Energy, RB branch (energy_routines.f90:384-398)
double dihedral_energy(const Species& s, const double* r, const char* exist) {
  double e = 0;
  size_t nd = s.dih_atoms.size() / 4;
  for (size_t k = 0; k < nd; ++k) {
    int a1 = s.dih_atoms[4 * k], a2 = s.dih_atoms[4 * k + 1], a3 = s.dih_atoms[4 * k + 2], a4 = s.dih_atoms[4 * k + 3];
    if (!(exist[a1] && exist[a2] && exist[a3] && exist[a4])) continue;
    double c1 = dihedral_cos(r, a1, a2, a3, a4);
    double cv[6];
    cv[0] = 1.0;
    cv[1] = c1;
    cv[2] = cv[1] * cv[1];
    cv[3] = cv[1] * cv[2];
    cv[4] = cv[2] * cv[2];
    cv[5] = cv[2] * cv[3];
    double d = 0;
    for (int j = 0; j < 6; ++j) d += cv[j] * s.dih_rb[6 * k + j];
    e += d;
  }
  return e;
}

// Compute_Molecule_Improper_Energy, harmonic (energy_routines.f90:451-496)
double improper_energy(const Species& s, const double* r) {
  double e = 0;
  size_t ni = s.imp_atoms.size() / 4;
  for (size_t k = 0; k < ni; ++k) {
    int a1 = s.imp_atoms[4 * k], a2 = s.imp_atoms[4 * k + 1], a3 = s.imp_atoms[4 * k + 2], a4 = s.imp_atoms[4 * k + 3];
    double rx12 = r[3 * a1] - r[3 * a2], ry12 = r[3 * a1 + 1] - r[3 * a2 + 1], rz12 = r[3 * a1 + 2] - r[3 * a2 + 2];
    double rx32 = r[3 * a3] - r[3 * a2], ry32 = r[3 * a3 + 1] - r[3 * a2 + 1], rz32 = r[3 * a3 + 2] - r[3 * a2 + 2];
    double rx34 = r[3 * a3] - r[3 * a4], ry34 = r[3 * a3 + 1] - r[3 * a4 + 1], rz34 = r[3 * a3 + 2] - r[3 * a4 + 2];
    double mx = ry12 * rz32 - ry32 * rz12, my = -rx12 * rz32 + rz12 * rx32, mz = rx12 * ry32 - ry12 * rx32;
    double nx = ry32 * rz34 - rz32 * ry34, ny = -rx32 * rz34 + rz32 * rx34, nz = rx32 * ry34 - ry32 * rx34;
    double cphi = (mx * nx + my * ny + mz * nz) / std::sqrt((mx * mx + my * my + mz * mz) * (nx * nx + ny * ny + nz * nz));
    cphi = std::min(1.0, std::max(-1.0, cphi));
    double r12dn = rx12 * nx + ry12 * ny + rz12 * nz;
    double phi = std::copysign(std::acos(cphi), r12dn);
    double kk = s.imp_param[2 * k], p0 = s.imp_param[2 * k + 1];
    e += kk * (phi - p0) * (phi - p0);
  }
  return e;
}

// ---------------------------------------------------------------------------
// Ewald (energy_routines.f90:2170-2323, 2326-2550, 4111-4231)

// Ewald_Reciprocal_Lattice_Vector_Setup, cubic/orthorhombic branch (:2260-2311)
int ewald_setup(orc_ctx* c, Box& b) {
  b.hx.clear(); b.hy.clear(); b.hz.clear(); b.hsq.clear(); b.Cn.clear();
  double const_val = 1.0 / (4.0 * b.alpha_ewald * b.alpha_ewald);
  double hcutsq = b.h_ewald_cut * b.h_ewald_cut;
  int kz_max = (int)((b.h_ewald_cut * b.L[2]) / TWOPI) + 1;
  int ky_max = (int)((b.h_ewald_cut * b.L[1]) / TWOPI) + 1;
  int kx_max = (int)((b.h_ewald_cut * b.L[0]) / TWOPI) + 1;
  for (int nz = -kz_max; nz <= kz_max; ++nz)
    for (int ny = -ky_max; ny <= ky_max; ++ny)
      for (int nx = 0; nx <= kx_max; ++nx) {
        if (nx == 0 && ny == 0 && nz == 0) continue;
        double hxv = TWOPI * (double)nx / b.L[0];
        double hyv = TWOPI * (double)ny / b.L[1];
        double hzv = TWOPI * (double)nz / b.L[2];
        double h2 = hxv * hxv + hyv * hyv + hzv * hzv;
        if (h2 < hcutsq) {
          if ((int)b.hx.size() >= c->max_kvec) return fail(CASS_ECAPACITY, "Total number of k vectors exceeded");
          b.hx.push_back(hxv);
          b.hy.push_back(hyv);
          b.hz.push_back(hzv);
          b.hsq.push_back(h2);
          double cn = TWOPI / b.volume * std::exp(-h2 * const_val) / h2;
          if (nx != 0) cn = 2.0 * TWOPI / b.volume * std::exp(-h2 * const_val) / h2;
          b.Cn.push_back(cn);
        }
      }
  size_t nv = b.hx.size();
  b.cos_sum.assign(nv, 0.0);
  b.sin_sum.assign(nv, 0.0);
  return CASS_OK;
}

bool box_has_ewald(const Box& b) {
  return b.charge_style == CASS_CHARGE_COUL && b.charge_sum_style == CASS_QQ_EWALD;
}

void mol_structure_factor(const orc_ctx* c, const Box& b, int is, const double* r, double* cosm, double* sinm) {
  const Species& s = c->sp[is];
  size_t nv = b.hx.size();
  for (size_t i = 0; i < nv; ++i) {
    double cs = 0, sn = 0;
    for (int ia = 0; ia < s.natoms; ++ia) {
      double hdotr = b.hx[i] * r[3 * ia] + b.hy[i] * r[3 * ia + 1] + b.hz[i] * r[3 * ia + 2];
      double q = s.q[ia];
      cs = cs + q * std::cos(hdotr);
      sn = sn + q * std::sin(hdotr);
    }
    cosm[i] = cs;
    sinm[i] = sn;
  }
}

// Compute_System_Ewald_Reciprocal_Energy (:4111-4231)
double system_recip(orc_ctx* c, int ibox) {
  Box& b = c->box[ibox];
  size_t nv = b.hx.size();
  std::fill(b.cos_sum.begin(), b.cos_sum.end(), 0.0);
  std::fill(b.sin_sum.begin(), b.sin_sum.end(), 0.0);
  for (int slot : c->members[ibox]) {
    Mol& m = c->mol[slot];
    const int is = m.is;
    if (!c->sp[is].has_charge) continue;
    {
      m.cos_mol.assign(nv, 0.0);
      m.sin_mol.assign(nv, 0.0);
      mol_structure_factor(c, b, is, m.r.data(), m.cos_mol.data(), m.sin_mol.data());
      for (size_t i = 0; i < nv; ++i) {
        b.cos_sum[i] += m.cos_mol[i];
        b.sin_sum[i] += m.sin_mol[i];
      }
    }
  }
  double E = 0;
  for (size_t i = 0; i < nv; ++i) E += b.Cn[i] * (b.cos_sum[i] * b.cos_sum[i] + b.sin_sum[i] * b.sin_sum[i]);
  return E * CHARGE_FACTOR;
}

// Compute_System_Self_Energy (:2553-2601)
double system_self(const orc_ctx* c, int ibox) {
  const Box& b = c->box[ibox];
  double es = 0;
  for (int slot : c->members[ibox]) {
    const Species& s = c->sp[c->mol[slot].is];
    for (int ia = 0; ia < s.natoms; ++ia) es = es + s.q[ia] * s.q[ia];
  }
  if (b.charge_sum_style == CASS_QQ_EWALD) return -es * CHARGE_FACTOR * b.alpha_ewald / ROOTPI;
  if (b.charge_sum_style == CASS_QQ_DSF) return -(es * (b.alpha_dsf / ROOTPI + b.dsf_factor1 / 2.0)) * CHARGE_FACTOR;
  return 0.0;
}

// Compute_Molecule_Self_Energy (:2606-2645)
double molecule_self(const orc_ctx* c, const Box& b, int is) {
  const Species& s = c->sp[is];
  double qq = 0;
  for (int ia = 0; ia < s.natoms; ++ia) qq += s.q[ia] * s.q[ia];
  if (b.charge_sum_style == CASS_QQ_EWALD) return -qq * CHARGE_FACTOR * b.alpha_ewald / ROOTPI;
  if (b.charge_sum_style == CASS_QQ_DSF) return -qq * (b.alpha_dsf / ROOTPI + b.dsf_factor1 / 2.0) * CHARGE_FACTOR;
  return 0.0;
}

// Compute_LR_Correction (:2956-3023); nint_beads counts atoms per type.
double lr_correction(const orc_ctx* c, const Box& b, const std::vector<double>& nbeads) {
  double e_lrc = 0.0;
  int nt = c->ntypes;
  if (b.vdw_style == CASS_VDW_LJ) {
    for (int ia = 0; ia < nt; ++ia) {
      double eij = 0.0;
      for (int ja = 0; ja < nt; ++ja) {
        double epsij = c->eps[ia * nt + ja], sigij = c->sig[ia * nt + ja];
        double s2 = sigij * sigij, s6 = s2 * s2 * s2, s12 = s6 * s6;
        eij = eij + nbeads[ja] * 4.0 * epsij * (s12 / (9.0 * b.rcut9) - (s6 / (3.0 * b.rcut3)));
      }
      e_lrc = e_lrc + nbeads[ia] * eij;
    }
    e_lrc = 2.0 * PI * e_lrc / b.volume;
  } else if (b.vdw_style == CASS_VDW_MIE) {
    for (int ia = 0; ia < nt; ++ia) {
      double eij = 0.0;
      for (int ja = 0; ja < nt; ++ja) {
        double epsij = c->eps[ia * nt + ja], sigij = c->sig[ia * nt + ja];
        double n = c->mie_n[ia * nt + ja], m = c->mie_m[ia * nt + ja];
        double coeff = n / (n - m) * std::pow(n / m, m / (n - m));
        double sor = sigij / b.rcut_vdw;
        eij = eij + nbeads[ja] * coeff * epsij * std::pow(b.rcut_vdw, 3.0) *
                        ((std::pow(sor, n) / (3.0 - n)) + (std::pow(sor, m) / (m - 3.0)));
      }
      e_lrc = e_lrc + nbeads[ia] * eij;
    }
    e_lrc = -2.0 * PI * e_lrc / b.volume;
  }
  return e_lrc;
}

std::vector<double> count_beads(const orc_ctx* c, int ibox) {
  std::vector<double> nb(c->ntypes, 0.0);
  for (int slot : c->members[ibox]) {
    const Species& s = c->sp[c->mol[slot].is];
    for (int ia = 0; ia < s.natoms; ++ia)
      if (s.type[ia] >= 0) nb[s.type[ia]] += 1.0;
  }
  return nb;
}

// ---------------------------------------------------------------------------
// CBMC growth (fragment_growth.f90) for a Widom test molecule.

struct TestMol {
  int is;
  std::vector<double> r;
  std::vector<char> exist;
  double com[3];
  double max_dcom;
  MolView view() const { return MolView{is, r.data(), exist.data(), com, max_dcom}; }
};

// Get_Aligner_Hanger (fragment_growth.f90:2135-2185); row-major 3x3.
void aligner_hanger(double v1[3], double v2[3], double al[9], double hg[9]) {
  double n1 = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  for (int i = 0; i < 3; ++i) v1[i] = v1[i] / n1;
  double n2 = std::sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  for (int i = 0; i < 3; ++i) v2[i] = v2[i] / n2;
  double p1[3] = {v1[1] * v2[2] - v1[2] * v2[1], -v1[0] * v2[2] + v1[2] * v2[0], v1[0] * v2[1] - v1[1] * v2[0]};
  double np1 = std::sqrt(p1[0] * p1[0] + p1[1] * p1[1] + p1[2] * p1[2]);
  for (int i = 0; i < 3; ++i) p1[i] = p1[i] / np1;
  double p2[3] = {v1[1] * p1[2] - v1[2] * p1[1], -v1[0] * p1[2] + v1[2] * p1[0], v1[0] * p1[1] - v1[1] * p1[0]};
  double np2 = std::sqrt(p2[0] * p2[0] + p2[1] * p2[1] + p2[2] * p2[2]);
  for (int i = 0; i < 3; ++i) p2[i] = p2[i] / np2;
  for (int i = 0; i < 3; ++i) {
    al[0 * 3 + i] = v1[i];
    al[1 * 3 + i] = p2[i];
    al[2 * 3 + i] = p1[i];
    hg[i * 3 + 0] = v1[i];
    hg[i * 3 + 1] = p2[i];
    hg[i * 3 + 2] = p1[i];
  }
}

// Fragment_Order (fragment_growth.f90:1317-1446)
void fragment_order(const Species& s, int start, std::vector<int>& order, std::vector<int>& live,
                    double& ln_pseq, Rng& rng) {
  std::vector<int> hanging;
  for (int f : s.frag_connect[start])
    if (!live[f]) hanging.push_back(f);
  while (!hanging.empty()) {
    int n = (int)hanging.size();
    std::vector<double> prob(n), cum(n);
    for (int k = 0; k < n; ++k) {
      prob[k] = (double)(s.frag_atoms[hanging[k]].size() - 2);
      cum[k] = (k == 0 ? 0.0 : cum[k - 1]) + prob[k];
    }
    double tot = cum[n - 1];
    for (int k = 0; k < n; ++k) {
      prob[k] = prob[k] / tot;
      cum[k] = cum[k] / tot;
    }
    double u = rng.next();
    int k = 0;
    while (k < n && !(u < cum[k])) ++k;
    if (k >= n) k = n - 1;
    int f = hanging[k];
    ln_pseq = ln_pseq + std::log(prob[k]);
    order.push_back(f);
    live[f] = 1;
    hanging.erase(hanging.begin() + k);
    for (int g : s.frag_connect[f])
      if (!live[g]) hanging.push_back(g);
  }
}

// Compute_Molecule_Nonbond_Inter_Energy_Widom molecule loop (energy_routines.f90:
// 1266-1297) for the test molecule; returns overlap, sets the combined energy.
bool widom_inter(const orc_ctx* c, int ibox, const TestMol& t, bool cbmc, double& e, double* eabs = nullptr) {
  double ev, eq;
  bool ov = mol_inter_energy(c, ibox, t.view(), -1, cbmc, ev, eq, eabs);
  e = ev + eq;
  return ov;
}

struct InsertionOut {
  double widom_var = 0, ln_pbias = 0, e_inter = 0, first_trial_sum = 0, e_inter_abs = 0;
  int selected = 0, overlap = 0;
};

// One Widom insertion: Build_Molecule (fragment_growth.f90:72-707) with
// Fragment_Placement (:1449-2132), then the body of the insertion loop of
// Widom_Insert (widom_insert.f90:320-488).
InsertionOut widom_one(const orc_ctx* c, int is, int ibox, int kappa_ins, int kappa_dih,
                       double E_inter_constant, Rng& rng) {
  const Species& s = c->sp[is];
  const Box& b = c->box[ibox];
  const double beta = b.beta;
  InsertionOut out;
  TestMol t;
  t.is = is;
  t.r.assign(3 * s.natoms, 0.0);
  t.exist.assign(s.natoms, 0);
  double ln_pbias = 0.0, ln_pseq = 0.0;

  // Step 1: first fragment and growth order (fragment_growth.f90:218-253)
  double u = rng.next();
  int fstart = 0;
  while (fstart < s.nfrag && !(u < s.cum_prob_ins[fstart])) ++fstart;
  if (fstart >= s.nfrag) fstart = s.nfrag - 1;
  ln_pseq = std::log(s.prob_ins[fstart]);
  std::vector<int> order{fstart}, live(s.nfrag, 0);
  live[fstart] = 1;
  if (s.nfrag > 1) fragment_order(s, fstart, order, live, ln_pseq, rng);

  // Step 2: conformation of the first fragment (:274-304)
  const std::vector<int>& fa = s.frag_atoms[fstart];
  int nfa = (int)fa.size();
  int conf = (int)(rng.next() * s.frag_nconfig[fstart]);
  if (conf >= s.frag_nconfig[fstart]) conf = s.frag_nconfig[fstart] - 1;
  for (int i = 0; i < nfa; ++i)
    for (int d = 0; d < 3; ++d) t.r[3 * fa[i] + d] = s.frag_lib[fstart][(size_t)(conf * nfa + i) * 3 + d];
  for (int i = 0; i < nfa; ++i) t.exist[fa[i]] = 1;

  // Step 3: Get_COM + Rotate_Molecule_Eulerian (rotation_routines.f90:41-137)
  get_com(c, is, t.r.data(), t.exist.data(), t.com);
  {
    double theta = std::acos(1.0 - 2.0 * rng.next());
    double phi = (1.0 - 2.0 * rng.next()) * PI;
    double psi = (1.0 - 2.0 * rng.next()) * PI;
    for (int ia = 0; ia < s.natoms; ++ia)
      if (t.exist[ia])
        for (int d = 0; d < 3; ++d) t.r[3 * ia + d] -= t.com[d];
    double r11 = std::cos(psi) * std::cos(phi) - std::cos(theta) * std::sin(phi) * std::sin(psi);
    double r12 = std::cos(psi) * std::sin(phi) + std::cos(theta) * std::cos(phi) * std::sin(psi);
    double r13 = std::sin(psi) * std::sin(theta);
    double r21 = -std::sin(psi) * std::cos(phi) - std::cos(theta) * std::sin(phi) * std::cos(psi);
    double r22 = -std::sin(psi) * std::sin(phi) + std::cos(theta) * std::cos(phi) * std::cos(psi);
    double r23 = std::cos(psi) * std::sin(theta);
    double r31 = std::sin(theta) * std::sin(phi);
    double r32 = -std::sin(theta) * std::cos(phi);
    double r33 = std::cos(theta);
    for (int ia = 0; ia < s.natoms; ++ia) {
      if (!t.exist[ia]) continue;
      double x = t.r[3 * ia], y = t.r[3 * ia + 1], z = t.r[3 * ia + 2];
      double xn = r11 * x + r12 * y + r13 * z;
      double yn = r21 * x + r22 * y + r23 * z;
      double zn = r31 * x + r32 * y + r33 * z;
      t.r[3 * ia] = xn + t.com[0];
      t.r[3 * ia + 1] = yn + t.com[1];
      t.r[3 * ia + 2] = zn + t.com[2];
    }
  }

  // Step 4: kappa_ins trial positions (:383-579)
  std::vector<double> r0(t.r);
  double com_old[3] = {t.com[0], t.com[1], t.com[2]};
  std::vector<double> weight(kappa_ins, 0.0), nrg(kappa_ins, 0.0), anchors(3 * kappa_ins, 0.0);
  std::vector<char> ov_trial(kappa_ins, 0);
  bool need_max_dcom = true;
  for (int it = 0; it < kappa_ins; ++it) {
    double ax = (0.5 - rng.next()) * b.L[0];
    double ay = (0.5 - rng.next()) * b.L[1];
    double az = (0.5 - rng.next()) * b.L[2];
    for (int i = 0; i < nfa; ++i) {
      int a = fa[i];
      t.r[3 * a] = r0[3 * a] - com_old[0] + ax;
      t.r[3 * a + 1] = r0[3 * a + 1] - com_old[1] + ay;
      t.r[3 * a + 2] = r0[3 * a + 2] - com_old[2] + az;
    }
    anchors[3 * it] = ax;
    anchors[3 * it + 1] = ay;
    anchors[3 * it + 2] = az;
    t.com[0] = ax;
    t.com[1] = ay;
    t.com[2] = az;
    if (need_max_dcom) {
      t.max_dcom = max_com_distance(c, is, t.r.data(), t.exist.data(), t.com);
      need_max_dcom = false;
    }
    double e = 0.0;
    bool ov = false;
    if (c->opt.sector_overlap)  // check_overlap of each placed atom (fragment_growth.f90:475-488)
      for (int i = 0; i < nfa && !ov; ++i) ov = check_overlap_atom(c, ibox, is, fa[i], &t.r[3 * fa[i]]);
    if (!ov) ov = widom_inter(c, ibox, t, true, e);
    nrg[it] = nrg[it] + e;
    if (ov) {
      weight[it] = 0.0;
      ov_trial[it] = 1;
    } else {
      double nk = beta * nrg[it];
      if (nk >= MAX_KBT) {
        weight[it] = 0.0;
        ov_trial[it] = 1;
      } else {
        weight[it] = std::exp(-nk);
        out.first_trial_sum += nrg[it];
      }
    }
    if (it > 0) weight[it] = weight[it - 1] + weight[it];
  }
  bool cbmc_overlap = std::all_of(ov_trial.begin(), ov_trial.end(), [](char v) { return v != 0; });
  int sel = -1;
  if (!cbmc_overlap) {
    double rn = rng.next() * weight[kappa_ins - 1];
    int i = 0;
    while (i < kappa_ins && !(rn < weight[i])) ++i;
    if (i == kappa_ins) cbmc_overlap = true;
    else sel = i;
  }
  if (!cbmc_overlap) {
    ln_pbias = ln_pbias - beta * nrg[sel] - std::log(weight[kappa_ins - 1]);
    for (int i = 0; i < nfa; ++i) {
      int a = fa[i];
      t.r[3 * a] = r0[3 * a] - com_old[0] + anchors[3 * sel];
      t.r[3 * a + 1] = r0[3 * a + 1] - com_old[1] + anchors[3 * sel + 1];
      t.r[3 * a + 2] = r0[3 * a + 2] - com_old[2] + anchors[3 * sel + 2];
    }
    t.com[0] = anchors[3 * sel];
    t.com[1] = anchors[3 * sel + 1];
    t.com[2] = anchors[3 * sel + 2];
    out.selected = sel + 1;
  }

  // Step 5: remaining fragments, Fragment_Placement (:1449-2132)
  if (!cbmc_overlap && (int)order.size() > 1) {
    double e_prev = dihedral_energy(s, t.r.data(), t.exist.data());
    std::vector<int> placed(s.nfrag, 0);
    placed[fstart] = 1;
    std::vector<double> cfg(3 * s.natoms, 0.0);
    std::vector<double> ctmp(3 * s.natoms * kappa_dih, 0.0);
    std::vector<double> dw(kappa_dih), dn(kappa_dih), dd(kappa_dih);
    std::vector<char> dov(kappa_dih);
    for (size_t oi = 1; oi < order.size() && !cbmc_overlap; ++oi) {
      int f = order[oi];
      const std::vector<int>& atoms = s.frag_atoms[f];
      int nf = (int)atoms.size();
      std::vector<char> grown(t.exist);
      int nconf = s.frag_nconfig[f];
      int cf = (int)(rng.next() * nconf);
      cf = (int)(rng.next() * nconf);  // the duplicated draw of fragment_growth.f90:1578,1584
      if (cf >= nconf) cf = nconf - 1;
      for (int j = 0; j < nf; ++j) {
        int a = atoms[j];
        t.exist[a] = 1;
        for (int d = 0; d < 3; ++d) cfg[3 * a + d] = s.frag_lib[f][(size_t)(cf * nf + j) * 3 + d];
      }
      std::vector<char> combined(t.exist), newex(s.natoms);
      for (int a = 0; a < s.natoms; ++a) newex[a] = combined[a] && !grown[a];
      int fc = -1;
      for (int g : s.frag_connect[f])
        if (placed[g]) { fc = g; break; }
      if (fc < 0) {  // no placed neighbour: the fragment graph is not connected
        cbmc_overlap = true;
        break;
      }
      int anc_i = atoms[0];
      int anc_c = s.frag_atoms[fc][0];
      std::vector<int> atom_id;
      for (int a : atoms)
        if (a != anc_i && a != anc_c) atom_id.push_back(a);
      int atom_ifrag = atoms[nf - 1];
      for (int a : atoms)
        if (a != anc_i && a != anc_c) { atom_ifrag = a; break; }
      int atom_fc = s.frag_atoms[fc].back();
      for (int a : s.frag_atoms[fc])
        if (a != anc_i && a != anc_c) { atom_fc = a; break; }
      double v1[3], v2[3], al_i[9], hg_i[9], al_c[9], hg_c[9];
      for (int d = 0; d < 3; ++d) {
        v1[d] = cfg[3 * anc_i + d] - cfg[3 * anc_c + d];
        v2[d] = cfg[3 * atom_ifrag + d] - cfg[3 * anc_c + d];
      }
      aligner_hanger(v1, v2, al_i, hg_i);
      for (int d = 0; d < 3; ++d) {
        v1[d] = t.r[3 * anc_i + d] - t.r[3 * anc_c + d];
        v2[d] = t.r[3 * atom_fc + d] - t.r[3 * anc_c + d];
      }
      aligner_hanger(v1, v2, al_c, hg_c);
      double tx = cfg[3 * anc_c], ty = cfg[3 * anc_c + 1], tz = cfg[3 * anc_c + 2];
      for (int a = 0; a < s.natoms; ++a) {
        cfg[3 * a] -= tx;
        cfg[3 * a + 1] -= ty;
        cfg[3 * a + 2] -= tz;
      }
      for (int a : atoms) {
        double x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
        cfg[3 * a] = x * al_i[0] + y * al_i[1] + z * al_i[2];
        cfg[3 * a + 1] = x * al_i[3] + y * al_i[4] + z * al_i[5];
        cfg[3 * a + 2] = x * al_i[6] + y * al_i[7] + z * al_i[8];
      }
      double theta = TWOPI * rng.next();
      for (int ii = 0; ii < kappa_dih; ++ii) {
        double* ct = &ctmp[(size_t)ii * 3 * s.natoms];
        double cth = std::cos(theta), sth = std::sin(theta);
        for (int a : atoms) {
          double x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
          double yr = cth * y + sth * z, zr = -sth * y + cth * z;
          double xn = x * hg_c[0] + yr * hg_c[1] + zr * hg_c[2];
          double yn = x * hg_c[3] + yr * hg_c[4] + zr * hg_c[5];
          double zn = x * hg_c[6] + yr * hg_c[7] + zr * hg_c[8];
          if (a != anc_i && a != anc_c) {
            xn = xn + t.r[3 * anc_c];
            yn = yn + t.r[3 * anc_c + 1];
            zn = zn + t.r[3 * anc_c + 2];
          }
          ct[3 * a] = xn;
          ct[3 * a + 1] = yn;
          ct[3 * a + 2] = zn;
        }
        theta = theta + TWOPI / (double)kappa_dih;
      }
      // Step 4 of Fragment_Placement: trial energies (:1926-2058)
      for (int ii = 0; ii < kappa_dih; ++ii) {
        dn[ii] = 0.0;
        dd[ii] = 0.0;
        dov[ii] = 0;
        const double* ct = &ctmp[(size_t)ii * 3 * s.natoms];
        for (int a : atom_id)
          for (int d = 0; d < 3; ++d) t.r[3 * a + d] = ct[3 * a + d];
        if (c->opt.sector_overlap) {  // check_overlap of the fragment's atoms (fragment_growth.f90:1930-1949)
          bool sov = false;
          for (int a : atom_id)
            if (!sov) sov = check_overlap_atom(c, ibox, is, a, &t.r[3 * a]);
          if (sov) {
            dw[ii] = ii > 0 ? dw[ii - 1] : 0.0;
            dov[ii] = 1;
            continue;
          }
        }
        for (int a : atom_id) t.exist[a] = 0;
        double niv = 0, niq = 0, noq = 0;
        bool ov = false;
        for (int a : atom_id) {
          t.exist[a] = 1;
          double eiv, eiq, eoq;
          if (atom_intra_energy(c, b, is, a, t.r.data(), t.exist.data(), true, eiv, eiq, eoq)) {
            ov = true;
            break;
          }
          niv += eiv;
          niq += eiq;
          noq += eoq;
        }
        if (ov) {
          dw[ii] = ii > 0 ? dw[ii - 1] : 0.0;
          dov[ii] = 1;
          for (int a : atom_id) t.exist[a] = 1;
          continue;
        }
        t.exist = newex;
        get_com(c, is, t.r.data(), t.exist.data(), t.com);
        t.max_dcom = max_com_distance(c, is, t.r.data(), t.exist.data(), t.com);
        double einter = 0.0;
        ov = widom_inter(c, ibox, t, true, einter);
        t.exist = combined;
        if (ov) {
          dw[ii] = 0.0;
          dov[ii] = 1;
        } else {
          double ed = dihedral_energy(s, t.r.data(), t.exist.data());
          dd[ii] = ed;
          dn[ii] = ed + niv + niq + einter + noq - e_prev;
          double nk = beta * dn[ii];
          if (nk >= MAX_KBT) {
            dw[ii] = 0.0;
            dov[ii] = 1;
          } else {
            dw[ii] = std::exp(-nk);
          }
        }
        if (ii > 0) dw[ii] = dw[ii - 1] + dw[ii];
      }
      if (std::all_of(dov.begin(), dov.end(), [](char v) { return v != 0; })) {
        cbmc_overlap = true;
        break;
      }
      double pp = rng.next() * dw[kappa_dih - 1];
      int tr = 0;
      while (tr < kappa_dih && !(pp < dw[tr])) ++tr;
      if (tr == kappa_dih) {
        cbmc_overlap = true;
        break;
      }
      ln_pbias = ln_pbias - beta * dn[tr] - std::log(dw[kappa_dih - 1]);
      const double* ct = &ctmp[(size_t)tr * 3 * s.natoms];
      for (int a : atoms)
        if (a != anc_i && a != anc_c)
          for (int d = 0; d < 3; ++d) t.r[3 * a + d] = ct[3 * a + d];
      e_prev = dd[tr];
      placed[f] = 1;
    }
    if (!cbmc_overlap) {
      get_com(c, is, t.r.data(), t.exist.data(), t.com);
      t.max_dcom = max_com_distance(c, is, t.r.data(), t.exist.data(), t.com);
    }
  }

  // widom_insert.f90:350-447
  ln_pbias = ln_pbias + ln_pseq;
  ln_pbias = ln_pbias + std::log((double)kappa_ins);
  if (kappa_dih != 0) ln_pbias = ln_pbias + (double)(s.nfrag - 1) * std::log((double)kappa_dih);
  out.ln_pbias = ln_pbias;
  if (cbmc_overlap) {
    out.overlap = 1;
    return out;
  }
  for (int a = 0; a < s.natoms; ++a) t.exist[a] = 1;
  if (s.nfrag > 1) {
    // Fold_Molecule, cubic branch (minimum_image_separation.f90:180-216)
    for (int d = 0; d < 3; ++d) {
      if (t.com[d] > b.hL[d]) {
        t.com[d] = t.com[d] - b.L[d];
        for (int a = 0; a < s.natoms; ++a) t.r[3 * a + d] -= b.L[d];
      } else if (t.com[d] < -b.hL[d]) {
        t.com[d] = t.com[d] + b.L[d];
        for (int a = 0; a < s.natoms; ++a) t.r[3 * a + d] += b.L[d];
      }
    }
  }
  double e_inter = 0.0;
  if (widom_inter(c, ibox, t, false, e_inter, &out.e_inter_abs)) {
    out.overlap = 2;
    return out;
  }
  double eiv, eiq, eoq;
  if (mol_intra_energy(c, b, is, t.r.data(), t.exist.data(), false, eiv, eiq, eoq)) {
    out.overlap = 3;
    return out;
  }
  e_inter = e_inter + eoq;
  double dE_inter = e_inter + E_inter_constant;
  double dE_intra = eiv + eiq;
  double E_bond = bond_energy(s, t.r.data());
  double E_angle = angle_energy(s, t.r.data(), t.exist.data());
  double E_dih = dihedral_energy(s, t.r.data(), t.exist.data());
  double E_imp = improper_energy(s, t.r.data());
  dE_intra = dE_intra + E_bond + E_angle + E_dih + E_imp;
  if (box_has_ewald(b) && s.has_charge) {
    // Update_System_Ewald_Reciprocal_Energy_Widom (energy_routines.f90:2500-2550)
    double E = 0.0;
    for (size_t i = 0; i < b.hx.size(); ++i) {
      double cs = b.cos_sum[i], sn = b.sin_sum[i];
      double dc = 0, ds = 0;
      for (int ia = 0; ia < s.natoms; ++ia) {
        double hdotr = b.hx[i] * t.r[3 * ia] + b.hy[i] * t.r[3 * ia + 1] + b.hz[i] * t.r[3 * ia + 2];
        dc += s.q[ia] * std::cos(hdotr);
        ds += s.q[ia] * std::sin(hdotr);
      }
      cs = cs + dc;
      sn = sn + ds;
      E = E + b.Cn[i] * (cs * cs + sn * sn);
    }
    dE_inter = dE_inter + E * CHARGE_FACTOR;
  }
  double dE = dE_intra + dE_inter;
  double dE_frag = E_angle;
  out.e_inter = dE_inter - E_inter_constant;
  out.widom_var = std::exp(-beta * (dE - dE_frag) - ln_pbias);
  return out;
}

int check_ctx(orc_ctx* c) { return c ? CASS_OK : fail(CASS_EINVAL, "NULL context"); }

int check_mol(orc_ctx* c, int im, int is) {
  if (is < 1 || is > c->nspecies) return fail(CASS_EINVAL, "species index out of range");
  if (im < 1 || im > c->max_mol[is - 1]) return fail(CASS_EINVAL, "molecule locate out of range");
  if (!c->sp[is - 1].defined) return fail(CASS_ESTATE, "species not defined");
  return CASS_OK;
}

void invalidate_box(orc_ctx* c, int ibox) {
  if (ibox >= 0 && ibox < c->nboxes) c->box[ibox].energy_valid = false;
}

// ---------------------------------------------------------------------------
// NVT Monte Carlo moves (move_translate.f90, move_rotate.f90,
// accept_or_reject.f90), one chain per box.

// accept_or_reject (accept_or_reject.f90:22-65)
bool accept_or_reject(double ln_pacc, Rng& rng) {
  if (ln_pacc <= 0.0) return true;
  if (ln_pacc < MAX_KBT) return rng.next() <= std::exp(-ln_pacc);
  return false;
}

// species_list%linear (input_routines.f90:1955-1967): every angle fixed at 180 degrees
bool species_linear(const Species& s) {
  for (size_t k = 0; k < s.angle_kind.size(); ++k)
    if (s.angle_kind[k] != CASS_BONDED_FIXED || s.angle_param[2 * k] != 180.0) return false;
  return true;
}

// Update_System_Ewald_Reciprocal_Energy for a translated / rotated molecule
// (energy_routines.f90:2384-2431); keeps the old sums for ewald_revert
double ewald_move(const orc_ctx* c, Box& b, Mol& m) {
  const size_t nv = b.hx.size();
  b.cos_sum_old = b.cos_sum;
  b.sin_sum_old = b.sin_sum;
  if (m.cos_mol.size() != nv) {
    m.cos_mol.assign(nv, 0.0);
    m.sin_mol.assign(nv, 0.0);
  }
  m.cos_mol_old = m.cos_mol;
  m.sin_mol_old = m.sin_mol;
  std::vector<double> cn(nv), sn(nv);
  mol_structure_factor(c, b, m.is, m.r.data(), cn.data(), sn.data());
  double E = 0.0;
  for (size_t i = 0; i < nv; ++i) {
    b.cos_sum[i] = b.cos_sum[i] + (cn[i] - m.cos_mol[i]);
    b.sin_sum[i] = b.sin_sum[i] + (sn[i] - m.sin_mol[i]);
    E = E + b.Cn[i] * (b.cos_sum[i] * b.cos_sum[i] + b.sin_sum[i] * b.sin_sum[i]);
    m.cos_mol[i] = cn[i];
    m.sin_mol[i] = sn[i];
  }
  return E * CHARGE_FACTOR;
}

void ewald_revert(Box& b, Mol& m) {
  b.cos_sum = b.cos_sum_old;
  b.sin_sum = b.sin_sum_old;
  m.cos_mol = m.cos_mol_old;
  m.sin_mol = m.sin_mol_old;
}

struct McChain {
  orc_ctx* c;
  int ibox;
  const CassMCParams* p;
  double* max_disp;  // [nspecies] of this box
  double* max_rot;
  Rng rng;
  CassEnergy E;
  CassMCResult res{};
  std::vector<int64_t> nt_disp, ns_disp, nt_rot, ns_rot;  // trials, successes since the last update
  int err = CASS_OK;

  int nmols(int is) const { return c->sp_off[ibox][is + 1] - c->sp_off[ibox][is]; }

  // species choice of Translate / Rotate (move_translate.f90:150-170): only
  // species with a nonzero step take part; -1 when none does
  int pick_species(const double* step) {
    int ntot = 0;
    for (int is = 0; is < c->nspecies; ++is)
      if (step[is] > 0.0) ntot += nmols(is);
    if (ntot == 0) return -1;
    double x = 0.0;
    std::vector<double> xs(c->nspecies);
    for (int is = 0; is < c->nspecies; ++is) {
      xs[is] = (step[is] > 0.0 ? (double)nmols(is) / (double)ntot : 0.0) + (is > 0 ? x : 0.0);
      x = xs[is];
    }
    const double u = rng.next();
    int is = 0;
    while (is < c->nspecies && !(u <= xs[is])) ++is;
    if (is == c->nspecies)  // rounding left u above the last sum
      for (is = c->nspecies - 1; is > 0 && !(step[is] > 0.0 && nmols(is) > 0); --is) {
      }
    return is;
  }

  Mol& pick_molecule(int is) {
    const int im = std::min((int)(rng.next() * nmols(is)) + 1, nmols(is));  // rranf() may round to 1.0
    return c->mol[c->members[ibox][c->sp_off[ibox][is] + im - 1]];
  }

  // the energy of m against the rest of the box; false sets err on an
  // overlapping starting configuration (Clean_Abort in the reference)
  bool old_energy(const Mol& m, int slot, double& ev, double& eq) {
    if (mol_inter_energy(c, ibox, view_of(m), slot, false, ev, eq)) {
      err = fail(CASS_ESTATE, "molecule energy too high before the move");
      return false;
    }
    return true;
  }

  // energies after the trial position, the Ewald difference and the
  // Metropolis test; reverts on rejection.  Returns acceptance.
  bool finish_move(Mol& m, int slot, double ev_old, double eq_old, const std::vector<double>& r_old,
                   const double* com_old) {
    Box& b = c->box[ibox];
    double ev, eq;
    if (mol_inter_energy(c, ibox, view_of(m), slot, false, ev, eq)) {
      m.r = r_old;
      std::copy(com_old, com_old + 3, m.com);
      ++res.n_overlap;
      return false;
    }
    const bool ew = box_has_ewald(b) && c->sp[m.is].has_charge;
    double dE = 0.0, E_recip = 0.0;
    if (ew) {
      E_recip = ewald_move(c, b, m);
      dE = E_recip - E.reciprocal;
    }
    dE = dE + (ev - ev_old) + (eq - eq_old);
    const bool acc = accept_or_reject(b.beta * dE, rng);
    if (acc) {
      E.total = E.total + dE;
      E.inter = E.inter + dE;
      E.inter_vdw = E.inter_vdw + ev - ev_old;
      E.inter_q = E.inter_q + eq - eq_old;
      if (ew) E.reciprocal = E_recip;
    } else {
      m.r = r_old;
      std::copy(com_old, com_old + 3, m.com);
      if (ew) ewald_revert(b, m);
    }
    return acc;
  }

  // Translate (move_translate.f90:22-355)
  void translate() {
    const int is = pick_species(max_disp);
    if (is < 0) return;
    Mol& m = pick_molecule(is);
    const int slot = (int)(&m - c->mol.data());
    ++res.n_translate;
    ++nt_disp[is];
    double ev_old, eq_old;
    if (!old_energy(m, slot, ev_old, eq_old)) return;
    const std::vector<double> r_old = m.r;
    const double com_old[3] = {m.com[0], m.com[1], m.com[2]};
    const Species& s = c->sp[is];
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = (2.0 * rng.next() - 1.0) * max_disp[is];
    for (int a = 0; a < s.natoms; ++a)
      for (int k = 0; k < 3; ++k) m.r[3 * a + k] = m.r[3 * a + k] + d[k];
    for (int k = 0; k < 3; ++k) m.com[k] = m.com[k] + d[k];
    // Fold_Molecule, orthorhombic branch (minimum_image_separation.f90:162-235)
    const Box& b = c->box[ibox];
    for (int k = 0; k < 3; ++k) {
      double sh = 0.0;
      if (m.com[k] > b.hL[k]) sh = -b.L[k];
      else if (m.com[k] < -b.hL[k]) sh = b.L[k];
      if (sh != 0.0) {
        m.com[k] = m.com[k] + sh;
        for (int a = 0; a < s.natoms; ++a) m.r[3 * a + k] = m.r[3 * a + k] + sh;
      }
    }
    if (finish_move(m, slot, ev_old, eq_old, r_old, com_old)) {
      ++res.n_translate_accepted;
      ++ns_disp[is];
    }
    if (p->nupdate > 0 && nt_disp[is] % p->nupdate == 0) {  // :330-352, equilibration rule
      const double ratio = (double)ns_disp[is] / (double)p->nupdate;
      ns_disp[is] = 0;
      if (ratio < 0.00005) {
        max_disp[is] = 0.1 * max_disp[is];
      } else {
        double rsmall = b.rcut_vdw;
        if (s.has_charge && b.charge_style != CASS_CHARGE_NONE) rsmall = std::min(b.rcut_vdw, b.rcut_coul);
        max_disp[is] = std::min(rsmall, ratio / p->target_accept * max_disp[is]);
      }
    }
  }

  // Rotate (move_rotate.f90:22-536)
  void rotate() {
    const int is = pick_species(max_rot);
    if (is < 0) return;
    Mol& m = pick_molecule(is);
    const int slot = (int)(&m - c->mol.data());
    ++res.n_rotate;
    ++nt_rot[is];
    double ev_old, eq_old;
    if (!old_energy(m, slot, ev_old, eq_old)) return;
    const std::vector<double> r_old = m.r;
    const double com_old[3] = {m.com[0], m.com[1], m.com[2]};
    const Species& s = c->sp[is];
    double R[9];
    if (species_linear(s)) {  // Rotate_Molecule_Eulerian (:466-536)
      const double theta = std::acos(1.0 - 2.0 * rng.next());
      const double phi = (1.0 - 2.0 * rng.next()) * PI;
      const double psi = (1.0 - 2.0 * rng.next()) * PI;
      R[0] = std::cos(psi) * std::cos(phi) - std::cos(theta) * std::sin(phi) * std::sin(psi);
      R[1] = std::cos(psi) * std::sin(phi) + std::cos(theta) * std::cos(phi) * std::sin(psi);
      R[2] = std::sin(psi) * std::sin(theta);
      R[3] = -std::sin(psi) * std::cos(phi) - std::cos(theta) * std::sin(phi) * std::cos(psi);
      R[4] = -std::sin(psi) * std::sin(phi) + std::cos(theta) * std::cos(phi) * std::cos(psi);
      R[5] = std::cos(psi) * std::sin(theta);
      R[6] = std::sin(theta) * std::sin(phi);
      R[7] = -std::sin(theta) * std::cos(phi);
      R[8] = std::cos(theta);
    } else {  // Rotate_Molecule_Axis (:362-463)
      double psi1 = 0.0, psi2 = 0.0, psi3 = 0.0;
      const int axis = (int)(3.0 * rng.next()) + 1;
      const double ang = (2.0 * rng.next() - 1.0) * max_rot[is];
      if (axis == 1) psi1 = ang;
      else if (axis == 2) psi2 = ang;
      else psi3 = ang;
      const double c1 = std::cos(psi1), c2 = std::cos(psi2), c3 = std::cos(psi3);
      const double s1 = std::sin(psi1), s2 = std::sin(psi2), s3 = std::sin(psi3);
      R[0] = c1 * c3 - s1 * c2 * s3;
      R[1] = s1 * c3 + c1 * c2 * s3;
      R[2] = s2 * s3;
      R[3] = -c1 * s3 - s1 * c2 * c3;
      R[4] = -s1 * s3 + c1 * c2 * c3;
      R[5] = s2 * c3;
      R[6] = s1 * s2;
      R[7] = -c1 * s2;
      R[8] = c2;
    }
    for (int a = 0; a < s.natoms; ++a) {
      const double x = m.r[3 * a] - m.com[0], y = m.r[3 * a + 1] - m.com[1], z = m.r[3 * a + 2] - m.com[2];
      m.r[3 * a] = (R[0] * x + R[1] * y + R[2] * z) + m.com[0];
      m.r[3 * a + 1] = (R[3] * x + R[4] * y + R[5] * z) + m.com[1];
      m.r[3 * a + 2] = (R[6] * x + R[7] * y + R[8] * z) + m.com[2];
    }
    if (finish_move(m, slot, ev_old, eq_old, r_old, com_old)) {
      get_com(c, is, m.r.data(), m.exist.data(), m.com);  // Get_COM on acceptance
      ++res.n_rotate_accepted;
      ++ns_rot[is];
    }
    if (p->nupdate > 0 && nt_rot[is] % p->nupdate == 0) {  // :307-326, equilibration rule
      const double ratio = (double)ns_rot[is] / (double)p->nupdate;
      ns_rot[is] = 0;
      if (ratio < 0.5) max_rot[is] = std::max(0.01, 0.95 * max_rot[is]);
      else max_rot[is] = std::min(PI, 1.05 * max_rot[is]);
    }
  }

  void run() {
    int nmol = 0;
    for (int is = 0; is < c->nspecies; ++is) nmol += nmols(is);
    const int64_t steps = p->nsweeps * (int64_t)(p->steps_per_sweep > 0 ? p->steps_per_sweep : nmol);
    for (int64_t k = 0; k < steps && err == CASS_OK; ++k) {
      if (rng.next() <= p->prob_translate) translate();  // nvtmc_driver.f90:107-134
      else rotate();
    }
    res.energy = E;
  }
};

// ---------------------------------------------------------------------------
// Grand-canonical moves: Insertion (move_insert.f90), Deletion
// (move_delete.f90) and Cut_N_Grow (move_regrow.f90), with Build_Molecule,
// Fragment_Placement and Cut_Regrow (fragment_growth.f90) for a molecule of
// the box.  del = true computes the Rosenbluth weight of the molecule as it is
// (trial 1 is its present configuration and is always the one chosen).

// Fold_Molecule, orthorhombic branch (minimum_image_separation.f90:162-235)
void fold_molecule(const Box& b, Mol& m) {
  const int n = (int)m.exist.size();
  for (int k = 0; k < 3; ++k) {
    if (m.com[k] > b.hL[k]) {
      m.com[k] = m.com[k] - b.L[k];
      for (int a = 0; a < n; ++a) m.r[3 * a + k] = m.r[3 * a + k] - b.L[k];
    } else if (m.com[k] < -b.hL[k]) {
      m.com[k] = m.com[k] + b.L[k];
      for (int a = 0; a < n; ++a) m.r[3 * a + k] = m.r[3 * a + k] + b.L[k];
    }
  }
}

// Fragment_Placement (fragment_growth.f90:1449-2132) for the fragments
// order[first..]; placed[] marks the fragments already in place.  Returns
// cbmc_overlap.
bool place_fragments(orc_ctx* c, int ibox, Mol& m, int slot, const std::vector<int>& order, size_t first,
                     std::vector<int>& placed, bool del, int kappa_dih, double e_prev, double& ln_pbias, Rng& rng) {
  const Species& s = c->sp[m.is];
  const Box& b = c->box[ibox];
  const double beta = b.beta;
  const int n = s.natoms;
  std::vector<double> cfg(3 * n, 0.0), ctmp(3 * (size_t)n * kappa_dih, 0.0);
  std::vector<double> dw(kappa_dih), dn(kappa_dih), dd(kappa_dih);
  std::vector<char> dov(kappa_dih);
  for (size_t oi = first; oi < order.size(); ++oi) {
    const int f = order[oi];
    const std::vector<int>& atoms = s.frag_atoms[f];
    const int nf = (int)atoms.size();
    std::vector<char> grown(m.exist);
    std::fill(cfg.begin(), cfg.end(), 0.0);
    if (del) {
      for (int a : atoms) {
        m.exist[a] = 1;
        for (int d = 0; d < 3; ++d) cfg[3 * a + d] = m.r[3 * a + d];
      }
    } else {
      const int nconf = s.frag_nconfig[f];
      int cf = (int)(rng.next() * nconf);
      cf = (int)(rng.next() * nconf);  // the duplicated draw of fragment_growth.f90:1578,1584
      if (cf >= nconf) cf = nconf - 1;
      for (int j = 0; j < nf; ++j) {
        const int a = atoms[j];
        m.exist[a] = 1;
        for (int d = 0; d < 3; ++d) cfg[3 * a + d] = s.frag_lib[f][(size_t)(cf * nf + j) * 3 + d];
      }
    }
    const std::vector<char> combined(m.exist);
    std::vector<char> newex(n);
    for (int a = 0; a < n; ++a) newex[a] = combined[a] && !grown[a];
    int fc = -1;
    for (int g : s.frag_connect[f])
      if (placed[g]) {
        fc = g;
        break;
      }
    if (fc < 0) return true;
    const int anc_i = atoms[0], anc_c = s.frag_atoms[fc][0];
    std::vector<int> atom_id;
    for (int a : atoms)
      if (a != anc_i && a != anc_c) atom_id.push_back(a);
    int atom_ifrag = atoms[nf - 1];
    for (int a : atoms)
      if (a != anc_i && a != anc_c) {
        atom_ifrag = a;
        break;
      }
    int atom_fc = s.frag_atoms[fc].back();
    for (int a : s.frag_atoms[fc])
      if (a != anc_i && a != anc_c) {
        atom_fc = a;
        break;
      }
    double v1[3], v2[3], al_i[9], hg_i[9], al_c[9], hg_c[9];
    for (int d = 0; d < 3; ++d) {
      v1[d] = cfg[3 * anc_i + d] - cfg[3 * anc_c + d];
      v2[d] = cfg[3 * atom_ifrag + d] - cfg[3 * anc_c + d];
    }
    aligner_hanger(v1, v2, al_i, hg_i);
    if (!del) {
      for (int d = 0; d < 3; ++d) {
        v1[d] = m.r[3 * anc_i + d] - m.r[3 * anc_c + d];
        v2[d] = m.r[3 * atom_fc + d] - m.r[3 * anc_c + d];
      }
      aligner_hanger(v1, v2, al_c, hg_c);
    }
    const double tx = cfg[3 * anc_c], ty = cfg[3 * anc_c + 1], tz = cfg[3 * anc_c + 2];
    for (int a = 0; a < n; ++a) {
      cfg[3 * a] -= tx;
      cfg[3 * a + 1] -= ty;
      cfg[3 * a + 2] -= tz;
    }
    for (int a : atoms) {
      const double x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
      cfg[3 * a] = x * al_i[0] + y * al_i[1] + z * al_i[2];
      cfg[3 * a + 1] = x * al_i[3] + y * al_i[4] + z * al_i[5];
      cfg[3 * a + 2] = x * al_i[6] + y * al_i[7] + z * al_i[8];
    }
    double theta;
    if (del) {
      theta = 0.0;
      std::copy(hg_i, hg_i + 9, hg_c);
    } else {
      theta = TWOPI * rng.next();
    }
    for (int ii = 0; ii < kappa_dih; ++ii) {
      double* ct = &ctmp[(size_t)ii * 3 * n];
      const double cth = std::cos(theta), sth = std::sin(theta);
      for (int a : atoms) {
        const double x = cfg[3 * a], y = cfg[3 * a + 1], z = cfg[3 * a + 2];
        const double yr = cth * y + sth * z, zr = -sth * y + cth * z;
        double xn = x * hg_c[0] + yr * hg_c[1] + zr * hg_c[2];
        double yn = x * hg_c[3] + yr * hg_c[4] + zr * hg_c[5];
        double zn = x * hg_c[6] + yr * hg_c[7] + zr * hg_c[8];
        if (a != anc_i && a != anc_c) {
          xn = xn + m.r[3 * anc_c];
          yn = yn + m.r[3 * anc_c + 1];
          zn = zn + m.r[3 * anc_c + 2];
        }
        ct[3 * a] = xn;
        ct[3 * a + 1] = yn;
        ct[3 * a + 2] = zn;
      }
      theta = theta + TWOPI / (double)kappa_dih;
    }
    for (int ii = 0; ii < kappa_dih; ++ii) {
      dn[ii] = 0.0;
      dd[ii] = 0.0;
      dov[ii] = 0;
      const double* ct = &ctmp[(size_t)ii * 3 * n];
      for (int a : atom_id)
        for (int d = 0; d < 3; ++d) m.r[3 * a + d] = ct[3 * a + d];
      for (int a : atom_id) m.exist[a] = 0;
      double niv = 0, niq = 0, noq = 0;
      bool ov = false;
      for (int a : atom_id) {
        m.exist[a] = 1;
        double eiv, eiq, eoq;
        if (atom_intra_energy(c, b, m.is, a, m.r.data(), m.exist.data(), true, eiv, eiq, eoq)) {
          ov = true;
          break;
        }
        niv += eiv;
        niq += eiq;
        noq += eoq;
      }
      if (ov) {
        dw[ii] = ii > 0 ? dw[ii - 1] : 0.0;
        dov[ii] = 1;
        for (int a : atom_id) m.exist[a] = 1;
        continue;
      }
      m.exist = newex;
      get_com(c, m.is, m.r.data(), m.exist.data(), m.com);
      m.max_dcom = max_com_distance(c, m.is, m.r.data(), m.exist.data(), m.com);
      double ev = 0.0, eq = 0.0;
      ov = mol_inter_energy(c, ibox, view_of(m), slot, true, ev, eq);
      m.exist = combined;
      if (ov) {
        dw[ii] = 0.0;
        dov[ii] = 1;
      } else {
        const double ed = dihedral_energy(s, m.r.data(), m.exist.data());
        dd[ii] = ed;
        dn[ii] = ed + niv + niq + (ev + eq) + noq - e_prev;
        const double nk = beta * dn[ii];
        if (nk >= MAX_KBT) {
          dw[ii] = 0.0;
          dov[ii] = 1;
        } else {
          dw[ii] = std::exp(-nk);
        }
      }
      if (ii > 0) dw[ii] = dw[ii - 1] + dw[ii];
    }
    if (std::all_of(dov.begin(), dov.end(), [](char v) { return v != 0; })) return true;
    int tr = 0;
    if (!del) {
      const double pp = rng.next() * dw[kappa_dih - 1];
      while (tr < kappa_dih && !(pp < dw[tr])) ++tr;
      if (tr == kappa_dih) return true;
    }
    ln_pbias = ln_pbias - beta * dn[tr] - std::log(dw[kappa_dih - 1]);
    const double* ct = &ctmp[(size_t)tr * 3 * n];
    for (int a : atoms)
      if (a != anc_i && a != anc_c)
        for (int d = 0; d < 3; ++d) m.r[3 * a + d] = ct[3 * a + d];
    e_prev = dd[tr];
    placed[f] = 1;
  }
  return false;
}

// Build_Molecule (fragment_growth.f90:72-707) for molecule m (slot) of box
// ibox.  Returns cbmc_overlap; sets ln_pseq and ln_pbias.
bool build_molecule(orc_ctx* c, int ibox, Mol& m, int slot, bool del, int kappa_ins, int kappa_dih, double& ln_pseq,
                    double& ln_pbias, Rng& rng, std::vector<int>* order_out = nullptr) {
  const Species& s = c->sp[m.is];
  const Box& b = c->box[ibox];
  const double beta = b.beta;
  ln_pbias = 0.0;
  std::fill(m.exist.begin(), m.exist.end(), 0);
  const double u = rng.next();
  int fstart = 0;
  while (fstart < s.nfrag && !(u < s.cum_prob_ins[fstart])) ++fstart;
  if (fstart >= s.nfrag) fstart = s.nfrag - 1;
  ln_pseq = std::log(s.prob_ins[fstart]);
  std::vector<int> order{fstart}, live(s.nfrag, 0);
  live[fstart] = 1;
  if (s.nfrag > 1) fragment_order(s, fstart, order, live, ln_pseq, rng);
  if (order_out) *order_out = order;
  const std::vector<int>& fa = s.frag_atoms[fstart];
  const int nfa = (int)fa.size();
  if (!del) {
    int conf = (int)(rng.next() * s.frag_nconfig[fstart]);
    if (conf >= s.frag_nconfig[fstart]) conf = s.frag_nconfig[fstart] - 1;
    for (int i = 0; i < nfa; ++i)
      for (int d = 0; d < 3; ++d) m.r[3 * fa[i] + d] = s.frag_lib[fstart][(size_t)(conf * nfa + i) * 3 + d];
  }
  for (int a : fa) m.exist[a] = 1;
  get_com(c, m.is, m.r.data(), m.exist.data(), m.com);
  if (!del) {  // Rotate_Molecule_Eulerian (rotation_routines.f90:41-137)
    const double theta = std::acos(1.0 - 2.0 * rng.next());
    const double phi = (1.0 - 2.0 * rng.next()) * PI;
    const double psi = (1.0 - 2.0 * rng.next()) * PI;
    const double r11 = std::cos(psi) * std::cos(phi) - std::cos(theta) * std::sin(phi) * std::sin(psi);
    const double r12 = std::cos(psi) * std::sin(phi) + std::cos(theta) * std::cos(phi) * std::sin(psi);
    const double r13 = std::sin(psi) * std::sin(theta);
    const double r21 = -std::sin(psi) * std::cos(phi) - std::cos(theta) * std::sin(phi) * std::cos(psi);
    const double r22 = -std::sin(psi) * std::sin(phi) + std::cos(theta) * std::cos(phi) * std::cos(psi);
    const double r23 = std::cos(psi) * std::sin(theta);
    const double r31 = std::sin(theta) * std::sin(phi);
    const double r32 = -std::sin(theta) * std::cos(phi);
    const double r33 = std::cos(theta);
    for (int a : fa) {
      const double x = m.r[3 * a] - m.com[0], y = m.r[3 * a + 1] - m.com[1], z = m.r[3 * a + 2] - m.com[2];
      m.r[3 * a] = (r11 * x + r12 * y + r13 * z) + m.com[0];
      m.r[3 * a + 1] = (r21 * x + r22 * y + r23 * z) + m.com[1];
      m.r[3 * a + 2] = (r31 * x + r32 * y + r33 * z) + m.com[2];
    }
  }
  const std::vector<double> r0(m.r);
  const double com_old[3] = {m.com[0], m.com[1], m.com[2]};
  std::vector<double> weight(kappa_ins, 0.0), nrg(kappa_ins, 0.0), anchors(3 * kappa_ins, 0.0);
  std::vector<char> ov_trial(kappa_ins, 0);
  bool need_max_dcom = true;
  for (int it = 0; it < kappa_ins; ++it) {
    double ax, ay, az;
    if (del && it == 0) {
      ax = com_old[0];
      ay = com_old[1];
      az = com_old[2];
    } else {
      ax = (0.5 - rng.next()) * b.L[0];
      ay = (0.5 - rng.next()) * b.L[1];
      az = (0.5 - rng.next()) * b.L[2];
    }
    for (int a : fa) {
      m.r[3 * a] = r0[3 * a] - com_old[0] + ax;
      m.r[3 * a + 1] = r0[3 * a + 1] - com_old[1] + ay;
      m.r[3 * a + 2] = r0[3 * a + 2] - com_old[2] + az;
    }
    anchors[3 * it] = ax;
    anchors[3 * it + 1] = ay;
    anchors[3 * it + 2] = az;
    m.com[0] = ax;
    m.com[1] = ay;
    m.com[2] = az;
    if (need_max_dcom) {
      m.max_dcom = max_com_distance(c, m.is, m.r.data(), m.exist.data(), m.com);
      need_max_dcom = false;
    }
    double ev = 0.0, eq = 0.0;
    const bool ov = mol_inter_energy(c, ibox, view_of(m), slot, true, ev, eq);
    nrg[it] = ev + eq;
    if (ov) {
      weight[it] = 0.0;
      ov_trial[it] = 1;
    } else {
      const double nk = beta * nrg[it];
      if (nk >= MAX_KBT) {
        weight[it] = 0.0;
        ov_trial[it] = 1;
      } else {
        weight[it] = std::exp(-nk);
      }
    }
    if (it > 0) weight[it] = weight[it - 1] + weight[it];
  }
  if (std::all_of(ov_trial.begin(), ov_trial.end(), [](char v) { return v != 0; })) return true;
  int sel = 0;
  if (!del) {
    const double rn = rng.next() * weight[kappa_ins - 1];
    while (sel < kappa_ins && !(rn < weight[sel])) ++sel;
    if (sel == kappa_ins) return true;
  }
  ln_pbias = ln_pbias - beta * nrg[sel] - std::log(weight[kappa_ins - 1]);
  for (int a : fa) {
    m.r[3 * a] = r0[3 * a] - com_old[0] + anchors[3 * sel];
    m.r[3 * a + 1] = r0[3 * a + 1] - com_old[1] + anchors[3 * sel + 1];
    m.r[3 * a + 2] = r0[3 * a + 2] - com_old[2] + anchors[3 * sel + 2];
  }
  m.com[0] = anchors[3 * sel];
  m.com[1] = anchors[3 * sel + 1];
  m.com[2] = anchors[3 * sel + 2];
  const double e_prev = dihedral_energy(s, m.r.data(), m.exist.data());
  std::vector<int> placed(s.nfrag, 0);
  placed[fstart] = 1;
  if (place_fragments(c, ibox, m, slot, order, 1, placed, del, kappa_dih, e_prev, ln_pbias, rng)) return true;
  if (order.size() > 1) {
    get_com(c, m.is, m.r.data(), m.exist.data(), m.com);
    m.max_dcom = max_com_distance(c, m.is, m.r.data(), m.exist.data(), m.com);
  }
  return false;
}

struct GcmcChain {
  McChain mc;  // RNG, energy, translate / rotate
  int is = 0;  // exchanged species (0-based)
  double mu = 0.0, log_lambda3 = 0.0;
  const CassGCMCParams* gp = nullptr;
  std::vector<int> pool;  // free slots of this box, ascending; insertion takes the last
  std::vector<int> frag_bond_a, frag_bond_b;
  std::vector<double> prob_del1;
  CassGCMCResult res{};

  orc_ctx* c() const { return mc.c; }
  int ibox() const { return mc.ibox; }

  void set_members_changed() {
    // sp_off after an insertion or deletion (members stay sorted by slot)
    orc_ctx* cc = mc.c;
    const std::vector<int>& mem = cc->members[mc.ibox];
    size_t k = 0;
    for (int s2 = 0; s2 <= cc->nspecies; ++s2) {
      const int lim = s2 < cc->nspecies ? cc->mol_base[s2] : INT32_MAX;
      while (k < mem.size() && mem[k] < lim) ++k;
      cc->sp_off[mc.ibox][s2] = (int)k;
    }
  }

  std::vector<double> beads_with(const Species& s, double sign) const {
    std::vector<double> nb = count_beads(mc.c, mc.ibox);
    for (int a = 0; a < s.natoms; ++a)
      if (s.type[a] >= 0) nb[s.type[a]] += sign;
    return nb;
  }

  // Insertion (move_insert.f90)
  void insert() {
    orc_ctx* cc = c();
    const Box& b = cc->box[ibox()];
    Rng& rng = mc.rng;
    (void)(int)(rng.next() * 1.0);  // is_rand = INT(rranf() * nspec_insert) + 1
    if (pool.empty()) {
      mc.err = fail(CASS_ECAPACITY, "no free molecule slot left for an insertion");
      return;
    }
    ++res.n_insert;
    const int slot = pool.back();
    Mol& m = cc->mol[slot];
    const Species& s = cc->sp[is];
    m.is = is;
    m.ibox = ibox();
    m.r.assign(3 * s.natoms, 0.0);
    m.exist.assign(s.natoms, 0);
    double ln_pseq = 0.0, ln_pbias = 0.0;
    const bool cbmc_ov = build_molecule(cc, ibox(), m, slot, false, gp->kappa_ins, gp->kappa_dih, ln_pseq, ln_pbias, rng);
    std::fill(m.exist.begin(), m.exist.end(), 1);
    ln_pbias = ln_pbias + ln_pseq + std::log((double)gp->kappa_ins);
    if (gp->kappa_dih != 0) ln_pbias = ln_pbias + (double)(s.nfrag - 1) * std::log((double)gp->kappa_dih);
    if (cbmc_ov) return;
    fold_molecule(b, m);
    refresh_com(cc, m);
    double ev, eq, eiv, eiq, eoq;
    if (mol_inter_energy(cc, ibox(), view_of(m), slot, false, ev, eq)) return;
    if (mol_intra_energy(cc, b, is, m.r.data(), m.exist.data(), false, eiv, eiq, eoq)) return;
    eq = eq + eoq;
    double dE_inter = ev + eq, dE_intra = eiv + eiq;
    const double eb = bond_energy(s, m.r.data()), ea = angle_energy(s, m.r.data(), m.exist.data());
    const double ed = dihedral_energy(s, m.r.data(), m.exist.data()), ei = improper_energy(s, m.r.data());
    dE_intra = dE_intra + eb + ea + ed + ei;
    // Ewald energies (move_insert.f90:274-291): the molecule's structure factor
    // added to the box's (Update_System_Ewald_Reciprocal_Energy, int_insertion)
    // and its self energy (Compute_Molecule_Self_Energy)
    Box& bw = cc->box[ibox()];
    const bool ew = box_has_ewald(b) && s.has_charge;
    std::vector<double> cn, sn;
    double E_recip = mc.E.reciprocal, E_self = 0.0;
    if (b.charge_style == CASS_CHARGE_COUL) {
      if (ew) {
        const size_t nv = b.hx.size();
        cn.assign(nv, 0.0);
        sn.assign(nv, 0.0);
        mol_structure_factor(cc, b, is, m.r.data(), cn.data(), sn.data());
        double Er = 0.0;
        for (size_t i = 0; i < nv; ++i) {
          const double cs = b.cos_sum[i] + cn[i], ss = b.sin_sum[i] + sn[i];
          Er = Er + b.Cn[i] * (cs * cs + ss * ss);
        }
        E_recip = Er * CHARGE_FACTOR;
        dE_inter = dE_inter + (E_recip - mc.E.reciprocal);
      }
      E_self = molecule_self(cc, b, is);
      dE_inter = dE_inter + E_self;
    }
    double e_lrc = mc.E.lrc;
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) {
      e_lrc = lr_correction(cc, b, beads_with(s, 1.0));
      dE_inter = dE_inter + e_lrc - mc.E.lrc;
    }
    const double dE = dE_intra + dE_inter;
    const double dE_frag = ea;
    const int nmols = mc.nmols(is) + 1;
    double ln_pacc = b.beta * (dE - dE_frag);
    ln_pacc = ln_pacc - mu * b.beta;
    ln_pacc = ln_pacc + ln_pbias;
    ln_pacc = ln_pacc + std::log((double)nmols) + log_lambda3;
    ln_pacc = ln_pacc - std::log(b.volume);
    if (!accept_or_reject(ln_pacc, rng)) return;
    CassEnergy& E = mc.E;
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
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) E.lrc = e_lrc;
    if (ew) {
      for (size_t i = 0; i < cn.size(); ++i) {
        bw.cos_sum[i] = bw.cos_sum[i] + cn[i];
        bw.sin_sum[i] = bw.sin_sum[i] + sn[i];
      }
      m.cos_mol = cn;
      m.sin_mol = sn;
      E.reciprocal = E_recip;
    }
    E.self += E_self;
    ++res.n_insert_accepted;
    pool.pop_back();
    m.live = true;
    std::vector<int>& mem = cc->members[ibox()];
    mem.insert(std::lower_bound(mem.begin(), mem.end(), slot), slot);
    set_members_changed();
  }

  // Deletion (move_delete.f90)
  void remove() {
    orc_ctx* cc = c();
    const Box& b = cc->box[ibox()];
    Rng& rng = mc.rng;
    (void)(int)(rng.next() * 1.0);  // is_rand
    const int nmols = mc.nmols(is);
    if (nmols == 0) return;
    ++res.n_delete;
    const int im = std::min((int)(rng.next() * nmols) + 1, nmols);
    const int slot = cc->members[ibox()][cc->sp_off[ibox()][is] + im - 1];
    Mol& m = cc->mol[slot];
    const Species& s = cc->sp[is];
    double ln_pseq = 0.0, ln_pbias = 0.0;
    const bool cbmc_ov = build_molecule(cc, ibox(), m, slot, true, gp->kappa_ins, gp->kappa_dih, ln_pseq, ln_pbias, rng);
    std::fill(m.exist.begin(), m.exist.end(), 1);
    if (cbmc_ov) {
      mc.err = fail(CASS_ESTATE, "molecule energy too high for a deletion");
      return;
    }
    ln_pbias = ln_pbias + ln_pseq + std::log((double)gp->kappa_ins);
    if (gp->kappa_dih != 0) ln_pbias = ln_pbias + (double)(s.nfrag - 1) * std::log((double)gp->kappa_dih);
    refresh_com(cc, m);
    double ev, eq, eiv, eiq, eoq;
    mol_inter_energy(cc, ibox(), view_of(m), slot, false, ev, eq);
    double dE_inter = -ev - eq;
    const double eb = bond_energy(s, m.r.data()), ea = angle_energy(s, m.r.data(), m.exist.data());
    const double ed = dihedral_energy(s, m.r.data(), m.exist.data()), ei = improper_energy(s, m.r.data());
    double dE_intra = -eb - ea - ed - ei;
    mol_intra_energy(cc, b, is, m.r.data(), m.exist.data(), false, eiv, eiq, eoq);
    eq = eq + eoq;
    dE_intra = dE_intra - eiv - eiq;
    dE_inter = dE_inter - eoq;
    // Ewald energies (move_delete.f90:261-277): the molecule's structure factor
    // taken out of the box's (int_deletion) and its self energy
    Box& bw = cc->box[ibox()];
    const bool ew = box_has_ewald(b) && s.has_charge;
    double E_recip = mc.E.reciprocal, E_self = 0.0;
    if (b.charge_style == CASS_CHARGE_COUL) {
      if (ew) {
        double Er = 0.0;
        for (size_t i = 0; i < b.hx.size(); ++i) {
          const double cs = b.cos_sum[i] - m.cos_mol[i], ss = b.sin_sum[i] - m.sin_mol[i];
          Er = Er + b.Cn[i] * (cs * cs + ss * ss);
        }
        E_recip = Er * CHARGE_FACTOR;
        dE_inter = dE_inter + (E_recip - mc.E.reciprocal);
      }
      E_self = molecule_self(cc, b, is);
      dE_inter = dE_inter - E_self;
    }
    double e_lrc = mc.E.lrc;
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) {
      e_lrc = lr_correction(cc, b, beads_with(s, -1.0));
      dE_inter = dE_inter + (e_lrc - mc.E.lrc);
    }
    const double dE = dE_intra + dE_inter;
    const double dE_frag = -ea;
    double ln_pacc = b.beta * (dE - dE_frag);
    ln_pacc = ln_pacc + b.beta * mu;
    ln_pacc = ln_pacc - ln_pbias;
    ln_pacc = ln_pacc - std::log((double)nmols) - log_lambda3;
    ln_pacc = ln_pacc + std::log(b.volume);
    if (!accept_or_reject(ln_pacc, rng)) return;
    CassEnergy& E = mc.E;
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
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) E.lrc = e_lrc;
    if (ew) {
      for (size_t i = 0; i < b.hx.size(); ++i) {
        bw.cos_sum[i] = bw.cos_sum[i] - m.cos_mol[i];
        bw.sin_sum[i] = bw.sin_sum[i] - m.sin_mol[i];
      }
      E.reciprocal = E_recip;
    }
    E.self -= E_self;
    ++res.n_delete_accepted;
    m.live = false;
    std::vector<int>& mem = cc->members[ibox()];
    mem.erase(std::lower_bound(mem.begin(), mem.end(), slot));
    set_members_changed();
    pool.push_back(slot);
  }

  // energies of molecule m for Cut_N_Grow: bonded + intra + inter (full cutoffs)
  bool mol_energies(Mol& m, int slot, double& eb, double& ea, double& ed, double& ei, double& eiv, double& eiq,
                    double& ev, double& eq) {
    orc_ctx* cc = c();
    const Species& s = cc->sp[m.is];
    eb = bond_energy(s, m.r.data());
    ea = angle_energy(s, m.r.data(), m.exist.data());
    ed = dihedral_energy(s, m.r.data(), m.exist.data());
    ei = improper_energy(s, m.r.data());
    double eoq;
    mol_intra_energy(cc, cc->box[ibox()], m.is, m.r.data(), m.exist.data(), false, eiv, eiq, eoq);
    const bool ov = mol_inter_energy(cc, ibox(), view_of(m), slot, false, ev, eq);
    eq = eq + eoq;
    return ov;
  }

  // Cut_Regrow (fragment_growth.f90:1118-1312) on molecule m
  bool cut_regrow(Mol& m, int slot, bool del, std::vector<int>& order, int& f_live, int& f_dead, double& e_prev,
                  double& ln_pbias) {
    orc_ctx* cc = c();
    const Species& s = cc->sp[m.is];
    Rng& rng = mc.rng;
    ln_pbias = 0.0;
    if (!del) {
      const int nfb = (int)frag_bond_a.size();
      const int fb = std::min((int)(rng.next() * nfb), nfb - 1);
      if (rng.next() < prob_del1[fb]) {
        f_dead = frag_bond_a[fb];
        f_live = frag_bond_b[fb];
      } else {
        f_dead = frag_bond_b[fb];
        f_live = frag_bond_a[fb];
      }
      std::vector<int> live(s.nfrag, 0);
      live[f_live] = 1;
      order.assign(1, f_dead);
      live[f_dead] = 1;
      double ln_pseq = 0.0;
      fragment_order(s, f_dead, order, live, ln_pseq, rng);
    }
    std::fill(m.exist.begin(), m.exist.end(), 1);
    std::vector<int> placed(s.nfrag, 1);
    for (int f : order) {
      placed[f] = 0;
      for (int a : s.frag_atoms[f]) m.exist[a] = 0;
    }
    m.exist[s.frag_atoms[f_live][0]] = 1;
    m.exist[s.frag_atoms[f_dead][0]] = 1;
    if (!del) e_prev = dihedral_energy(s, m.r.data(), m.exist.data());
    return place_fragments(cc, ibox(), m, slot, order, 0, placed, del, gp->kappa_dih, e_prev, ln_pbias, rng);
  }

  // Cut_N_Grow (move_regrow.f90)
  void regrow() {
    orc_ctx* cc = c();
    const Box& b = cc->box[ibox()];
    Rng& rng = mc.rng;
    const int nmols = mc.nmols(is);
    if (nmols == 0) return;
    (void)rng.next();  // the box choice
    (void)rng.next();  // the species choice
    const int im = std::min((int)(rng.next() * nmols) + 1, nmols);
    const int slot = cc->members[ibox()][cc->sp_off[ibox()][is] + im - 1];
    Mol& m = cc->mol[slot];
    const Species& s = cc->sp[is];
    ++res.n_regrow;
    if (s.nfrag < 2) return;  // single-fragment regrowth is not on this path
    const std::vector<double> r_old(m.r);
    const double com_old[3] = {m.com[0], m.com[1], m.com[2]}, dcom_old = m.max_dcom;
    std::vector<int> order;
    int f_live = 0, f_dead = 0;
    double e_prev = 0.0, ln_pfor = 0.0, ln_prev = 0.0;
    bool ov = cut_regrow(m, slot, false, order, f_live, f_dead, e_prev, ln_pfor);
    std::fill(m.exist.begin(), m.exist.end(), 1);
    refresh_com(cc, m);
    fold_molecule(b, m);
    auto revert = [&]() {  // Revert_Old_Cartesian_Coordinates
      m.r = r_old;
      std::copy(com_old, com_old + 3, m.com);
      m.max_dcom = dcom_old;
    };
    if (ov) {
      revert();
      return;
    }
    double eb_n, ea_n, ed_n, ei_n, eiv_n, eiq_n, ev_n, eq_n;
    if (mol_energies(m, slot, eb_n, ea_n, ed_n, ei_n, eiv_n, eiq_n, ev_n, eq_n)) {
      revert();
      return;
    }
    double dE_intra = eb_n + ea_n + ed_n + ei_n + eiq_n + eiv_n;
    double dE_inter = eq_n + ev_n;
    // the reciprocal energy of the new conformation (move_regrow.f90:338-354,
    // Update_System_Ewald_Reciprocal_Energy with int_intra), kept for acceptance
    Box& bw = cc->box[ibox()];
    const bool ew = box_has_ewald(b) && s.has_charge;
    double E_recip = mc.E.reciprocal;
    if (ew) {
      E_recip = ewald_move(cc, bw, m);
      dE_inter = dE_inter + (E_recip - mc.E.reciprocal);
    }
    const std::vector<double> r_new(m.r);
    const double com_new[3] = {m.com[0], m.com[1], m.com[2]}, dcom_new = m.max_dcom;
    revert();
    ov = cut_regrow(m, slot, true, order, f_live, f_dead, e_prev, ln_prev);
    std::fill(m.exist.begin(), m.exist.end(), 1);
    if (ov) {
      if (ew) ewald_revert(bw, m);
      mc.err = fail(CASS_ESTATE, "molecule energy too high for a regrowth");
      return;
    }
    refresh_com(cc, m);
    double eb_o, ea_o, ed_o, ei_o, eiv_o, eiq_o, ev_o, eq_o;
    mol_energies(m, slot, eb_o, ea_o, ed_o, ei_o, eiv_o, eiq_o, ev_o, eq_o);
    dE_intra = dE_intra - eb_o - ea_o - ed_o - ei_o - eiq_o - eiv_o;
    dE_inter = dE_inter - eq_o - ev_o;
    const double dE = dE_intra + dE_inter;
    const double dE_frag = ea_n - ea_o;
    const double ln_pacc = b.beta * (dE - dE_frag) + ln_pfor - ln_prev;
    if (!accept_or_reject(ln_pacc, rng)) {
      if (ew) ewald_revert(bw, m);
      return;
    }
    if (ew) mc.E.reciprocal = E_recip;
    m.r = r_new;
    std::copy(com_new, com_new + 3, m.com);
    m.max_dcom = dcom_new;
    CassEnergy& E = mc.E;
    E.total += dE;
    E.intra += dE_intra;
    E.inter += dE_inter;
    E.bond += eb_n - eb_o;
    E.angle += ea_n - ea_o;
    E.dihedral += ed_n - ed_o;
    E.improper += ei_n - ei_o;
    E.intra_vdw += eiv_n - eiv_o;
    E.intra_q += eiq_n - eiq_o;
    E.inter_vdw += ev_n - ev_o;
    E.inter_q += eq_n - eq_o;
    ++res.n_regrow_accepted;
  }

  void run() {
    for (int64_t k = 0; k < gp->nsteps && mc.err == CASS_OK; ++k) {
      const double u = mc.rng.next();  // gcmc_driver.f90:30
      if (u <= gp->cut_translate) mc.translate();
      else if (u <= gp->cut_rotate) mc.rotate();
      else if (u <= gp->cut_insert) insert();
      else if (u <= gp->cut_delete) remove();
      else if (u <= gp->cut_regrow) regrow();
      res.sum_n_molecules += (double)mc.nmols(is);
    }
    res.n_translate = mc.res.n_translate;
    res.n_translate_accepted = mc.res.n_translate_accepted;
    res.n_rotate = mc.res.n_rotate;
    res.n_rotate_accepted = mc.res.n_rotate_accepted;
    res.n_molecules = mc.nmols(is);
    res.energy = mc.E;
  }
};

}  // namespace

extern "C" {

int orc_abi_version(void) { return CASS_ABI_VERSION; }
const char* orc_last_error(void) { return g_err.c_str(); }

int orc_ctx_create(const CassConfig* cfg, orc_ctx** out) {
  if (!cfg || !out || cfg->nspecies < 1 || cfg->ntypes < 1 || cfg->nboxes < 1 || !cfg->max_molecules)
    return fail(CASS_EINVAL, "bad config");
  orc_ctx* c = new orc_ctx();
  c->nspecies = cfg->nspecies;
  c->ntypes = cfg->ntypes;
  c->nboxes = cfg->nboxes;
  if (cfg->max_kvectors > 0) c->max_kvec = cfg->max_kvectors;
  c->max_mol.assign(cfg->max_molecules, cfg->max_molecules + cfg->nspecies);
  c->mol_base.resize(c->nspecies);
  int tot = 0;
  for (int i = 0; i < c->nspecies; ++i) {
    c->mol_base[i] = tot;
    tot += c->max_mol[i];
  }
  c->mol.resize(tot);
  c->sp.resize(c->nspecies);
  c->box.resize(c->nboxes);
  c->eps.assign(c->ntypes * c->ntypes, 0.0);
  c->sig = c->eps;
  c->mie_n = c->eps;
  c->mie_m = c->eps;
  *out = c;
  return CASS_OK;
}

int orc_ctx_destroy(orc_ctx* c) {
  delete c;
  return CASS_OK;
}

int orc_set_nonbond_table(orc_ctx* c, int32_t nt, const double* eps, const double* sig, const double* mn,
                          const double* mm) {
  if (check_ctx(c) || nt != c->ntypes || !eps || !sig) return fail(CASS_EINVAL, "bad nonbond table");
  c->eps.assign(eps, eps + nt * nt);
  c->sig.assign(sig, sig + nt * nt);
  if (mn) c->mie_n.assign(mn, mn + nt * nt);
  if (mm) c->mie_m.assign(mm, mm + nt * nt);
  c->cbmc_dirty = true;
  return CASS_OK;
}

int orc_set_species(orc_ctx* c, int32_t is, const CassSpeciesDesc* d) {
  if (check_ctx(c) || is < 1 || is > c->nspecies || !d || d->natoms < 1) return fail(CASS_EINVAL, "bad species");
  if (!d->atom_type || !d->charge || !d->mass || !d->vdw_intra_scale || !d->charge_intra_scale || !d->bonded)
    return fail(CASS_EINVAL, "species arrays missing");
  if (d->nfragments > 0 && (!d->frag_natoms || !d->frag_atoms || !d->frag_nconnect || !d->frag_nconfig))
    return fail(CASS_EINVAL, "fragment arrays missing");
  for (int f = 0; f < d->nfragments; ++f)
    if (d->frag_natoms[f] < 1 || d->frag_natoms[f] > d->natoms) return fail(CASS_EINVAL, "bad fragment sizes");
  Species& s = c->sp[is - 1];
  int n = d->natoms;
  c->cbmc_dirty = true;
  s = Species();
  s.natoms = n;
  s.type.resize(n);
  for (int i = 0; i < n; ++i) s.type[i] = d->atom_type[i] - 1;
  s.q.assign(d->charge, d->charge + n);
  s.mass.assign(d->mass, d->mass + n);
  s.vdw_scale.assign(d->vdw_intra_scale, d->vdw_intra_scale + n * n);
  s.qq_scale.assign(d->charge_intra_scale, d->charge_intra_scale + n * n);
  s.bonded.assign(d->bonded, d->bonded + n * n);
  for (int k = 0; k < d->nbonds; ++k) {
    s.bond_atoms.push_back(d->bond_atoms[2 * k] - 1);
    s.bond_atoms.push_back(d->bond_atoms[2 * k + 1] - 1);
    s.bond_kind.push_back(d->bond_kind[k]);
    s.bond_param.push_back(d->bond_param[2 * k]);
    s.bond_param.push_back(d->bond_param[2 * k + 1]);
  }
  for (int k = 0; k < d->nangles; ++k) {
    for (int j = 0; j < 3; ++j) s.angle_atoms.push_back(d->angle_atoms[3 * k + j] - 1);
    s.angle_kind.push_back(d->angle_kind[k]);
    s.angle_param.push_back(d->angle_param[2 * k]);
    s.angle_param.push_back(d->angle_param[2 * k + 1]);
  }
  for (int k = 0; k < d->ndihedrals; ++k) {
    for (int j = 0; j < 4; ++j) s.dih_atoms.push_back(d->dihedral_atoms[4 * k + j] - 1);
    for (int j = 0; j < 6; ++j) s.dih_rb.push_back(d->dihedral_rb[6 * k + j]);
  }
  for (int k = 0; k < d->nimpropers; ++k) {
    for (int j = 0; j < 4; ++j) s.imp_atoms.push_back(d->improper_atoms[4 * k + j] - 1);
    s.imp_param.push_back(d->improper_param[2 * k]);
    s.imp_param.push_back(d->improper_param[2 * k + 1]);
  }
  s.nfrag = d->nfragments;
  int off = 0, coff = 0;
  size_t loff = 0;
  int tot_atoms = 0;
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
    s.frag_lib.emplace_back(d->frag_library + loff, d->frag_library + loff + len);
    loff += len;
    tot_atoms += d->frag_natoms[f];
  }
  // prob_ins / cum_prob_ins (input_routines.f90:2844-2848)
  int acc = 0;
  for (int f = 0; f < s.nfrag; ++f) {
    s.prob_ins.push_back((double)d->frag_natoms[f] / (double)tot_atoms);
    acc += d->frag_natoms[f];
    s.cum_prob_ins.push_back(f == 0 ? s.prob_ins[0] : (double)acc / (double)tot_atoms);
  }
  s.l_coul_cbmc = d->l_coul_cbmc != 0;
  s.has_charge = false;
  for (int i = 0; i < n; ++i)
    if (s.q[i] != 0.0) s.has_charge = true;
  s.defined = true;
  for (int im = 0; im < c->max_mol[is - 1]; ++im) {
    Mol& m = mol_of(c, is - 1, im);
    m.is = is - 1;
    m.r.assign(3 * n, 0.0);
    m.exist.assign(n, 1);
  }
  return CASS_OK;
}

int orc_set_box(orc_ctx* c, int32_t ibox, const CassBoxDesc* d) {
  if (check_ctx(c) || ibox < 1 || ibox > c->nboxes || !d) return fail(CASS_EINVAL, "bad box");
  Box& b = c->box[ibox - 1];
  b = Box();
  b.desc = *d;
  c->cbmc_dirty = true;
  for (int k = 0; k < 3; ++k) {
    b.L[k] = d->length[k];
    b.hL[k] = 0.5 * d->length[k];
  }
  b.volume = b.L[0] * b.L[1] * b.L[2];
  b.vdw_style = d->vdw_style;
  b.vdw_sum_style = d->vdw_sum_style;
  b.charge_style = d->charge_style;
  b.charge_sum_style = d->charge_sum_style;
  b.rcut_vdw = d->rcut_vdw;
  b.rcut_coul = d->charge_style == CASS_CHARGE_COUL ? d->rcut_coul : 0.0;
  b.rcut_cbmc = d->rcut_cbmc;
  b.rcut_low = d->rcut_low;
  b.rcut_vdwsq = b.rcut_vdw * b.rcut_vdw;
  b.rcut_coulsq = b.rcut_coul * b.rcut_coul;
  b.rcut_cbmcsq = b.rcut_cbmc * b.rcut_cbmc;
  b.rcut_lowsq = b.rcut_low * b.rcut_low;
  // precalculate.f90:79-83
  b.rcut_max = std::max(b.rcut_vdw, b.rcut_coul);
  b.rcut3 = b.rcut_vdw * b.rcut_vdw * b.rcut_vdw;
  b.rcut9 = b.rcut3 * b.rcut3 * b.rcut3;
  b.ron_switch_sq = d->ron_switch * d->ron_switch;
  b.roff_switch_sq = d->roff_switch * d->roff_switch;
  if (d->vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) {
    double d2 = b.roff_switch_sq - b.ron_switch_sq;
    b.switch_factor1 = 1.0 / (d2 * d2 * d2);
    b.switch_factor2 = b.roff_switch_sq - 3.0 * b.ron_switch_sq;
  }
  b.beta = 1.0 / (KBOLTZ * d->temperature);
  if (b.charge_style == CASS_CHARGE_COUL && b.charge_sum_style == CASS_QQ_EWALD) {
    // input_routines.f90:711-716
    double p = -std::log(d->ewald_tol);
    b.alpha_ewald = std::sqrt(p) / b.rcut_coul;
    b.h_ewald_cut = 2.0 * p / b.rcut_coul;
    int rc = ewald_setup(c, b);
    if (rc) return rc;
  }
  if (b.charge_style == CASS_CHARGE_COUL && b.charge_sum_style == CASS_QQ_DSF) {
    double a = d->alpha_dsf;
    if (a <= 0.0) {
      a = 0.425 - b.rcut_coul * 0.02;
      if (a < 0.0) a = 3.3930702 / b.rcut_coul;
    }
    b.alpha_dsf = a;
    b.dsf_factor1 = std::erfc(a * b.rcut_coul) / b.rcut_coul;
    b.dsf_factor2 = b.dsf_factor1 / b.rcut_coul +
                    2.0 * a * std::exp(-a * a * b.rcut_coul * b.rcut_coul) / (ROOTPI * b.rcut_coul);
  }
  b.defined = true;
  return CASS_OK;
}

int orc_set_molecules(orc_ctx* c, int32_t n, const int32_t* im, const int32_t* is, const int32_t* ibox,
                      const double* xyz) {
  if (check_ctx(c) || n < 0) return fail(CASS_EINVAL, "bad molecule list");
  size_t off = 0;
  for (int k = 0; k < n; ++k) {
    int rc = check_mol(c, im[k], is[k]);
    if (rc) return rc;
    if (ibox[k] < 1 || ibox[k] > c->nboxes) return fail(CASS_EINVAL, "box index out of range");
    Mol& m = mol_of(c, is[k] - 1, im[k] - 1);
    int na = c->sp[is[k] - 1].natoms;
    if (m.live) invalidate_box(c, m.ibox);
    if (!m.live || m.ibox != ibox[k] - 1) c->members_dirty = true;
    m.ibox = ibox[k] - 1;
    m.live = true;
    m.r.assign(xyz + off, xyz + off + 3 * na);
    m.exist.assign(na, 1);
    off += 3 * na;
    refresh_com(c, m);
    invalidate_box(c, m.ibox);
  }
  return CASS_OK;
}

int orc_remove_molecule(orc_ctx* c, int32_t im, int32_t is) {
  int rc = check_ctx(c) ? CASS_EINVAL : check_mol(c, im, is);
  if (rc) return rc;
  Mol& m = mol_of(c, is - 1, im - 1);
  if (m.live) invalidate_box(c, m.ibox);
  if (m.live) c->members_dirty = true;
  m.live = false;
  return CASS_OK;
}

int orc_get_molecule(orc_ctx* c, int32_t im, int32_t is, double* xyz) {
  int rc = check_ctx(c) ? CASS_EINVAL : check_mol(c, im, is);
  if (rc) return rc;
  Mol& m = mol_of(c, is - 1, im - 1);
  std::copy(m.r.begin(), m.r.end(), xyz);
  return CASS_OK;
}

int orc_get_molecule_boxes(orc_ctx* c, int32_t is, int32_t n, int32_t* which_box) {
  if (check_ctx(c) || (!which_box && n > 0)) return fail(CASS_EINVAL, "NULL argument");
  if (is < 1 || is > c->nspecies) return fail(CASS_EINVAL, "species index out of range");
  if (n < 0 || n > c->max_mol[is - 1]) return fail(CASS_EINVAL, "n out of range");
  for (int im = 1; im <= n; ++im) {
    const Mol& m = mol_of(c, is - 1, im - 1);
    which_box[im - 1] = m.live ? m.ibox + 1 : 0;
  }
  return CASS_OK;
}

// the tables of the CBMC options, rebuilt after a change of boxes, species,
// pair table or options
static int cbmc_ready(orc_ctx* c) {
  if (c->opt.energy_table_res <= 0 && !c->opt.sector_overlap) return CASS_OK;
  return build_cbmc(c);
}

int orc_system_total_energy(orc_ctx* c, int32_t ibox1, int32_t intra_flag, CassEnergy* out, int32_t* overlap);

// Volume_Change (move_volume.f90:24-679), cubic box, up to its acceptance
// test: fractional COMs kept and molecules moved rigidly (:296-336), new edge
// and k-vectors (:374), system energy recomputed (:426); the old state kept.
int orc_volume_scale(orc_ctx* c, int32_t ibox1, double new_length, CassEnergy* e_new, int32_t* overlap) {
  if (c) refresh_members(c);
  if (check_ctx(c) || ibox1 < 1 || ibox1 > c->nboxes || !e_new || !overlap || !(new_length > 0.0))
    return fail(CASS_EINVAL, "bad volume move arguments");
  const Box& b = c->box[ibox1 - 1];
  if (!b.defined) return fail(CASS_ESTATE, "box not defined");
  if (!b.energy_valid) return fail(CASS_ESTATE, "system energy of box not computed");
  const CassBoxDesc d0 = b.desc;
  if (d0.length[0] != d0.length[1] || d0.length[0] != d0.length[2]) return fail(CASS_EUNSUPPORTED, "volume moves need a cubic box");
  const double half = 0.5 * new_length;
  if (half < d0.rcut_vdw || (d0.charge_style == CASS_CHARGE_COUL && half < d0.rcut_coul) ||
      (d0.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH && half < d0.roff_switch))
    return fail(CASS_EINVAL, "cutoff greater than half the new box length");
  if ((int)c->vol.size() < c->nboxes) c->vol.resize(c->nboxes);
  orc_ctx::VolSave& v = c->vol[ibox1 - 1];
  v = orc_ctx::VolSave();
  v.saved = true;
  v.desc = d0;
  v.energy = b.energy;
  const double L0 = d0.length[0];
  std::vector<double> xyz_new;
  for (int slot : c->members[ibox1 - 1]) {
    const Mol& m = c->mol[slot];
    const Species& sp = c->sp[m.is];
    double tm = 0.0, com[3] = {0.0, 0.0, 0.0};  // Get_COM (get_com.f90:45-105)
    for (int a = 0; a < sp.natoms; ++a) {
      tm += sp.mass[a];
      for (int k = 0; k < 3; ++k) com[k] += sp.mass[a] * m.r[3 * a + k];
    }
    double sh[3];
    for (int k = 0; k < 3; ++k) {
      com[k] = com[k] / tm;
      sh[k] = new_length * (com[k] / L0) - com[k];
    }
    v.im.push_back(slot - c->mol_base[m.is] + 1);
    v.is.push_back(m.is + 1);
    for (int a = 0; a < 3 * sp.natoms; ++a) {
      v.xyz.push_back(m.r[a]);
      xyz_new.push_back(m.r[a] + sh[a % 3]);
    }
  }
  const int n = (int)v.im.size();
  std::vector<int32_t> boxes(n, ibox1);
  int rc;
  if (n > 0 && (rc = orc_set_molecules(c, n, v.im.data(), v.is.data(), boxes.data(), xyz_new.data()))) return rc;
  CassBoxDesc d1 = d0;
  d1.length[0] = d1.length[1] = d1.length[2] = new_length;
  if ((rc = orc_set_box(c, ibox1, &d1))) return rc;
  return orc_system_total_energy(c, ibox1, 1, e_new, overlap);
}

// Reset_Coords (move_volume.f90:555-677)
int orc_volume_restore(orc_ctx* c, int32_t ibox1) {
  if (check_ctx(c) || ibox1 < 1 || ibox1 > c->nboxes) return fail(CASS_EINVAL, "bad box");
  if ((int)c->vol.size() < c->nboxes || !c->vol[ibox1 - 1].saved) return fail(CASS_ESTATE, "no volume move to restore");
  orc_ctx::VolSave v = c->vol[ibox1 - 1];
  const int n = (int)v.im.size();
  std::vector<int32_t> boxes(n, ibox1);
  int rc;
  if (n > 0 && (rc = orc_set_molecules(c, n, v.im.data(), v.is.data(), boxes.data(), v.xyz.data()))) return rc;
  if ((rc = orc_set_box(c, ibox1, &v.desc))) return rc;
  CassEnergy e;
  int32_t ov = 0;
  if ((rc = orc_system_total_energy(c, ibox1, 1, &e, &ov))) return rc;
  c->box[ibox1 - 1].energy = v.energy;
  c->vol[ibox1 - 1].saved = false;
  return CASS_OK;
}

int orc_set_cbmc_options(orc_ctx* c, const CassCBMCOptions* o) {
  if (check_ctx(c) || !o || o->energy_table_res < 0 || o->rmin_u_max < 0.0) return fail(CASS_EINVAL, "bad CBMC options");
  c->opt = *o;
  c->cbmc_dirty = true;
  return CASS_OK;
}

int orc_mol_inter_energy(orc_ctx* c, int32_t im, int32_t is, int32_t cbmc, double* ev, double* eq, int32_t* ov) {
  if (c) refresh_members(c);
  int rc = check_ctx(c) ? CASS_EINVAL : check_mol(c, im, is);
  if (rc) return rc;
  if (cbmc && (rc = cbmc_ready(c))) return rc;
  Mol& m = mol_of(c, is - 1, im - 1);
  if (!m.live) return fail(CASS_ESTATE, "molecule not live");
  int slot = c->mol_base[is - 1] + im - 1;
  double a, b;
  bool o = mol_inter_energy(c, m.ibox, view_of(m), slot, cbmc != 0, a, b);
  *ev = o ? 0.0 : a;
  *eq = o ? 0.0 : b;
  *ov = o ? 1 : 0;
  return CASS_OK;
}

int orc_mol_intra_energy(orc_ctx* c, int32_t im, int32_t is, int32_t cbmc, double* eiv, double* eiq, double* eoq,
                         int32_t* ov) {
  if (c) refresh_members(c);
  int rc = check_ctx(c) ? CASS_EINVAL : check_mol(c, im, is);
  if (rc) return rc;
  Mol& m = mol_of(c, is - 1, im - 1);
  if (!m.live) return fail(CASS_ESTATE, "molecule not live");
  bool o = mol_intra_energy(c, c->box[m.ibox], is - 1, m.r.data(), m.exist.data(), cbmc != 0, *eiv, *eiq, *eoq);
  *ov = o ? 1 : 0;
  return CASS_OK;
}

// Compute_System_Total_Energy (energy_routines.f90:2648-2953)
int orc_system_total_energy(orc_ctx* c, int32_t ibox1, int32_t intra_flag, CassEnergy* out, int32_t* overlap) {
  if (c) refresh_members(c);
  if (check_ctx(c) || ibox1 < 1 || ibox1 > c->nboxes || !out || !overlap) return fail(CASS_EINVAL, "bad args");
  int ibox = ibox1 - 1;
  Box& b = c->box[ibox];
  CassEnergy& E = b.energy;
  double keep_intra[8] = {E.intra, E.bond, E.angle, E.dihedral, E.improper, E.intra_vdw, E.intra_q, E.self};
  E = CassEnergy{};
  *overlap = 0;
  if (intra_flag) {
    for (int is = 0; is < c->nspecies; ++is) {
      const Species& s = c->sp[is];
      double vi = 0, vb = 0, va = 0, vd = 0, vim = 0, viv = 0, viq = 0, voq = 0;
      const std::vector<int>& mem = c->members[ibox];
      for (int k = c->sp_off[ibox][is]; k < c->sp_off[ibox][is + 1]; ++k) {
        Mol& m = c->mol[mem[k]];
        double mb = bond_energy(s, m.r.data());
        double ma = angle_energy(s, m.r.data(), m.exist.data());
        double md = dihedral_energy(s, m.r.data(), m.exist.data());
        double mi = improper_energy(s, m.r.data());
        double eiv, eiq, eoq;
        if (mol_intra_energy(c, b, is, m.r.data(), m.exist.data(), false, eiv, eiq, eoq)) {
          *overlap = 1;
          return CASS_OK;
        }
        vi = vi + mb + ma + md + mi + eiq + eiv;
        vb += mb;
        va += ma;
        vd += md;
        vim += mi;
        viv += eiv;
        viq += eiq;
        voq += eoq;
      }
      E.intra += vi;
      E.bond += vb;
      E.angle += va;
      E.dihedral += vd;
      E.improper += vim;
      E.intra_vdw += viv;
      E.intra_q += viq;
      E.inter_q += voq;
    }
  } else {
    E.intra = keep_intra[0]; E.bond = keep_intra[1]; E.angle = keep_intra[2]; E.dihedral = keep_intra[3];
    E.improper = keep_intra[4]; E.intra_vdw = keep_intra[5]; E.intra_q = keep_intra[6]; E.self = keep_intra[7];
  }
  // inter-molecular pairs, same species then cross species
  const std::vector<int>& mem = c->members[ibox];
  const std::vector<int>& so = c->sp_off[ibox];
  for (int is1 = 0; is1 < c->nspecies; ++is1) {
    for (int k1 = so[is1]; k1 < so[is1 + 1]; ++k1) {
      Mol& m1 = c->mol[mem[k1]];
      for (int is2 = is1; is2 < c->nspecies; ++is2) {
        double ev = 0, eq = 0;
        for (int k2 = (is2 == is1 ? k1 + 1 : so[is2]); k2 < so[is2 + 1]; ++k2) {
          Mol& m2 = c->mol[mem[k2]];
          MolView a = view_of(m1), v = view_of(m2);
          if (!check_molpair_cutoff(b, a, v, false)) continue;
          double vlj, vqq;
          if (molpair_energy(c, b, a, v, false, vlj, vqq)) {
            *overlap = 1;
            return CASS_OK;
          }
          ev += vlj;
          eq += vqq;
        }
        E.inter_vdw += ev;
        E.inter_q += eq;
      }
    }
  }
  E.inter = E.inter_q + E.inter_vdw;
  if (b.charge_style == CASS_CHARGE_COUL) {
    if (b.charge_sum_style == CASS_QQ_EWALD) {
      E.reciprocal = system_recip(c, ibox);
      E.inter = E.inter + E.reciprocal;
    }
    E.self = system_self(c, ibox);
    E.inter = E.inter + E.self;
  }
  if (b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) {
    E.lrc = lr_correction(c, b, count_beads(c, ibox));
    E.inter = E.inter + E.lrc;
  }
  E.total = E.intra + E.inter;
  *out = E;
  b.energy_valid = true;
  return CASS_OK;
}

// Update_System_Ewald_Reciprocal_Energy (energy_routines.f90:2326-2497)
int orc_ewald_update(orc_ctx* c, int32_t im, int32_t is, int32_t ibox1, int32_t move_flag, double* e_recip) {
  if (c) refresh_members(c);
  int rc = check_ctx(c) ? CASS_EINVAL : check_mol(c, im, is);
  if (rc) return rc;
  if (ibox1 < 1 || ibox1 > c->nboxes) return fail(CASS_EINVAL, "box index");
  Box& b = c->box[ibox1 - 1];
  if (!box_has_ewald(b)) return fail(CASS_ESTATE, "box has no Ewald sum");
  Mol& m = mol_of(c, is - 1, im - 1);
  size_t nv = b.hx.size();
  b.cos_sum_old = b.cos_sum;
  b.sin_sum_old = b.sin_sum;
  if (m.cos_mol.size() != nv) {
    m.cos_mol.assign(nv, 0.0);
    m.sin_mol.assign(nv, 0.0);
  }
  m.cos_mol_old = m.cos_mol;
  m.sin_mol_old = m.sin_mol;
  double E = 0.0;
  if (move_flag == CASS_MOVE_TRANSLATION || move_flag == CASS_MOVE_ROTATION || move_flag == CASS_MOVE_INTRA) {
    std::vector<double> cn(nv), sn(nv);
    mol_structure_factor(c, b, is - 1, m.r.data(), cn.data(), sn.data());
    for (size_t i = 0; i < nv; ++i) {
      b.cos_sum[i] = b.cos_sum[i] + (cn[i] - m.cos_mol[i]);
      b.sin_sum[i] = b.sin_sum[i] + (sn[i] - m.sin_mol[i]);
      E = E + b.Cn[i] * (b.cos_sum[i] * b.cos_sum[i] + b.sin_sum[i] * b.sin_sum[i]);
      m.cos_mol[i] = cn[i];
      m.sin_mol[i] = sn[i];
    }
  } else if (move_flag == CASS_MOVE_DELETION) {
    for (size_t i = 0; i < nv; ++i) {
      b.cos_sum[i] = b.cos_sum[i] - m.cos_mol[i];
      b.sin_sum[i] = b.sin_sum[i] - m.sin_mol[i];
    }
    for (size_t i = 0; i < nv; ++i) E = E + b.Cn[i] * (b.cos_sum[i] * b.cos_sum[i] + b.sin_sum[i] * b.sin_sum[i]);
  } else if (move_flag == CASS_MOVE_INSERTION) {
    mol_structure_factor(c, b, is - 1, m.r.data(), m.cos_mol.data(), m.sin_mol.data());
    for (size_t i = 0; i < nv; ++i) {
      b.cos_sum[i] = b.cos_sum[i] + m.cos_mol[i];
      b.sin_sum[i] = b.sin_sum[i] + m.sin_mol[i];
      E = E + b.Cn[i] * (b.cos_sum[i] * b.cos_sum[i] + b.sin_sum[i] * b.sin_sum[i]);
    }
  } else {
    return fail(CASS_EINVAL, "bad move_flag");
  }
  *e_recip = E * CHARGE_FACTOR;
  return CASS_OK;
}

int orc_ewald_restore(orc_ctx* c, int32_t im, int32_t is, int32_t ibox1) {
  if (c) refresh_members(c);
  int rc = check_ctx(c) ? CASS_EINVAL : check_mol(c, im, is);
  if (rc) return rc;
  Box& b = c->box[ibox1 - 1];
  Mol& m = mol_of(c, is - 1, im - 1);
  b.cos_sum = b.cos_sum_old;
  b.sin_sum = b.sin_sum_old;
  m.cos_mol = m.cos_mol_old;
  m.sin_mol = m.sin_mol_old;
  return CASS_OK;
}

int orc_ewald_widom(orc_ctx* c, int32_t is, int32_t ibox1, int32_t n, const double* xyz, double* e) {
  if (c) refresh_members(c);
  if (check_ctx(c) || is < 1 || is > c->nspecies || ibox1 < 1 || ibox1 > c->nboxes) return fail(CASS_EINVAL, "bad");
  Box& b = c->box[ibox1 - 1];
  const Species& s = c->sp[is - 1];
  for (int k = 0; k < n; ++k) {
    const double* r = xyz + (size_t)k * 3 * s.natoms;
    double E = 0.0;
    for (size_t i = 0; i < b.hx.size(); ++i) {
      double dc = 0, ds = 0;
      for (int ia = 0; ia < s.natoms; ++ia) {
        double hdotr = b.hx[i] * r[3 * ia] + b.hy[i] * r[3 * ia + 1] + b.hz[i] * r[3 * ia + 2];
        dc += s.q[ia] * std::cos(hdotr);
        ds += s.q[ia] * std::sin(hdotr);
      }
      double cs = b.cos_sum[i] + dc, sn = b.sin_sum[i] + ds;
      E = E + b.Cn[i] * (cs * cs + sn * sn);
    }
    e[k] = E * CHARGE_FACTOR;
  }
  return CASS_OK;
}

// Widom_Insert (widom_insert.f90:22-594) over a list of boxes; OpenMP over
// insertions as in the reference (widom_insert.f90:255-320).
int orc_widom_insert(orc_ctx* c, int32_t is1, int32_t nboxes, const int32_t* iboxes, int64_t n_ins,
                     int32_t kappa_ins, int32_t kappa_dih, uint64_t seed, CassWidomResult* out,
                     CassWidomTrace* trace) {
  if (c) refresh_members(c);
  if (check_ctx(c) || is1 < 1 || is1 > c->nspecies || nboxes < 1 || !iboxes || !out || n_ins < 0 || kappa_ins < 1)
    return fail(CASS_EINVAL, "bad widom args");
  int is = is1 - 1;
  const Species& s = c->sp[is];
  if (s.nfrag < 1) return fail(CASS_EINVAL, "species has no fragments");
  if (int rc = cbmc_ready(c)) return rc;
  if (s.nfrag > 1 && kappa_dih < 1) return fail(CASS_EINVAL, "kappa_dih must be >= 1");
  for (int k = 0; k < nboxes; ++k) {
    int ib = iboxes[k] - 1;
    if (ib < 0 || ib >= c->nboxes) return fail(CASS_EINVAL, "box index");
    if (!c->box[ib].energy_valid) return fail(CASS_ESTATE, "system energy of box not computed");
  }
  // Widom_Insert set-up per box (widom_insert.f90:201-245)
  std::vector<double> Ec(nboxes), prefactor(nboxes);
  for (int k = 0; k < nboxes; ++k) {
    int ibox = iboxes[k] - 1;
    const Box& b = c->box[ibox];
    const int nmols = 1 + c->sp_off[ibox][is + 1] - c->sp_off[ibox][is];
    prefactor[k] = b.volume / (double)nmols;
    double lrc_diff = 0.0;
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL) {
      std::vector<double> nb = count_beads(c, ibox);
      for (int ia = 0; ia < s.natoms; ++ia)
        if (s.type[ia] >= 0) nb[s.type[ia]] += 1.0;
      lrc_diff = lr_correction(c, b, nb) - b.energy.lrc;
    }
    double E_self = 0.0, E_recip_in = 0.0;
    if (b.charge_style == CASS_CHARGE_COUL && s.has_charge) {
      E_self = molecule_self(c, b, is);
      E_recip_in = b.energy.reciprocal;
    }
    Ec[k] = lrc_diff + E_self - E_recip_in;
  }
  // every (box, insertion) is independent: one parallel loop over all of them,
  // then per-box sums in insertion order (independent of the thread count)
  const int64_t total = (int64_t)nboxes * n_ins;
  std::vector<InsertionOut> res((size_t)total);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t g = 0; g < total; ++g) {
    const int k = (int)(g / n_ins);
    const int64_t i = g % n_ins;
    Rng rng = seed_stream(seed, iboxes[k], i);
    res[(size_t)g] = widom_one(c, is, iboxes[k] - 1, kappa_ins, kappa_dih, Ec[k], rng);
  }
  for (int k = 0; k < nboxes; ++k) {
    double wsum = 0.0;
    int64_t nov = 0;
    for (int64_t i = 0; i < n_ins; ++i) {
      const InsertionOut& o = res[(size_t)k * n_ins + i];
      if (o.overlap) ++nov;
      else wsum += o.widom_var;
      if (trace) {
        CassWidomTrace& tr = trace[(size_t)k * n_ins + i];
        tr.widom_var = o.overlap ? 0.0 : o.widom_var;
        tr.ln_pbias = o.ln_pbias;
        tr.e_inter = o.e_inter;
        tr.e_first_trial_sum = o.first_trial_sum;
        tr.e_inter_abs = o.e_inter_abs;
        tr.selected_trial = o.selected;
        tr.overlap = o.overlap;
      }
    }
    out[k].widom_sum = wsum * prefactor[k];
    out[k].prefactor = prefactor[k];
    out[k].n_insertions = n_ins;
    out[k].n_overlaps = nov;
    out[k].n_trials = n_ins * (int64_t)(kappa_ins + (s.nfrag - 1) * kappa_dih);
  }
  return CASS_OK;
}

// Compute_Molecule_Nonbond_Inter_Energy_Widom for each trial position
int orc_atom_intra_energies(orc_ctx* c, int32_t ibox1, int32_t is1, int32_t ia, int32_t ntrial, const double* xyz,
                            const int32_t* exist, int32_t cbmc, double* e, int32_t* overlap) {
  if (check_ctx(c) || ibox1 < 1 || ibox1 > c->nboxes || is1 < 1 || is1 > c->nspecies || ntrial < 0 ||
      (ntrial > 0 && (!xyz || !e || !overlap)))
    return fail(CASS_EINVAL, "bad atom intra arguments");
  const Species& s = c->sp[is1 - 1];
  if (!s.defined) return fail(CASS_ESTATE, "species not defined");
  if (s.natoms > 32) return fail(CASS_ECAPACITY, "at most 32 atoms per molecule");
  if (ia < 1 || ia > s.natoms) return fail(CASS_EINVAL, "atom index out of range");
  std::vector<char> ex(s.natoms, 1);
  if (exist)
    for (int a = 0; a < s.natoms; ++a) ex[a] = exist[a] ? 1 : 0;
  for (int k = 0; k < ntrial; ++k) {
    double eiv, eiq, eoq;
    const bool ov = atom_intra_energy(c, c->box[ibox1 - 1], is1 - 1, ia - 1, xyz + (size_t)k * s.natoms * 3, ex.data(),
                                      cbmc != 0, eiv, eiq, eoq);
    overlap[k] = ov ? 1 : 0;
    e[3 * k] = ov ? 0.0 : eiv;
    e[3 * k + 1] = ov ? 0.0 : eiq;
    e[3 * k + 2] = ov ? 0.0 : eoq;
  }
  return CASS_OK;
}

int orc_cbmc_trial_energies(orc_ctx* c, int32_t ibox1, int32_t is1, int32_t skip_im, int32_t nat, const int32_t* atoms,
                            int32_t ntrial, const double* xyz, int32_t cbmc, double* e, int32_t* overlap) {
  if (c) refresh_members(c);
  if (check_ctx(c) || ibox1 < 1 || ibox1 > c->nboxes || is1 < 1 || is1 > c->nspecies || nat < 1 || !atoms ||
      ntrial < 0 || (ntrial > 0 && (!xyz || !e || !overlap)))
    return fail(CASS_EINVAL, "bad trial arguments");
  const Species& s = c->sp[is1 - 1];
  if (!s.defined) return fail(CASS_ESTATE, "species not defined");
  if (cbmc)
    if (int rc = cbmc_ready(c)) return rc;
  for (int a = 0; a < nat; ++a)
    if (atoms[a] < 1 || atoms[a] > s.natoms) return fail(CASS_EINVAL, "trial atom index out of range");
  if (skip_im < 0 || skip_im > c->max_mol[is1 - 1]) return fail(CASS_EINVAL, "molecule locate out of range");
  const int skip = skip_im > 0 ? c->mol_base[is1 - 1] + skip_im - 1 : -1;
  for (int k = 0; k < ntrial; ++k) {
    TestMol t;
    t.is = is1 - 1;
    t.r.assign(3 * s.natoms, 0.0);
    t.exist.assign(s.natoms, 0);
    for (int a = 0; a < nat; ++a) {
      const int ia = atoms[a] - 1;
      for (int d = 0; d < 3; ++d) t.r[3 * ia + d] = xyz[((size_t)k * nat + a) * 3 + d];
      t.exist[ia] = 1;
    }
    get_com(c, t.is, t.r.data(), t.exist.data(), t.com);
    t.max_dcom = max_com_distance(c, t.is, t.r.data(), t.exist.data(), t.com);
    double ev, eq;
    const bool ov = mol_inter_energy(c, ibox1 - 1, t.view(), skip, cbmc != 0, ev, eq);
    overlap[k] = ov ? 1 : 0;
    e[k] = ov ? 0.0 : ev + eq;
  }
  return CASS_OK;
}

// NVT translate / rotate Monte Carlo, one chain per box (boxes in parallel)
int orc_mc_sweeps(orc_ctx* c, int32_t nboxes, const int32_t* iboxes, const CassMCParams* p, double* max_disp,
                  double* max_rot, uint64_t seed, CassMCResult* out) {
  if (c) refresh_members(c);
  if (check_ctx(c) || nboxes < 1 || !iboxes || !p || !max_disp || !max_rot || !out || p->nsweeps < 0 ||
      p->steps_per_sweep < 0 || p->nupdate < 0 || !(p->target_accept > 0.0))
    return fail(CASS_EINVAL, "bad mc arguments");
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    if (ib < 0 || ib >= c->nboxes) return fail(CASS_EINVAL, "box index");
    for (int j = 0; j < k; ++j)
      if (iboxes[j] == iboxes[k]) return fail(CASS_EINVAL, "box listed twice");
    if (!c->box[ib].energy_valid) return fail(CASS_ESTATE, "system energy of box not computed");
  }
  std::vector<int> errs(nboxes, CASS_OK);
  std::vector<std::string> msgs(nboxes);
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    McChain ch;
    ch.c = c;
    ch.ibox = ib;
    ch.p = p;
    ch.max_disp = max_disp + (size_t)k * c->nspecies;
    ch.max_rot = max_rot + (size_t)k * c->nspecies;
    ch.rng = seed_stream(seed, iboxes[k], 0);
    ch.E = c->box[ib].energy;
    ch.nt_disp.assign(c->nspecies, 0);
    ch.ns_disp.assign(c->nspecies, 0);
    ch.nt_rot.assign(c->nspecies, 0);
    ch.ns_rot.assign(c->nspecies, 0);
    ch.run();
    c->box[ib].energy = ch.E;
    out[k] = ch.res;
    errs[k] = ch.err;
    if (ch.err) msgs[k] = g_err;
  }
  for (int k = 0; k < nboxes; ++k)
    if (errs[k]) return fail(errs[k], msgs[k]);
  return CASS_OK;
}

// Grand-canonical Monte Carlo, one chain per box (boxes in parallel)
// Build_Molecule for one molecule (the cass_build_molecule entry point): a
// not-live molecule grown anew in a scratch record, or the old-weight pass of
// a live one, whose stored coordinates are left as they were
int orc_build_molecule(orc_ctx* c, int32_t im, int32_t is1, int32_t ibox1, int32_t del_flag, int32_t kappa_ins,
                       int32_t kappa_dih, uint64_t* rng_state, int32_t* frag_order, double* ln_pseq, double* ln_pbias,
                       double* xyz, int32_t* cbmc_overlap) {
  if (c) refresh_members(c);
  if (check_ctx(c) || is1 < 1 || is1 > c->nspecies || ibox1 < 1 || ibox1 > c->nboxes || kappa_ins < 1 || !rng_state ||
      !ln_pseq || !ln_pbias || !cbmc_overlap)
    return fail(CASS_EINVAL, "bad build_molecule arguments");
  const int is = is1 - 1, ib = ibox1 - 1;
  const Species& s = c->sp[is];
  if (!s.defined || s.nfrag < 1) return fail(CASS_ESTATE, "species not defined or without fragments");
  if (im < 1 || im > c->max_mol[is]) return fail(CASS_EINVAL, "molecule index out of range");
  if (s.nfrag > 1 && kappa_dih < 1) return fail(CASS_EINVAL, "kappa_dih must be >= 1");
  if (c->box[ib].charge_style != CASS_CHARGE_NONE && c->box[ib].charge_sum_style != CASS_QQ_EWALD)
    return fail(CASS_EUNSUPPORTED, "build_molecule: charges need the Ewald sum");
  if (int rc = cbmc_ready(c)) return rc;
  const int slot = c->mol_base[is] + im - 1;
  const Mol& live = c->mol[slot];
  if (del_flag && !(live.live && live.ibox == ib)) return fail(CASS_ESTATE, "del_flag: the molecule is not live in the box");
  if (!del_flag && live.live) return fail(CASS_ESTATE, "the molecule to grow is live");
  Mol m;
  if (del_flag) {
    m = live;
  } else {
    m.is = is;
    m.ibox = ib;
    m.r.assign(3 * s.natoms, 0.0);
    m.exist.assign(s.natoms, 0);
  }
  Rng rng;
  for (int k = 0; k < 5; ++k) rng.s[k] = (int64_t)rng_state[k];
  std::vector<int> order;
  double lp = 0.0, lb = 0.0;
  const bool ov = build_molecule(c, ib, m, slot, del_flag != 0, kappa_ins, kappa_dih, lp, lb, rng, &order);
  for (int k = 0; k < 5; ++k) rng_state[k] = (uint64_t)rng.s[k];
  *ln_pseq = lp;
  *ln_pbias = lb;
  *cbmc_overlap = ov ? 1 : 0;
  if (frag_order)
    for (int k = 0; k < s.nfrag; ++k) frag_order[k] = k < (int)order.size() ? order[k] + 1 : 0;
  if (xyz)
    for (int k = 0; k < 3 * s.natoms; ++k) xyz[k] = del_flag ? live.r[k] : m.r[k];
  return CASS_OK;
}

int orc_gcmc(orc_ctx* c, int32_t nboxes, const int32_t* iboxes, const CassGCMCParams* p, const double* mu,
             const double* max_disp, const double* max_rot, uint64_t seed, CassGCMCResult* out) {
  if (c) refresh_members(c);
  if (check_ctx(c) || nboxes < 1 || !iboxes || !p || !mu || !max_disp || !max_rot || !out || p->nsteps < 0 ||
      p->is_exchange < 1 || p->is_exchange > c->nspecies || p->kappa_ins < 1)
    return fail(CASS_EINVAL, "bad gcmc arguments");
  const int is = p->is_exchange - 1;
  const Species& s = c->sp[is];
  if (!s.defined || s.nfrag < 1) return fail(CASS_ESTATE, "exchanged species not defined or without fragments");
  if (int rc = cbmc_ready(c)) return rc;
  if (s.nfrag > 1 && p->kappa_dih < 1) return fail(CASS_EINVAL, "kappa_dih must be >= 1");
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    if (ib < 0 || ib >= c->nboxes) return fail(CASS_EINVAL, "box index");
    for (int j = 0; j < k; ++j)
      if (iboxes[j] == iboxes[k]) return fail(CASS_EINVAL, "box listed twice");
    if (!c->box[ib].energy_valid) return fail(CASS_ESTATE, "system energy of box not computed");
    if (c->box[ib].charge_style != CASS_CHARGE_NONE && c->box[ib].charge_sum_style != CASS_QQ_EWALD)
      return fail(CASS_EUNSUPPORTED, "gcmc: charges need the Ewald sum");
  }
  // free slots of the exchanged species, in ascending order, each to the box
  // holding the fewest atoms so far (live molecules of every species plus the
  // slots dealt; ties to the first listed box): the boxes' shares even out
  std::vector<std::vector<int>> pools(nboxes);
  {
    std::vector<long long> load(nboxes, 0);
    for (int k = 0; k < nboxes; ++k)
      for (int slot = 0; slot < (int)c->mol.size(); ++slot)
        if (c->mol[slot].live && c->mol[slot].ibox == iboxes[k] - 1) load[k] += c->sp[c->mol[slot].is].natoms;
    for (int im = 0; im < c->max_mol[is]; ++im) {
      const int slot = c->mol_base[is] + im;
      if (c->mol[slot].live) continue;
      int kmin = 0;
      for (int k = 1; k < nboxes; ++k)
        if (load[k] < load[kmin]) kmin = k;
      pools[kmin].push_back(slot);
      load[kmin] += c->sp[is].natoms;
    }
  }
  // fragment bonds (f, g), f < g, and prob_del1 (input_routines.f90:3035-3120)
  std::vector<int> fa, fb;
  std::vector<double> pd1;
  for (int f = 0; f < s.nfrag; ++f)
    for (int g : s.frag_connect[f])
      if (g > f) {
        fa.push_back(f);
        fb.push_back(g);
        int ndel[2];
        for (int side = 0; side < 2; ++side) {
          const int f1 = side ? g : f, f2 = side ? f : g;
          std::vector<int> live(s.nfrag, 0), order{f1};
          live[f2] = 1;
          live[f1] = 1;
          // every fragment reached from f1 without crossing f2 (the set Fragment_Order visits)
          for (size_t q = 0; q < order.size(); ++q)
            for (int h : s.frag_connect[order[q]])
              if (!live[h]) {
                live[h] = 1;
                order.push_back(h);
              }
          ndel[side] = 0;
          for (int h : order) ndel[side] += (int)s.frag_atoms[h].size() - 2;
        }
        pd1.push_back((double)ndel[1] / (double)(ndel[0] + ndel[1]));
      }
  double mw = 0.0;
  for (double m : s.mass) mw += m;
  std::vector<int> errs(nboxes, CASS_OK);
  std::vector<std::string> msgs(nboxes);
  std::vector<double> md((size_t)nboxes * c->nspecies), mr((size_t)nboxes * c->nspecies);
  std::copy(max_disp, max_disp + md.size(), md.begin());
  std::copy(max_rot, max_rot + mr.size(), mr.begin());
  CassMCParams mp{};
  mp.nupdate = 0;
  mp.target_accept = 0.5;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < nboxes; ++k) {
    const int ib = iboxes[k] - 1;
    const Box& b = c->box[ib];
    GcmcChain g;
    g.mc.c = c;
    g.mc.ibox = ib;
    g.mc.p = &mp;
    g.mc.max_disp = md.data() + (size_t)k * c->nspecies;
    g.mc.max_rot = mr.data() + (size_t)k * c->nspecies;
    g.mc.rng = seed_stream(seed, iboxes[k], 0);
    g.mc.E = b.energy;
    g.mc.nt_disp.assign(c->nspecies, 0);
    g.mc.ns_disp.assign(c->nspecies, 0);
    g.mc.nt_rot.assign(c->nspecies, 0);
    g.mc.ns_rot.assign(c->nspecies, 0);
    g.is = is;
    g.gp = p;
    g.mu = mu[k] / ATOMIC_TO_KJMOL;
    g.log_lambda3 = 3.0 * std::log(H_PLANK * std::sqrt(b.beta / (TWOPI * mw)));
    g.pool = pools[k];
    g.frag_bond_a = fa;
    g.frag_bond_b = fb;
    g.prob_del1 = pd1;
    g.run();
    c->box[ib].energy = g.mc.E;
    out[k] = g.res;
    errs[k] = g.mc.err;
    if (g.mc.err) msgs[k] = g_err;
  }
  for (int k = 0; k < nboxes; ++k)
    if (errs[k]) return fail(errs[k], msgs[k]);
  return CASS_OK;
}

// Raw lfsr258 stream of (seed, box, insertion), for RNG parity tests.
int orc_rng_stream(uint64_t seed, int64_t ibox, int64_t ins, int32_t n, double* outv) {
  Rng r = seed_stream(seed, ibox, ins);
  for (int k = 0; k < n; ++k) outv[k] = r.next();
  return CASS_OK;
}

// Reference-seeded stream: init_seeds(i1, i3) for one thread
// (random_generators.f90:51-91) followed by n rranf() draws.
int orc_rng_reference(int64_t i1, int64_t i3, int32_t n, double* outv) {
  Rng r;
  r.s[0] = i1;
  r.s[1] = -759022222;
  r.s[2] = i3;
  r.s[3] = -1718083407;
  r.s[4] = -123456789;
  if ((r.s[0] & -2LL) == 0) r.s[0] = i1 - 8388607LL;
  if ((r.s[2] & -4096LL) == 0) r.s[2] = i3 - 8388607LL;
  for (int k = 0; k < n; ++k) outv[k] = r.next();
  return CASS_OK;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// threads of the OpenMP regions that follow (n < 1: all the host's processors)
int orc_set_num_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n >= 1 ? n : omp_get_num_procs());
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // extern "C"
