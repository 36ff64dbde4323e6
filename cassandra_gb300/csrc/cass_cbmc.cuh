// cass_cbmc.cuh -- CBMC growth tables and FP64 geometry shared by the Widom
// and grand-canonical kernels (fragment_growth.f90, get_com.f90).
#pragma once

#include "cass_molecule.cuh"

namespace cassgpu {

// Tables of the grown species: fragments, connectivity, libraries and the
// insertion probabilities (Fragment_Info / Fragment_Connectivity, .mcf).
struct WidomSpecies {
  int natoms, nfrag, is0;
  int kappa_ins, kappa_dih;
  int want_qq_cbmc;  // Coulomb in CBMC trials (L_Coul_CBMC)
  double ln_kappa_ins, ln_kappa_dih_term;
  double mass[kMaxAtoms];
  double q[kMaxAtoms];
  int type[kMaxAtoms];
  int frag_natoms[kMaxFrags];
  signed char frag_atoms[kMaxFrags][kMaxAtoms];
  int frag_nconnect[kMaxFrags];
  signed char frag_connect[kMaxFrags][kMaxFrags];
  int nconfig[kMaxFrags];
  long long lib_off[kMaxFrags];
  double prob_ins[kMaxFrags], cum_prob_ins[kMaxFrags], ln_prob_ins[kMaxFrags];
};

// ---------------------------------------------------------------------------
// test-molecule helpers (FP64)

__device__ __forceinline__ void get_com(const WidomSpecies& S, const double* r, unsigned exist, double com[3]) {
  double tm = 0, x = 0, y = 0, z = 0;
  for (int k = 0; k < S.natoms; ++k) {
    if (!((exist >> k) & 1u)) continue;
    double m = S.mass[k];
    tm += m;
    x += m * r[3 * k];
    y += m * r[3 * k + 1];
    z += m * r[3 * k + 2];
  }
  com[0] = x / tm;
  com[1] = y / tm;
  com[2] = z / tm;
}

// Get_Aligner_Hanger (fragment_growth.f90:2135-2185), row-major
__device__ inline void aligner_hanger(double v1[3], double v2[3], double al[9], double hg[9]) {
  double n1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  for (int i = 0; i < 3; ++i) v1[i] = v1[i] / n1;
  double n2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  for (int i = 0; i < 3; ++i) v2[i] = v2[i] / n2;
  double p1[3] = {v1[1] * v2[2] - v1[2] * v2[1], -v1[0] * v2[2] + v1[2] * v2[0], v1[0] * v2[1] - v1[1] * v2[0]};
  double np1 = sqrt(p1[0] * p1[0] + p1[1] * p1[1] + p1[2] * p1[2]);
  for (int i = 0; i < 3; ++i) p1[i] = p1[i] / np1;
  double p2[3] = {v1[1] * p1[2] - v1[2] * p1[1], -v1[0] * p1[2] + v1[2] * p1[0], v1[0] * p1[1] - v1[1] * p1[0]};
  double np2 = sqrt(p2[0] * p2[0] + p2[1] * p2[1] + p2[2] * p2[2]);
  for (int i = 0; i < 3; ++i) p2[i] = p2[i] / np2;
  for (int i = 0; i < 3; ++i) {
    al[i] = v1[i];
    al[3 + i] = p2[i];
    al[6 + i] = p1[i];
    hg[i * 3 + 0] = v1[i];
    hg[i * 3 + 1] = p2[i];
    hg[i * 3 + 2] = p1[i];
  }
}

// Compute_Molecule_Dihedral_Energy over dihedrals whose atoms all exist (RB form)
__device__ inline double dihedral_masked(const SpeciesDevHdr& H, const SpeciesPools& P, const double* r, unsigned exist) {
  double e = 0.0;
  for (int k = 0; k < H.ndih; ++k) {
    const int* a = P.ip + H.dih_atoms_off + 4 * k;
    unsigned m = (1u << a[0]) | (1u << a[1]) | (1u << a[2]) | (1u << a[3]);
    if ((exist & m) != m) continue;
    double c1 = dihedral_cos_d(r, a[0], a[1], a[2], a[3]);
    double cv[6] = {1.0, c1, c1 * c1, 0, 0, 0};
    cv[3] = cv[1] * cv[2];
    cv[4] = cv[2] * cv[2];
    cv[5] = cv[2] * cv[3];
    double d = 0;
    for (int j = 0; j < 6; ++j) d += cv[j] * P.dp[H.dih_rb_off + 6 * k + j];
    e += d;
  }
  return e;
}

// Compute_Atom_Nonbond_Intra_Energy (energy_routines.f90:691-737), CBMC cutoffs
__device__ inline bool atom_intra(const SpeciesDevHdr& H, const SpeciesPools& P, const BoxDev& b, const PairTable& T, int ia,
                           const double* r, unsigned exist, double& eiv, double& eiq, double& eoq, bool cbmc = true) {
  eiv = eiq = eoq = 0.0;
  int n = H.natoms;
  for (int ja = 0; ja < n; ++ja) {
    if (ja == ia || !((exist >> ja) & 1u)) continue;
    double vs = P.dp[H.vs_off + ia * n + ja], qs = P.dp[H.qs_off + ia * n + ja];
    bool nzv = vs > 0.0, nzq = qs > 0.0;
    if (!(nzv || nzq)) continue;
    double dx = r[3 * ja] - r[3 * ia], dy = r[3 * ja + 1] - r[3 * ia + 1], dz = r[3 * ja + 2] - r[3 * ia + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < b.rcut_lowsq && nzv) return true;
    int m = cutoff_mask(b, r2, cbmc);
    if (!nzv) m &= ~1;
    if (!nzq) m &= ~2;
    if (m & 1) eiv += vdw_pair(T, b, P.ip[H.type_off + ja], P.ip[H.type_off + ia], r2, P.dp[H.vs_off + ja * n + ia]);
    if (m & 2) {
      double per = 0.0;
      eiq += qq_pair_intra(b, P.dp[H.q_off + ja] * P.dp[H.q_off + ia], r2, P.dp[H.qs_off + ja * n + ia], &per);
      eoq += per;
    }
  }
  return false;
}

}  // namespace cassgpu
