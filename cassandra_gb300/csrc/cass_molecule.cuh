// cass_molecule.cuh -- device species tables and whole-molecule energies
// shared by the energy kernels and the Widom kernel.
#pragma once

#include "cass_device.cuh"

namespace cassgpu {

// ---------------------------------------------------------------------------
// device species table (flexible sizes via offsets into two pools)
struct SpeciesDevHdr {
  int natoms, has_charge, l_coul_cbmc;
  int type_off, bonded_off;          // int pool
  int q_off, mass_off, vs_off, qs_off;  // double pool
  int nbonds, bond_atoms_off, bond_kind_off, bond_param_off;
  int nangles, angle_atoms_off, angle_kind_off, angle_param_off;
  int ndih, dih_atoms_off, dih_rb_off;
  int nimp, imp_atoms_off, imp_param_off;
};

struct SpeciesPools {
  const SpeciesDevHdr* hdr;
  const int* ip;
  const double* dp;
};

// ---------------------------------------------------------------------------
// Bonded and intramolecular nonbond energies of one molecule (FP64):
// Compute_Molecule_{Bond,Angle,Dihedral,Improper}_Energy (energy_routines.f90:197-496)
// and Compute_Molecule_Nonbond_Intra_Energy (:980-1085).
__device__ inline double dihedral_cos_d(const double* r, int a1, int a2, int a3, int a4) {
  double rx12 = r[3 * a1] - r[3 * a2], ry12 = r[3 * a1 + 1] - r[3 * a2 + 1], rz12 = r[3 * a1 + 2] - r[3 * a2 + 2];
  double rx32 = r[3 * a3] - r[3 * a2], ry32 = r[3 * a3 + 1] - r[3 * a2 + 1], rz32 = r[3 * a3 + 2] - r[3 * a2 + 2];
  double rx34 = r[3 * a3] - r[3 * a4], ry34 = r[3 * a3 + 1] - r[3 * a4 + 1], rz34 = r[3 * a3 + 2] - r[3 * a4 + 2];
  double mx = ry12 * rz32 - ry32 * rz12, my = -rx12 * rz32 + rz12 * rx32, mz = rx12 * ry32 - ry12 * rx32;
  double nx = ry32 * rz34 - rz32 * ry34, ny = -rx32 * rz34 + rz32 * rx34, nz = rx32 * ry34 - ry32 * rx34;
  double msq = mx * mx + my * my + mz * mz, nsq = nx * nx + ny * ny + nz * nz, mdn = mx * nx + my * ny + mz * nz;
  return mdn / sqrt(msq * nsq);
}

struct IntraOut {
  double bond, angle, dih, imp, ivdw, iqq, pqq;
  bool overlap;
};

// cbmc: Check_AtomPair_Cutoff with rcut_cbmc, and no charge pairs when the
// species' L_Coul_CBMC is set (energy_routines.f90:1062-1064; the opposite sense
// of the intermolecular rule of :1684-1686, kept as the reference has it)
__device__ inline IntraOut molecule_intra(const SpeciesPools& P, int is, const BoxDev& b, const PairTable& t,
                                   const double* r, bool cbmc = false) {
  const SpeciesDevHdr& h = P.hdr[is];
  IntraOut o{0, 0, 0, 0, 0, 0, 0, false};
  const int* ip = P.ip;
  const double* dp = P.dp;
  for (int k = 0; k < h.nbonds; ++k) {
    if (ip[h.bond_kind_off + k] != CASS_BONDED_HARMONIC) continue;
    int a = ip[h.bond_atoms_off + 2 * k], c = ip[h.bond_atoms_off + 2 * k + 1];
    double dx = r[3 * a] - r[3 * c], dy = r[3 * a + 1] - r[3 * c + 1], dz = r[3 * a + 2] - r[3 * c + 2];
    double l = sqrt(dx * dx + dy * dy + dz * dz), l0 = dp[h.bond_param_off + 2 * k + 1];
    o.bond += dp[h.bond_param_off + 2 * k] * (l - l0) * (l - l0);
  }
  for (int k = 0; k < h.nangles; ++k) {
    if (ip[h.angle_kind_off + k] != CASS_BONDED_HARMONIC) continue;
    int a1 = ip[h.angle_atoms_off + 3 * k], a2 = ip[h.angle_atoms_off + 3 * k + 1], a3 = ip[h.angle_atoms_off + 3 * k + 2];
    double rx21 = r[3 * a2] - r[3 * a1], ry21 = r[3 * a2 + 1] - r[3 * a1 + 1], rz21 = r[3 * a2 + 2] - r[3 * a1 + 2];
    double rx32 = r[3 * a3] - r[3 * a2], ry32 = r[3 * a3 + 1] - r[3 * a2 + 1], rz32 = r[3 * a3 + 2] - r[3 * a2 + 2];
    double C23 = rx21 * rx32 + ry21 * ry32 + rz21 * rz32, C22 = rx21 * rx21 + ry21 * ry21 + rz21 * rz21,
           C33 = rx32 * rx32 + ry32 * ry32 + rz32 * rz32;
    double ct = C23 * (1.0 / sqrt(C33 * C22));
    ct = fmin(ct, 0.999999);
    ct = fmax(ct, -0.999999);
    double th = kPI - acos(ct), t0 = dp[h.angle_param_off + 2 * k + 1];
    o.angle += dp[h.angle_param_off + 2 * k] * (th - t0) * (th - t0);
  }
  for (int k = 0; k < h.ndih; ++k) {
    const int* a = ip + h.dih_atoms_off + 4 * k;
    double c1 = dihedral_cos_d(r, a[0], a[1], a[2], a[3]);
    double cv[6] = {1.0, c1, c1 * c1, 0, 0, 0};
    cv[3] = cv[1] * cv[2];
    cv[4] = cv[2] * cv[2];
    cv[5] = cv[2] * cv[3];
    double d = 0;
    for (int j = 0; j < 6; ++j) d += cv[j] * dp[h.dih_rb_off + 6 * k + j];
    o.dih += d;
  }
  for (int k = 0; k < h.nimp; ++k) {
    const int* a = ip + h.imp_atoms_off + 4 * k;
    double rx12 = r[3 * a[0]] - r[3 * a[1]], ry12 = r[3 * a[0] + 1] - r[3 * a[1] + 1], rz12 = r[3 * a[0] + 2] - r[3 * a[1] + 2];
    double rx32 = r[3 * a[2]] - r[3 * a[1]], ry32 = r[3 * a[2] + 1] - r[3 * a[1] + 1], rz32 = r[3 * a[2] + 2] - r[3 * a[1] + 2];
    double rx34 = r[3 * a[2]] - r[3 * a[3]], ry34 = r[3 * a[2] + 1] - r[3 * a[3] + 1], rz34 = r[3 * a[2] + 2] - r[3 * a[3] + 2];
    double mx = ry12 * rz32 - ry32 * rz12, my = -rx12 * rz32 + rz12 * rx32, mz = rx12 * ry32 - ry12 * rx32;
    double nx = ry32 * rz34 - rz32 * ry34, ny = -rx32 * rz34 + rz32 * rx34, nz = rx32 * ry34 - ry32 * rx34;
    double cp = (mx * nx + my * ny + mz * nz) / sqrt((mx * mx + my * my + mz * mz) * (nx * nx + ny * ny + nz * nz));
    cp = fmin(1.0, fmax(-1.0, cp));
    double phi = copysign(acos(cp), rx12 * nx + ry12 * ny + rz12 * nz);
    double p0 = dp[h.imp_param_off + 2 * k + 1];
    o.imp += dp[h.imp_param_off + 2 * k] * (phi - p0) * (phi - p0);
  }
  int n = h.natoms;
  for (int ia = 0; ia < n; ++ia) {
    for (int ja = ia + 1; ja < n; ++ja) {
      double dx = r[3 * ia] - r[3 * ja], dy = r[3 * ia + 1] - r[3 * ja + 1], dz = r[3 * ia + 2] - r[3 * ja + 2];
      double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 <= b.rcut_lowsq && !ip[h.bonded_off + ia * n + ja]) {
        o.overlap = true;
        return o;
      }
      int m = cutoff_mask(b, r2, cbmc);
      if (cbmc && h.l_coul_cbmc) m &= ~2;
      if (m & 1) o.ivdw += vdw_pair(t, b, ip[h.type_off + ia], ip[h.type_off + ja], r2, dp[h.vs_off + ia * n + ja]);
      if (m & 2)
        o.iqq += qq_pair_intra(b, dp[h.q_off + ia] * dp[h.q_off + ja], r2, dp[h.qs_off + ia * n + ja], &o.pqq);
    }
  }
  return o;
}

}  // namespace cassgpu
