// k_grad.cu -- adjoint of the box energy: dU/dr, dU/d(eps, sigma), dU/dq.
//
// The energy differentiated is the one cass_system_total_energy returns for
// LJ cut / cut_tail boxes with no charges or an Ewald sum (energy_routines.f90
// :2648-2953): intramolecular nonbond pairs with their scale factors and no
// periodic image (:980-1085), intermolecular LJ and real-space Ewald pairs
// under the minimum image (:1589-1730, :1831-2053, :2088-2166), the long-range
// correction (:2956-3023), the reciprocal sum (:4111-4231) and the self
// energy (:2553-2601).  The real-space term is differentiated through the
// Abramowitz-Stegun 7.1.26 erfc the energy uses, so the gradient is the exact
// derivative of the computed energy (away from cutoff crossings, where the
// truncated energy is discontinuous).  FP64 throughout.
//
//   k_grad_pairs  thread per atom i, a chunk of the atoms j per grid row in
//                 shared-memory tiles: the force on i, sum_j q_j dE/d(q_i q_j),
//                 and, for j > i, the per-type-pair parameter derivatives (each
//                 pair counted once); one partial per (chunk, i)
//   k_grad_recip  thread per atom i, a chunk of the k-vectors per grid row:
//                 2 CF q_i sum_k Cn k (S_s cos - S_c sin) and
//                 2 CF sum_k Cn (S_c cos + S_s sin); one partial per (chunk, i)
//   k_grad_reduce thread per atom: the chunks' partials added in chunk order
//   k_grad_types  fixed-order tree reduction of the per-atom parameter
//                 derivatives per type
// The chunks spread the FP64 work of a box of a few thousand atoms over every
// SM (a grid of atom blocks alone fills fewer SMs than GB300 has); the partial
// buffers keep every sum in a fixed order, so repeated calls give equal bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cass_ctx.h"
#include "cass_molecule.cuh"

namespace cassgpu {

constexpr int kGradBlock = 128;
constexpr int kGradPairVals = 4 + 2 * kMaxTypes;  // gx, gy, gz, dq, deps[t], dsig[t]
constexpr int kMaxAtomsGrad = 64;  // atoms of a molecule with bonded terms (k_grad_bonded's arrays)

// A&S 7.1.26: erfc(x) = t P(t) exp(-x^2), t = 1/(1+px); returns erfc and its
// derivative with respect to x
__device__ __forceinline__ void erfc_as_d(double x, double& f, double& df) {
  const double A1 = 0.254829592, A2 = -0.284496736, A3 = 1.421413741, A4 = -1.453152027, A5 = 1.061405429,
               P = 0.3275911;
  const double t = 1.0 / (1.0 + P * x);
  const double poly = A1 + t * (A2 + t * (A3 + t * (A4 + t * A5)));
  const double dpoly = A2 + t * (2.0 * A3 + t * (3.0 * A4 + t * 4.0 * A5));
  const double e = exp(-x * x);
  const double tp = t * poly;
  f = tp * e;
  // d(t poly)/dx = (poly + t dpoly) dt/dx, dt/dx = -P t^2
  df = e * ((poly + t * dpoly) * (-P * t * t) - 2.0 * x * tp);
}

struct GradAtom {
  double4_32a p;  // x, y, z, q
  int mol, type, species, atom;
};

// The vdW pair energy of Compute_AtomPair_Energy (energy_routines.f90:1907-2000)
// in the box's style, differentiated: dE/d(r^2), dE/d(eps) and dE/d(sigma) of
// a pair within its cutoff (scale: vdw_intra_scale or 1).  LJ: cut, cut_tail,
// cut_shift, cut_switch, cut_shift_force and minimum image; Mie: cut and
// cut_shift.  The forms follow vdw_pair term by term.
__device__ __forceinline__ void vdw_pair_grad(const PairTable& T, const BoxDev& b, int k, double r2, double vs,
                                              double& dEdr2, double& dEde, double& dEds) {
  const double eps = T.eps[k], sig2 = T.sig2[k], sig = sqrt(sig2);
  if (b.vdw_style == CASS_VDW_MIE) {
    const double r = sqrt(r2), n = T.mie_n[k], m = T.mie_m[k], cm = T.mie_c[k];
    const double sn = pow(sig / r, n), sm = pow(sig / r, m);
    double e = sn - sm, de_sig = n * sn - m * sm;
    if (b.vdw_sum_style == CASS_VDW_SUM_CUT_SHIFT) {
      const double cn = pow(sig / b.rcut_vdw, n), cmm = pow(sig / b.rcut_vdw, m);
      e -= cn - cmm;
      de_sig -= n * cn - m * cmm;
    }
    dEdr2 = cm * eps * vs * (-n * sn + m * sm) / (2.0 * r2);
    dEde = cm * vs * e;
    dEds = cm * eps * vs * de_sig / sig;
    return;
  }
  const double s2 = sig2 / r2, s6 = s2 * s2 * s2, s12 = s6 * s6;
  const double elj = 4.0 * (s12 - s6);                  // E / eps
  const double dlj_dr2 = 4.0 * (-6.0 * s12 + 3.0 * s6) / r2;  // d(E / eps) / d(r^2)
  const double dlj_ds = 4.0 * (12.0 * s12 - 6.0 * s6) / sig;  // d(E / eps) / d(sigma)
  double fe = elj, fr = dlj_dr2, fs = dlj_ds;  // the style's E / eps and its derivatives
  switch (b.vdw_sum_style) {
    case CASS_VDW_SUM_CUT_SHIFT: {
      const double c2 = sig2 / b.rcut_vdwsq, c6 = c2 * c2 * c2, c12 = c6 * c6;
      fe -= 4.0 * (c12 - c6);
      fs -= 4.0 * (12.0 * c12 - 6.0 * c6) / sig;
      break;
    }
    case CASS_VDW_SUM_CUT_SWITCH:
      if (r2 >= b.ron_switch_sq) {  // E = S(r^2) E_LJ, S = d^2 (f2 + 2 r^2) f1, d = roff^2 - r^2
        const double d = b.roff_switch_sq - r2;
        const double S = d * d * (b.switch_factor2 + 2.0 * r2) * b.switch_factor1;
        const double dS = 2.0 * b.switch_factor1 * d * (d - (b.switch_factor2 + 2.0 * r2));
        fr = dS * elj + S * dlj_dr2;
        fe = S * elj;
        fs = S * dlj_ds;
      }
      break;
    case CASS_VDW_SUM_CUT_SHIFT_FORCE: {  // E - E(rc) - (r - rc) dE/dr(rc)
      const double c2 = sig2 / b.rcut_vdwsq, c6 = c2 * c2 * c2, c12 = c6 * c6, rc = b.rcut_vdw, r = sqrt(r2);
      const double g = -24.0 * (2.0 * c12 / rc - c6 / rc);  // dE/dr(rc) / eps
      fe = elj - 4.0 * (c12 - c6) - (r - rc) * g;
      fr = dlj_dr2 - g / (2.0 * r);
      fs = dlj_ds - 4.0 * (12.0 * c12 - 6.0 * c6) / sig + (r - rc) * 24.0 * (24.0 * c12 - 6.0 * c6) / (rc * sig);
      break;
    }
    default:
      break;
  }
  dEdr2 = eps * vs * fr;
  dEde = vs * fe;
  dEds = eps * vs * fs;
}

// d cos(phi) / d r of the dihedral angle of dihedral_cos_d (atoms a[0..3]):
// cos phi = m.n / (|m||n|), m = r12 x r32, n = r32 x r34 (r12 = r1 - r2,
// r32 = r3 - r2, r34 = r3 - r4); returns cos phi, adds scale * d cos / d r_k
// to g[3 a[k] ...]
__device__ inline double dihedral_cos_grad(const double* r, const int* a, double scale, double* g, bool add) {
  double r12[3], r32[3], r34[3];
  for (int d = 0; d < 3; ++d) {
    r12[d] = r[3 * a[0] + d] - r[3 * a[1] + d];
    r32[d] = r[3 * a[2] + d] - r[3 * a[1] + d];
    r34[d] = r[3 * a[2] + d] - r[3 * a[3] + d];
  }
  const double m[3] = {r12[1] * r32[2] - r32[1] * r12[2], -r12[0] * r32[2] + r12[2] * r32[0],
                       r12[0] * r32[1] - r12[1] * r32[0]};
  const double nv[3] = {r32[1] * r34[2] - r32[2] * r34[1], -r32[0] * r34[2] + r32[2] * r34[0],
                        r32[0] * r34[1] - r32[1] * r34[0]};
  const double mm = m[0] * m[0] + m[1] * m[1] + m[2] * m[2], nn = nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2];
  const double inv = 1.0 / sqrt(mm * nn);
  const double cphi = (m[0] * nv[0] + m[1] * nv[1] + m[2] * nv[2]) * inv;
  if (!add) return cphi;
  double gm[3], gn[3];  // d cos / d m, d cos / d n
  for (int d = 0; d < 3; ++d) {
    gm[d] = nv[d] * inv - cphi * m[d] / mm;
    gn[d] = m[d] * inv - cphi * nv[d] / nn;
  }
  // m = r12 x r32: d/d r12 = r32 x gm, d/d r32 = gm x r12; n = r32 x r34: d/d r32 = r34 x gn, d/d r34 = gn x r32
  const double d12[3] = {r32[1] * gm[2] - r32[2] * gm[1], r32[2] * gm[0] - r32[0] * gm[2], r32[0] * gm[1] - r32[1] * gm[0]};
  const double d32[3] = {gm[1] * r12[2] - gm[2] * r12[1] + r34[1] * gn[2] - r34[2] * gn[1],
                         gm[2] * r12[0] - gm[0] * r12[2] + r34[2] * gn[0] - r34[0] * gn[2],
                         gm[0] * r12[1] - gm[1] * r12[0] + r34[0] * gn[1] - r34[1] * gn[0]};
  const double d34[3] = {gn[1] * r32[2] - gn[2] * r32[1], gn[2] * r32[0] - gn[0] * r32[2], gn[0] * r32[1] - gn[1] * r32[0]};
  for (int d = 0; d < 3; ++d) {
    g[3 * a[0] + d] += scale * d12[d];
    g[3 * a[1] + d] += scale * (-d12[d] - d32[d]);
    g[3 * a[2] + d] += scale * (d32[d] + d34[d]);
    g[3 * a[3] + d] -= scale * d34[d];
  }
  return cphi;
}

// dU/dr of the bonded terms of Compute_Molecule_{Bond,Angle,Dihedral,Improper}_
// Energy (energy_routines.f90:197-496), as molecule_intra forms them: harmonic
// bonds k (l - l0)^2, harmonic angles k (theta - theta0)^2 with cos theta held
// within +-0.999999 (flat beyond), Ryckaert-Bellemans dihedrals sum c_j cos^j
// phi and harmonic impropers k (phi - phi0)^2.  One thread per molecule, added
// to the molecule's atoms of grad (packed order).
__global__ void k_grad_bonded(SpeciesPools P, const int4* __restrict__ molinfo, int nm,
                              const double4_32a* __restrict__ p64, double* grad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nm) return;
  const int4 mi = molinfo[q];  // slot, species, first atom, atoms
  const SpeciesDevHdr& h = P.hdr[mi.y];
  if (h.nbonds + h.nangles + h.ndih + h.nimp == 0) return;
  const int* ip = P.ip;
  const double* dp = P.dp;
  const int n = mi.w;
  double r[3 * kMaxAtomsGrad], g[3 * kMaxAtomsGrad];
  for (int a = 0; a < n; ++a) {
    const double4_32a p = p64[mi.z + a];
    r[3 * a] = p.x;
    r[3 * a + 1] = p.y;
    r[3 * a + 2] = p.z;
    g[3 * a] = g[3 * a + 1] = g[3 * a + 2] = 0.0;
  }
  for (int k = 0; k < h.nbonds; ++k) {
    if (ip[h.bond_kind_off + k] != CASS_BONDED_HARMONIC) continue;
    const int a = ip[h.bond_atoms_off + 2 * k], c = ip[h.bond_atoms_off + 2 * k + 1];
    const double dx = r[3 * a] - r[3 * c], dy = r[3 * a + 1] - r[3 * c + 1], dz = r[3 * a + 2] - r[3 * c + 2];
    const double l = sqrt(dx * dx + dy * dy + dz * dz), l0 = dp[h.bond_param_off + 2 * k + 1];
    const double f = 2.0 * dp[h.bond_param_off + 2 * k] * (l - l0) / l;
    g[3 * a] += f * dx;
    g[3 * a + 1] += f * dy;
    g[3 * a + 2] += f * dz;
    g[3 * c] -= f * dx;
    g[3 * c + 1] -= f * dy;
    g[3 * c + 2] -= f * dz;
  }
  for (int k = 0; k < h.nangles; ++k) {
    if (ip[h.angle_kind_off + k] != CASS_BONDED_HARMONIC) continue;
    const int a1 = ip[h.angle_atoms_off + 3 * k], a2 = ip[h.angle_atoms_off + 3 * k + 1],
              a3 = ip[h.angle_atoms_off + 3 * k + 2];
    double v21[3], v32[3];
    for (int d = 0; d < 3; ++d) {
      v21[d] = r[3 * a2 + d] - r[3 * a1 + d];
      v32[d] = r[3 * a3 + d] - r[3 * a2 + d];
    }
    const double C23 = v21[0] * v32[0] + v21[1] * v32[1] + v21[2] * v32[2];
    const double C22 = v21[0] * v21[0] + v21[1] * v21[1] + v21[2] * v21[2];
    const double C33 = v32[0] * v32[0] + v32[1] * v32[1] + v32[2] * v32[2];
    const double ct = C23 * (1.0 / sqrt(C33 * C22));
    if (ct >= 0.999999 || ct <= -0.999999) continue;  // the clamp: theta is constant there
    const double th = kPI - acos(ct), t0 = dp[h.angle_param_off + 2 * k + 1];
    // dE/dcos = 2 k (theta - theta0) dtheta/dcos, dtheta/dcos = 1 / sqrt(1 - cos^2)
    const double f = 2.0 * dp[h.angle_param_off + 2 * k] * (th - t0) / sqrt(1.0 - ct * ct);
    const double inv = 1.0 / sqrt(C22 * C33);
    for (int d = 0; d < 3; ++d) {
      const double d21 = v32[d] * inv - ct * v21[d] / C22;  // dcos / d v21
      const double d32 = v21[d] * inv - ct * v32[d] / C33;  // dcos / d v32
      g[3 * a1 + d] -= f * d21;
      g[3 * a2 + d] += f * (d21 - d32);
      g[3 * a3 + d] += f * d32;
    }
  }
  for (int k = 0; k < h.ndih; ++k) {
    const int* a = ip + h.dih_atoms_off + 4 * k;
    const double* c = dp + h.dih_rb_off + 6 * k;
    const double cp = dihedral_cos_grad(r, a, 0.0, g, false);
    double dEdc = 0.0, pw = 1.0;  // sum_j j c_j cos^(j-1)
    for (int j = 1; j < 6; ++j) {
      dEdc += j * c[j] * pw;
      pw *= cp;
    }
    dihedral_cos_grad(r, a, dEdc, g, true);
  }
  for (int k = 0; k < h.nimp; ++k) {
    const int* a = ip + h.imp_atoms_off + 4 * k;
    const double cp = dihedral_cos_grad(r, a, 0.0, g, false);
    if (cp >= 1.0 || cp <= -1.0) continue;
    double n34[3];
    double r12[3], r32[3], r34[3];
    for (int d = 0; d < 3; ++d) {
      r12[d] = r[3 * a[0] + d] - r[3 * a[1] + d];
      r32[d] = r[3 * a[2] + d] - r[3 * a[1] + d];
      r34[d] = r[3 * a[2] + d] - r[3 * a[3] + d];
    }
    n34[0] = r32[1] * r34[2] - r32[2] * r34[1];
    n34[1] = -r32[0] * r34[2] + r32[2] * r34[0];
    n34[2] = r32[0] * r34[1] - r32[1] * r34[0];
    const double sgn = (r12[0] * n34[0] + r12[1] * n34[1] + r12[2] * n34[2]) < 0.0 ? -1.0 : 1.0;
    const double phi = sgn * acos(cp), p0 = dp[h.imp_param_off + 2 * k + 1];
    // dE/dcos = 2 k (phi - phi0) dphi/dcos, dphi/dcos = -sgn / sqrt(1 - cos^2)
    const double dEdc = 2.0 * dp[h.imp_param_off + 2 * k] * (phi - p0) * (-sgn / sqrt(1.0 - cp * cp));
    dihedral_cos_grad(r, a, dEdc, g, true);
  }
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) grad[3 * (size_t)(mi.z + a) + d] += g[3 * a + d];
}

// pre2: an FP32 bound on r^2 beyond every cutoff of the box (with a margin far
// above FP32 rounding of the coordinates): pairs beyond it are skipped before
// the FP64 arithmetic, which then decides every cutoff exactly
__global__ void __launch_bounds__(kGradBlock) k_grad_pairs(BoxDev b, PairTable T, SpeciesPools P,
                                                           const double4_32a* __restrict__ p64,
                                                           const float4* __restrict__ p32,
                                                           const int4* __restrict__ meta, int n, int jchunk,
                                                           float pre2, double* part, int* ovflag) {
  __shared__ double4_32a sp[kGradBlock];
  __shared__ float4 spf[kGradBlock];
  __shared__ int4 sm[kGradBlock];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < n;
  const double4_32a pi = live ? p64[i] : make_double4_32a(0, 0, 0, 0);
  const float4 pif = live ? p32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int4 mi = live ? meta[i] : make_int4(-1, -1, -1, -1);
  const bool vdw = b.vdw_style == CASS_VDW_LJ || b.vdw_style == CASS_VDW_MIE;
  const bool coul = b.charge_style == CASS_CHARGE_COUL;
  double gx = 0, gy = 0, gz = 0, dqi = 0;
  double de[kMaxTypes], ds[kMaxTypes];
#pragma unroll
  for (int t = 0; t < kMaxTypes; ++t) de[t] = ds[t] = 0.0;
  bool ov = false;
  const SpeciesDevHdr* hi = live ? &P.hdr[mi.z] : nullptr;
  const int jbeg = blockIdx.y * jchunk, jend = min(n, jbeg + jchunk);
  for (int j0 = jbeg; j0 < jend; j0 += kGradBlock) {
    __syncthreads();
    if (j0 + threadIdx.x < jend) {
      sp[threadIdx.x] = p64[j0 + threadIdx.x];
      spf[threadIdx.x] = p32[j0 + threadIdx.x];
      sm[threadIdx.x] = meta[j0 + threadIdx.x];
    }
    __syncthreads();
    if (!live) continue;
    const int cnt = min(kGradBlock, jend - j0);
    for (int k = 0; k < cnt; ++k) {
      const int j = j0 + k;
      if (j == i) continue;
      {
        const float4 q = spf[k];
        const float ex = fold(pif.x - q.x, b.hLf[0], b.Lf[0]), ey = fold(pif.y - q.y, b.hLf[1], b.Lf[1]),
                    ez = fold(pif.z - q.z, b.hLf[2], b.Lf[2]);
        if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > pre2) continue;
      }
      const double4_32a pj = sp[k];
      const int4 mj = sm[k];
      const bool intra = mj.x == mi.x;
      double dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      double vs = 1.0, qs = 1.0;
      if (intra) {  // Compute_Molecule_Nonbond_Intra_Energy: no periodic image
        const int na = hi->natoms;
        vs = P.dp[hi->vs_off + mi.w * na + mj.w];
        qs = P.dp[hi->qs_off + mi.w * na + mj.w];
      } else {
        dx = fold(dx, b.hL[0], b.L[0]);
        dy = fold(dy, b.hL[1], b.L[1]);
        dz = fold(dz, b.hL[2], b.L[2]);
      }
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (intra) {
        if (r2 <= b.rcut_lowsq && !P.ip[hi->bonded_off + mi.w * hi->natoms + mj.w]) ov = true;
      } else if (r2 < b.rcut_lowsq) {
        ov = true;
      }
      double dEdr2 = 0.0;  // dE/d(r^2) of this pair
      if (vdw && (cutoff_mask(b, r2, false) & 1) && mi.y >= 0 && mj.y >= 0) {
        const int kk = pidx(mi.y, mj.y, T.ntypes);
        if (T.eps[kk] != 0.0 && vs != 0.0) {
          double er, ee, es;
          vdw_pair_grad(T, b, kk, r2, vs, er, ee, es);
          dEdr2 += er;
          if (j > i) {
            de[mj.y] += ee;
            ds[mj.y] += es;
          }
        }
      }
      // Ewald real space: inter q q CF erfc(ar)/r; intra q q CF (qscale - erf(ar))/r
      if (coul && r2 <= b.rcut_coulsq) {
        const double r = sqrt(r2);
        double f, df;
        erfc_as_d(b.alpha * r, f, df);
        const double g = intra ? (qs - (1.0 - f)) : f;  // erf = 1 - erfc
        const double phi = kCHARGE_FACTOR * g / r;      // dE/d(q_i q_j)
        const double dphi_dr = kCHARGE_FACTOR * (b.alpha * df / r - g / r2);
        dqi += pj.w * phi;
        dEdr2 += pi.w * pj.w * dphi_dr / (2.0 * r);
      }
      gx += 2.0 * dEdr2 * dx;
      gy += 2.0 * dEdr2 * dy;
      gz += 2.0 * dEdr2 * dz;
    }
  }
  if (!live) return;
  if (ov) atomicOr(ovflag, 1);
  // partial of (chunk, i): component-major so that the reduction reads coalesced
  const size_t stride = (size_t)gridDim.y * n;
  double* o = part + (size_t)blockIdx.y * n + i;
  o[0] = gx;
  o[stride] = gy;
  o[2 * stride] = gz;
  o[3 * stride] = dqi;
#pragma unroll
  for (int t = 0; t < kMaxTypes; ++t) {
    o[(4 + t) * stride] = de[t];
    o[(4 + kMaxTypes + t) * stride] = ds[t];
  }
}

// The k-vectors come in rows of equal (ny, nz) with nx = n0, n0+1, ... (the
// loop order of Ewald_Reciprocal_Lattice_Vector_Setup, energy_routines.f90:
// 2260-2311), so along a row the phase advances by the factor e^{i 2 pi x / Lx}:
// one complex product per k-vector, a sincos at the start of each row.
__global__ void __launch_bounds__(kGradBlock) k_grad_recip(const double4_32a* __restrict__ kvec,
                                                           const double* __restrict__ cos_sum,
                                                           const double* __restrict__ sin_sum, int nv, int kchunk,
                                                           double hx1, const double4_32a* __restrict__ p64, int n,
                                                           double* part) {
  __shared__ double4_32a sk[kGradBlock];
  __shared__ double2 ss[kGradBlock];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < n;
  const double4_32a pi = live ? p64[i] : make_double4_32a(0, 0, 0, 0);
  double gx = 0, gy = 0, gz = 0, dqi = 0;
  const int kbeg = blockIdx.y * kchunk, kend = min(nv, kbeg + kchunk);
  double us, uc;  // e^{i hx1 x}
  sincos(hx1 * pi.x, &us, &uc);
  double c = 1.0, s = 0.0, py = 0.0, pz = 0.0, pxh = 0.0;
  bool have = false;
  for (int k0 = kbeg; k0 < kend; k0 += kGradBlock) {
    __syncthreads();
    if (k0 + threadIdx.x < kend) {
      sk[threadIdx.x] = kvec[k0 + threadIdx.x];
      ss[threadIdx.x] = make_double2(cos_sum[k0 + threadIdx.x], sin_sum[k0 + threadIdx.x]);
    }
    __syncthreads();
    if (!live) continue;
    const int cnt = min(kGradBlock, kend - k0);
    for (int k = 0; k < cnt; ++k) {
      const double4_32a h = sk[k];
      if (have && h.y == py && h.z == pz && fabs(h.x - (pxh + hx1)) <= 1e-9 * fabs(hx1)) {
        const double c1 = c * uc - s * us;  // next nx of the row
        s = s * uc + c * us;
        c = c1;
      } else {
        sincos(h.x * pi.x + h.y * pi.y + h.z * pi.z, &s, &c);
        py = h.y;
        pz = h.z;
        have = true;
      }
      pxh = h.x;
      const double w = h.w * (ss[k].y * c - ss[k].x * s);
      gx += w * h.x;
      gy += w * h.y;
      gz += w * h.z;
      dqi += h.w * (ss[k].x * c + ss[k].y * s);
    }
  }
  if (!live) return;
  const size_t stride = (size_t)gridDim.y * n;
  double* o = part + (size_t)blockIdx.y * n + i;
  o[0] = gx;
  o[stride] = gy;
  o[2 * stride] = gz;
  o[3 * stride] = dqi;
}

// the chunks' partials of atom i added in chunk order: the pair terms, then
// 2 CF q_i times the reciprocal sums (no reciprocal part when nkc = 0)
__global__ void k_grad_reduce(const double* __restrict__ ppart, int npc, const double* __restrict__ rpart, int nkc,
                              const double4_32a* __restrict__ p64, int n, double* grad, double* dq,
                              double* deps_atom, double* dsig_atom) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t ps = (size_t)npc * n;
  double v[kGradPairVals];
#pragma unroll
  for (int c = 0; c < kGradPairVals; ++c) {
    double a = 0.0;
    for (int k = 0; k < npc; ++k) a += ppart[c * ps + (size_t)k * n + i];
    v[c] = a;
  }
  if (nkc > 0) {
    const size_t rs = (size_t)nkc * n;
    double r[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      double a = 0.0;
      for (int k = 0; k < nkc; ++k) a += rpart[c * rs + (size_t)k * n + i];
      r[c] = a;
    }
    const double f = 2.0 * kCHARGE_FACTOR, qi = p64[i].w;
    v[0] += f * qi * r[0];
    v[1] += f * qi * r[1];
    v[2] += f * qi * r[2];
    v[3] += f * r[3];
  }
  grad[3 * i] = v[0];
  grad[3 * i + 1] = v[1];
  grad[3 * i + 2] = v[2];
  dq[i] = v[3];
#pragma unroll
  for (int t = 0; t < kMaxTypes; ++t) {
    deps_atom[(size_t)i * kMaxTypes + t] = v[4 + t];
    dsig_atom[(size_t)i * kMaxTypes + t] = v[4 + kMaxTypes + t];
  }
}

constexpr int kTypeBlock = 256;

// out[ti*kMaxTypes+tj] = sum over atoms of type ti of the per-atom values: one
// block per type, each thread a fixed stride of atoms, then a fixed tree
__global__ void __launch_bounds__(kTypeBlock) k_grad_types(const int4* __restrict__ meta, int n,
                                                           const double* __restrict__ deps_atom,
                                                           const double* __restrict__ dsig_atom, double* out_eps,
                                                           double* out_sig) {
  __shared__ double se[kTypeBlock][kMaxTypes + 1], ssg[kTypeBlock][kMaxTypes + 1];
  const int ti = blockIdx.x;
  double e[kMaxTypes], s[kMaxTypes];
#pragma unroll
  for (int t = 0; t < kMaxTypes; ++t) e[t] = s[t] = 0.0;
  for (int i = threadIdx.x; i < n; i += kTypeBlock) {
    if (meta[i].y != ti) continue;
#pragma unroll
    for (int t = 0; t < kMaxTypes; ++t) {
      e[t] += deps_atom[(size_t)i * kMaxTypes + t];
      s[t] += dsig_atom[(size_t)i * kMaxTypes + t];
    }
  }
#pragma unroll
  for (int t = 0; t < kMaxTypes; ++t) {
    se[threadIdx.x][t] = e[t];
    ssg[threadIdx.x][t] = s[t];
  }
  __syncthreads();
  for (int h = kTypeBlock / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
#pragma unroll
      for (int t = 0; t < kMaxTypes; ++t) {
        se[threadIdx.x][t] += se[threadIdx.x + h][t];
        ssg[threadIdx.x][t] += ssg[threadIdx.x + h][t];
      }
    __syncthreads();
  }
  if (threadIdx.x < kMaxTypes) {
    out_eps[ti * kMaxTypes + threadIdx.x] = se[0][threadIdx.x];
    out_sig[ti * kMaxTypes + threadIdx.x] = ssg[0][threadIdx.x];
  }
}

int pack_box_ext(cass_ctx* c, int ibox);
const std::vector<int>& members_ext(cass_ctx* c, int ibox);
int ensure_pools(cass_ctx* c);

}  // namespace cassgpu

using namespace cassgpu;

extern "C" int cass_system_total_energy(cass_ctx* c, int32_t ibox, int32_t intra_flag, CassEnergy* out,
                                        int32_t* overlap);

extern "C" int cass_system_gradient(cass_ctx* c, int32_t ibox1, CassEnergy* energy, double* dU_dr, double* dU_deps,
                                    double* dU_dsig, double* dU_dq) {
  if (!c || ibox1 < 1 || ibox1 > c->nboxes) return set_error(CASS_EINVAL, "bad arguments");
  const int ib = ibox1 - 1;
  BoxH& B = c->box[ib];
  if (!B.defined) return set_error(CASS_ESTATE, "box not defined");
  const CassBoxDesc& d = B.desc;
  if (d.vdw_style == CASS_VDW_LJ && d.vdw_sum_style == CASS_VDW_SUM_CHARMM)
    return set_error(CASS_EUNSUPPORTED, "gradient: LJ CHARMM (molecule-pair cutoff) is not differentiated");
  if (d.vdw_style == CASS_VDW_MIE && d.vdw_sum_style != CASS_VDW_SUM_CUT && d.vdw_sum_style != CASS_VDW_SUM_CUT_SHIFT)
    return set_error(CASS_EUNSUPPORTED, "gradient: Mie with cut or cut_shift only");
  if (d.charge_style == CASS_CHARGE_COUL && d.charge_sum_style != CASS_QQ_EWALD)
    return set_error(CASS_EUNSUPPORTED, "gradient: charges need the Ewald sum");
  bool flexible = false;  // harmonic or torsional terms: their gradient runs too
  for (int is = 0; is < c->nspecies; ++is) {
    const SpeciesH& s = c->sp[is];
    if (!s.defined) continue;
    bool flex = !s.dih_atoms.empty() || !s.imp_atoms.empty();
    for (int k : s.bond_kind) flex = flex || k == CASS_BONDED_HARMONIC;
    for (int k : s.angle_kind) flex = flex || k == CASS_BONDED_HARMONIC;
    if (flex && s.natoms > kMaxAtomsGrad)
      return set_error(CASS_ECAPACITY, "gradient: a species with bonded terms has more than 64 atoms");
    flexible = flexible || flex;
  }
  // energy, packed atoms and structure factors of the current configuration
  CassEnergy E;
  int32_t ov = 0;
  int rc = cass_system_total_energy(c, ibox1, 1, &E, &ov);
  if (rc) return rc;
  if (ov) return set_error(CASS_ESTATE, "gradient: the configuration has a core overlap");
  if (energy) *energy = E;
  const int n = B.npacked;
  const int nt = c->ntypes;
  // chunks of j atoms / k-vectors per grid row: about four CTAs per SM in all
  int dev_sms = 0;
  CASS_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  const int nb = std::max(1, (n + kGradBlock - 1) / kGradBlock);
  const int want_rows = std::max(1, (4 * dev_sms + nb - 1) / nb);
  auto chunking = [&](int total, int& rows) {  // chunk length, a multiple of the tile
    rows = std::max(1, std::min(want_rows, (total + kGradBlock - 1) / kGradBlock));
    int len = (total + rows - 1) / rows;
    len = ((len + kGradBlock - 1) / kGradBlock) * kGradBlock;
    rows = std::max(1, (total + len - 1) / len);
    return len;
  };
  int npc = 1, nkc = 0;
  const int jchunk = n > 0 ? chunking(n, npc) : 1;
  const bool recip = d.charge_style == CASS_CHARGE_COUL && B.nvecs > 0;
  int kchunk = 1;
  if (recip) kchunk = chunking(B.nvecs, nkc);
  const size_t bytes = (size_t)n * (3 + 1 + 2 * kMaxTypes) * sizeof(double) + 2 * kMaxTypes * kMaxTypes * sizeof(double) +
                       (size_t)n * ((size_t)npc * kGradPairVals + (size_t)nkc * 4) * sizeof(double) + 64;
  if ((rc = c->d_grad.reserve(bytes))) return rc;
  double* d_g = c->d_grad.as<double>();
  double* d_dq = d_g + 3 * (size_t)n;
  double* d_de = d_dq + n;
  double* d_ds = d_de + (size_t)n * kMaxTypes;
  double* d_te = d_ds + (size_t)n * kMaxTypes;
  double* d_ts = d_te + kMaxTypes * kMaxTypes;
  double* d_pp = d_ts + kMaxTypes * kMaxTypes;
  double* d_rp = d_pp + (size_t)n * npc * kGradPairVals;
  if ((rc = c->d_query.reserve(16))) return rc;
  CASS_CUDA(cudaMemsetAsync(c->d_query.p, 0, sizeof(int), c->stream));
  if (n > 0) {
    // beyond every cutoff the kernel tests: pairs past it add nothing
    double rmax2 = 0.0;
    if (d.vdw_style != CASS_VDW_NONE) {
      if (d.vdw_sum_style == CASS_VDW_SUM_MINIMUM) rmax2 = 1.0e30;  // every pair within the minimum image
      else if (d.vdw_sum_style == CASS_VDW_SUM_CUT_SWITCH) rmax2 = std::max(rmax2, B.dev.roff_switch_sq);
      else rmax2 = std::max(rmax2, B.dev.rcut_vdwsq);
    }
    if (d.charge_style == CASS_CHARGE_COUL) rmax2 = std::max(rmax2, B.dev.rcut_coulsq);
    rmax2 = std::max(rmax2, B.dev.rcut_lowsq);
    const float pre2 = (float)(rmax2 * (1.0 + 1.0e-4) + 1.0e-3);
    k_grad_pairs<<<dim3(nb, npc), kGradBlock, 0, c->stream>>>(B.dev, c->pt, c->pools, B.d_p64.as<double4_32a>(),
                                                              B.d_p32.as<float4>(), B.d_meta.as<int4>(), n, jchunk,
                                                              pre2, d_pp, c->d_query.as<int>());
    CASS_CUDA(cudaGetLastError());
    count_launch(c);
    if (recip) {
      k_grad_recip<<<dim3(nb, nkc), kGradBlock, 0, c->stream>>>(B.d_kvec.as<double4_32a>(), B.d_cos_sum.as<double>(),
                                                                B.d_sin_sum.as<double>(), B.nvecs, kchunk,
                                                                kTWOPI / B.dev.L[0], B.d_p64.as<double4_32a>(), n, d_rp);
      CASS_CUDA(cudaGetLastError());
      count_launch(c);
    }
    k_grad_reduce<<<nb, kGradBlock, 0, c->stream>>>(d_pp, npc, d_rp, recip ? nkc : 0, B.d_p64.as<double4_32a>(), n, d_g,
                                                    d_dq, d_de, d_ds);
    CASS_CUDA(cudaGetLastError());
    count_launch(c);
    k_grad_types<<<kMaxTypes, kTypeBlock, 0, c->stream>>>(B.d_meta.as<int4>(), n, d_de, d_ds, d_te, d_ts);
    CASS_CUDA(cudaGetLastError());
    count_launch(c);
    if (flexible && B.npacked_mols > 0) {
      k_grad_bonded<<<(B.npacked_mols + 127) / 128, 128, 0, c->stream>>>(c->pools, B.d_molinfo.as<int4>(),
                                                                          B.npacked_mols, B.d_p64.as<double4_32a>(), d_g);
      CASS_CUDA(cudaGetLastError());
      count_launch(c);
    }
  }
  std::vector<double> g(3 * (size_t)n), q(n), te(kMaxTypes * kMaxTypes, 0.0), ts(kMaxTypes * kMaxTypes, 0.0);
  int hov = 0;
  if (n > 0) {
    CASS_CUDA(d2h(c, g.data(), d_g, g.size() * sizeof(double)));
    CASS_CUDA(d2h(c, q.data(), d_dq, q.size() * sizeof(double)));
    CASS_CUDA(d2h(c, te.data(), d_te, te.size() * sizeof(double)));
    CASS_CUDA(d2h(c, ts.data(), d_ts, ts.size() * sizeof(double)));
  }
  CASS_CUDA(d2h(c, &hov, c->d_query.p, sizeof(int)));
  CASS_CUDA(cudaStreamSynchronize(c->stream));
  if (hov) return set_error(CASS_ESTATE, "gradient: the configuration has a core overlap");
  // the packed order is species-major, locate order: the order of dU_dr
  if (dU_dr) memcpy(dU_dr, g.data(), g.size() * sizeof(double));
  if (dU_dq) {
    std::vector<int> off(c->nspecies + 1, 0);
    for (int is = 0; is < c->nspecies; ++is) off[is + 1] = off[is] + (c->sp[is].defined ? c->sp[is].natoms : 0);
    for (int k = 0; k < off[c->nspecies]; ++k) dU_dq[k] = 0.0;
    // d/dq_i of the self energy -CF alpha/sqrt(pi) sum q^2 (energy_routines.f90:2594)
    const bool ew = d.charge_style == CASS_CHARGE_COUL;
    for (size_t m = 0; m < B.pk_mol.size(); ++m) {
      const int slot = B.pk_mol[m], is = c->slot_sp[slot];
      const SpeciesH& s = c->sp[is];
      for (int a = 0; a < s.natoms; ++a) {
        double v = q[B.pk_mol_off[m] + a];
        if (ew) v += -2.0 * kCHARGE_FACTOR * B.dev.alpha / kROOTPI * s.q[a];
        dU_dq[off[is] + a] += v;
      }
    }
  }
  // the symmetric pair parameters: a pair of types (t, u) enters once per pair
  // of atoms; the long-range correction adds
  // 2 pi / V sum_t sum_u N_t N_u 4 eps_tu (sigma^12/(9 rc^9) - sigma^6/(3 rc^3))
  if (dU_deps || dU_dsig) {
    std::vector<double> nb(nt, 0.0);
    for (int slot : members_ext(c, ib)) {
      const SpeciesH& s = c->sp[c->slot_sp[slot]];
      for (int a = 0; a < s.natoms; ++a)
        if (s.type[a] >= 0) nb[s.type[a]] += 1.0;
    }
    const bool tail = d.vdw_style == CASS_VDW_LJ && d.vdw_sum_style == CASS_VDW_SUM_CUT_TAIL;
    for (int t = 0; t < nt; ++t)
      for (int u = 0; u < nt; ++u) {
        double e = te[t * kMaxTypes + u] + (t != u ? te[u * kMaxTypes + t] : 0.0);
        double s = ts[t * kMaxTypes + u] + (t != u ? ts[u * kMaxTypes + t] : 0.0);
        if (tail) {
          const double sig = std::sqrt(c->pt.sig2[pidx(t, u, nt)]), eps = c->pt.eps[pidx(t, u, nt)];
          const double mult = (t != u ? 2.0 : 1.0) * 2.0 * kPI / B.dev.volume * nb[t] * nb[u];
          const double s3 = sig * sig * sig, s6 = s3 * s3;
          e += mult * 4.0 * (s6 * s6 / (9.0 * B.rcut9) - s6 / (3.0 * B.rcut3));
          s += mult * 4.0 * eps * (12.0 * s6 * s6 / sig / (9.0 * B.rcut9) - 6.0 * s6 / sig / (3.0 * B.rcut3));
        }
        if (dU_deps) dU_deps[t * nt + u] = e;
        if (dU_dsig) dU_dsig[t * nt + u] = s;
      }
  }
  return CASS_OK;
}
