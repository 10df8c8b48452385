// Enhanced-assumed-strain Q1 hexahedra (sm_103a): the element kernel template, included by element_eas.cu
// (NeoHooke, StVenantKirchhoff, BlatzKo) and element_eas_hyper.cu (the hyperelastic framework).
//
// Reference: EnhancedAssumedStrains (ikarus/finiteelements/mechanics/enhancedassumedstrains.hh:225-434) with
// the strain functions easfunctions/{greenlagrangestrain,displacementgradient,displacementgradienttransposed}.hh
// and the ansatz spaces easvariants/{linearandglstrains,displacementgradient,helperfunctions}.hh.
//
// Same decomposition as the displacement kernel: 8 lanes per element, lane = node I.  Per Gauss point the
// lanes share F, S and the Voigt tangent C (each lane computes a few of its 36 entries into shared memory),
// and each lane computes the enhanced-strain columns E_alpha(:,k) and C E_alpha(:,k) for k = I, I+8, ...
// After the Gauss loop the element's D (n_alpha x n_alpha) is LU-factorised once per element (lane 0,
// partial pivoting, FP64); every lane solves for its own D^{-1} L_I, and the condensed quantities
//   f_I -= L_I^T D^{-1} R~,   K_IJ -= L_I^T D^{-1} L_J        (enhancedassumedstrains.hh:291-296, 336-345)
// are formed with the same 5-blocks-per-lane ownership as the displacement kernel.
// D^{-1} R~ and D^{-1} L are cached per element (FP64) when the residual is assembled, so the internal-state
// update alpha -= D^{-1} (R~ + L dd) (enhancedassumedstrains.hh:225-248) costs one pass over the cache.
//
// The enhancement modes are rank one.  H9: H_p = s_p a_r (x) a_c with p = 3r + c, s_p = (detJ0/detJ)(2 xi_c - 1)
// and a_k the k-th column of J0^{-T} (easvariants/displacementgradient.hh:136-161, helperfunctions.hh:27-36).
// Every enhanced-strain quantity is therefore written through (v, coef) with column i of the mode's
// displacement-gradient matrix equal to coef_i v:  H: v = a_r, coef = s a_c;   H9T (F_c0 H_p^T): v = F_c0 a_c,
// coef = s a_r.  GL (E9/E21): E_alpha(:,k) = (T0^{-1} / detJ) M0(:,k) with one nonzero per M0 column.
#pragma once
#include <cmath>

#include "common.cuh"
#include "hyperelastic.cuh"
#include "kernels.h"

namespace ikr {

namespace {

// E9 / E21 ansatz (easvariants/linearandglstrains.hh:252-327): column k has its single entry in row kRow[k],
// equal to the product of (2 xi_f - 1) over the listed factors (second factor -1 = none).
__constant__ int kRow[21] = {0, 1, 2, 3, 3, 4, 4, 5, 5, 3, 3, 4, 4, 5, 5, 0, 0, 1, 1, 2, 2};
__constant__ int kF1[21] = {0, 1, 2, 1, 2, 0, 2, 0, 1, 0, 0, 0, 1, 0, 1, 0, 0, 0, 1, 0, 1};
__constant__ int kF2[21] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, 1, 2, 1, 2, 2, 2, 1, 2, 1, 2, 2, 2};

template <int NA>
struct EasCfg {
  static constexpr int EPB = NA <= 9 ? 8 : 4;  // elements per 64/32-thread block
  static constexpr int NT = NA * (NA + 1) / 2; // packed upper triangle of D
  static constexpr int DSH = (NT + 7) / 8;     // D entries per lane
  static constexpr int RSH = (NA + 7) / 8;     // R~ entries per lane
  // shared memory per element (doubles)
  static constexpr int O_DN = 0;               // 8 x 3   modified nodal gradients
  static constexpr int O_C6 = O_DN + 24;       // 36      Voigt tangent
  static constexpr int O_EA = O_C6 + 36;       // NA x 6  E_alpha columns
  static constexpr int O_CEA = O_EA + 6 * NA;  // NA x 6  C E_alpha columns
  static constexpr int O_GEO = O_CEA + 6 * NA; // 36      T0^{-1} (GL)
  static constexpr int O_D = O_GEO + 36;       // NA x NA
  static constexpr int O_RT = O_D + NA * NA;   // NA
  static constexpr int O_Y = O_RT + NA;        // 8 x NA x 3   D^{-1} L_I
  static constexpr int O_PIV = O_Y + 24 * NA;  // NA (pivot rows, stored as doubles)
  static constexpr int PER = O_PIV + NA;
};

__device__ __forceinline__ void packed_index(int t, int na, int& a, int& b) {
  a = 0;
  int rowlen = na;
  while (t >= rowlen) {
    t -= rowlen;
    ++a;
    --rowlen;
  }
  b = a + t;
}

// Voigt form of sym(F^T (coef (x) ... )) for a displacement-gradient variation whose column i is coef_i v:
// E[0] = coef0 g0, ..., E[3] = coef2 g1 + coef1 g2, with g_j = v . F(:,j)  (easfunctions/displacementgradient.hh:153-166)
__device__ __forceinline__ void sym_voigt(const double coef[3], const double v[3], const double F[3][3], double E[6]) {
  double g[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) g[j] = v[0] * F[0][j] + v[1] * F[1][j] + v[2] * F[2][j];
  E[0] = coef[0] * g[0];
  E[1] = coef[1] * g[1];
  E[2] = coef[2] * g[2];
  E[3] = coef[2] * g[1] + coef[1] * g[2];
  E[4] = coef[2] * g[0] + coef[0] * g[2];
  E[5] = coef[1] * g[0] + coef[0] * g[1];
}

// B-operator (6x3) of the Green-Lagrange strain variation, rows as in easfunctions/displacementgradient.hh:135-145
__device__ __forceinline__ void bop(const double F[3][3], const double dN[3], double B[6][3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double g0 = F[a][0], g1 = F[a][1], g2 = F[a][2];
    B[0][a] = dN[0] * g0;
    B[1][a] = dN[1] * g1;
    B[2][a] = dN[2] * g2;
    B[3][a] = dN[2] * g1 + dN[1] * g2;
    B[4][a] = dN[2] * g0 + dN[0] * g2;
    B[5][a] = dN[1] * g0 + dN[0] * g1;
  }
}

// HYP: the hyperelastic framework's material point (hyperelastic.cuh) instead of the closed-form laws
template <int NA, int KIND, int MODE, typename KT, bool HYP>
__global__ void __launch_bounds__(EasCfg<NA>::EPB * 8) eas_element_kernel(ElemArgs a, const int32_t* __restrict__ list,
                                                                           int n_list, int e_base) {
  using Cfg = EasCfg<NA>;
  constexpr bool WANT_R = MODE & kWantR;
  constexpr bool WANT_K = MODE & kWantK;
  constexpr bool ELEM_OUT = MODE & kElemOut;
  extern __shared__ double smem[];

  const int lane = threadIdx.x & 31;
  const int sub = threadIdx.x & 7;
  const int es = threadIdx.x >> 3;
  double* sm = smem + (size_t)es * Cfg::PER;
  const int li = blockIdx.x * Cfg::EPB + es;
  const bool active = li < n_list;
  const int lic = active ? li : n_list - 1;
  const int e = list ? list[lic] : e_base + lic;
  const int ne = a.n_elems;
  const int node = a.conn[sub * ne + e];
  const int src = lane & ~7;

  double dX[3], dU[3], Ud[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double x = a.X[3 * node + c];
    Ud[c] = a.u ? a.u[3 * node + c] : 0.0;
    dX[c] = x - __shfl_sync(0xffffffffu, x, src);
    dU[c] = Ud[c] - __shfl_sync(0xffffffffu, Ud[c], src);
  }
  double al[NA];
#pragma unroll
  for (int p = 0; p < NA; ++p) al[p] = a.alpha[(size_t)p * ne + e];

  // centre data
  double A0[3][3] = {}, detJ0 = 0.0, dN0[3] = {0, 0, 0}, Fc0[3][3] = {}, Fa[3][3] = {};
  if (KIND == 1) {
    for (int k = sub; k < 36; k += 8) sm[Cfg::O_GEO + k] = a.eas_geo[(size_t)k * ne + e];
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) A0[i][j] = a.eas_geo[(size_t)(3 * i + j) * ne + e];
    detJ0 = a.eas_geo[(size_t)9 * ne + e];
    if (KIND == 3) {
#pragma unroll
      for (int k = 0; k < 3; ++k) dN0[k] = a.eas_geo[(size_t)(10 + 3 * sub + k) * ne + e];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Fc0[i][j] = sum8(dU[i] * dN0[j]) + (i == j ? 1.0 : 0.0);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) Fa[i][c] = Fc0[i][0] * A0[0][c] + Fc0[i][1] * A0[1][c] + Fc0[i][2] * A0[2][c];
    }
  }
  __syncwarp();

  const double lam = a.lam_e ? a.lam_e[e] : a.lam, mu = a.mu_e ? a.mu_e[e] : a.mu;
  double f[3] = {0, 0, 0};
  double Kacc[5][3][3];
#pragma unroll
  for (int d = 0; d < 5; ++d)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Kacc[d][i][j] = 0.0;
  double Lacc[NA][3];
#pragma unroll
  for (int k = 0; k < NA; ++k) Lacc[k][0] = Lacc[k][1] = Lacc[k][2] = 0.0;
  double Dacc[Cfg::DSH], Racc[Cfg::RSH];
#pragma unroll
  for (int m = 0; m < Cfg::DSH; ++m) Dacc[m] = 0.0;
#pragma unroll
  for (int m = 0; m < Cfg::RSH; ++m) Racc[m] = 0.0;
  int bad = 0;

#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    const double xi[3] = {(q & 1) ? kGaussHi : kGaussLo, (q & 2) ? kGaussHi : kGaussLo, (q & 4) ? kGaussHi : kGaussLo};
    double dxi[3];
    ref_gradient_at_gp<double>(sub, q, dxi);
    double J[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) J[i][j] = sum8(dX[i] * dxi[j]);
    double Ji[3][3];
    const double detJ = inv3(J, Ji);
    double dN[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dN[k] = dxi[0] * Ji[0][k] + dxi[1] * Ji[1][k] + dxi[2] * Ji[2][k];
    double H[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) H[i][j] = sum8(dU[i] * dN[j]);

    // enhancement at this Gauss point
    double s[NA];  // H/HT mode scales, GL ansatz coefficients / detJ
    double Ht[3][3] = {};
    if (KIND == 1) {
#pragma unroll
      for (int k = 0; k < NA; ++k) {
        double v = 2.0 * xi[kF1[k]] - 1.0;
        if (kF2[k] >= 0) v *= 2.0 * xi[kF2[k]] - 1.0;
        s[k] = v / detJ;
      }
    } else {
      const double sc = detJ0 / detJ;
#pragma unroll
      for (int p = 0; p < NA; ++p) s[p] = sc * (2.0 * xi[p % 3] - 1.0);
#pragma unroll
      for (int p = 0; p < NA; ++p) {
        const int r = p / 3, c = p % 3;
        const double w = al[p] * s[p];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) Ht[i][j] += w * A0[i][r] * A0[j][c];
      }
      if (KIND == 2) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) H[i][j] += Ht[i][j];
      } else {  // H = Hc + Fc0 Ht^T (displacementgradienttransposed.hh:353-368)
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) H[i][j] += Fc0[i][0] * Ht[j][0] + Fc0[i][1] * Ht[j][1] + Fc0[i][2] * Ht[j][2];
      }
    }
    double F[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
    // Green-Lagrange strain (Voigt, doubled shears) plus the GL enhancement M alpha
    double Ev[6];
    {
      double E[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          E[i][j] = 0.5 * (H[i][j] + H[j][i] + H[0][i] * H[0][j] + H[1][i] * H[1][j] + H[2][i] * H[2][j]);
      Ev[0] = E[0][0], Ev[1] = E[1][1], Ev[2] = E[2][2];
      Ev[3] = 2.0 * E[1][2], Ev[4] = 2.0 * E[0][2], Ev[5] = 2.0 * E[0][1];
    }
    if (KIND == 1) {
#pragma unroll
      for (int k = 0; k < NA; ++k) {
        const double w = s[k] * al[k];
        const int rr = kRow[k];
#pragma unroll
        for (int r = 0; r < 6; ++r) Ev[r] += w * sm[Cfg::O_GEO + 6 * r + rr];
      }
    }
    double S[6], Sm[3][3];
    if constexpr (HYP) {
      // Hyperelastic<Deviatoric<DF>, Volumetric<VF>> on C = 2E + I (hyper::evaluate; moduli needed for D and L)
      double C[3][3];
      C[0][0] = 2.0 * Ev[0] + 1.0, C[1][1] = 2.0 * Ev[1] + 1.0, C[2][2] = 2.0 * Ev[2] + 1.0;
      C[1][2] = C[2][1] = Ev[3];
      C[0][2] = C[2][0] = Ev[4];
      C[0][1] = C[1][0] = Ev[5];
      hyper::Point pt;
      bad |= hyper::evaluate(a.hyper, C, pt, true);
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        const int i = voigt_a(v), j = voigt_b(v);
        S[v] = hyper::stress(pt, i, j);
        Sm[i][j] = Sm[j][i] = S[v];
      }
      for (int t = sub; t < 36; t += 8) {
        const int r = t / 6, c = t % 6;
        sm[Cfg::O_C6 + t] = hyper::modulus(pt, voigt_a(r), voigt_b(r), voigt_a(c), voigt_b(c));
      }
    } else if (a.material == 1) {
      // StVenantKirchhoff (svk.hh:96-163): S = lambda tr(E) + 2 mu E (Voigt shears mu * 2E_ij), constant moduli
      const double trE = Ev[0] + Ev[1] + Ev[2];
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        const int i = voigt_a(v), j = voigt_b(v);
        S[v] = v < 3 ? lam * trE + 2.0 * mu * Ev[v] : mu * Ev[v];
        Sm[i][j] = Sm[j][i] = S[v];
      }
      for (int t = sub; t < 36; t += 8) {
        const int r = t / 6, c = t % 6;
        sm[Cfg::O_C6 + t] = (r < 3 && c < 3 ? lam : 0.0) + (r == c ? (r < 3 ? 2.0 * mu : mu) : 0.0);
      }
    } else if (a.material == 2) {
      // BlatzKo on C = 2E + I: S = mu (J C^-1 - C^-2), moduli mu [J Ci_ij Ci_kl - J (Ci_ik Ci_jl + Ci_il Ci_jk)
      // + Ci_ik Ci2_jl + Ci_il Ci2_jk + Ci2_ik Ci_jl + Ci2_il Ci_jk] with Ci2 = C^-2
      double C[3][3], Ci[3][3], Ci2[3][3];
      C[0][0] = 2.0 * Ev[0] + 1.0, C[1][1] = 2.0 * Ev[1] + 1.0, C[2][2] = 2.0 * Ev[2] + 1.0;
      C[1][2] = C[2][1] = Ev[3];
      C[0][2] = C[2][0] = Ev[4];
      C[0][1] = C[1][0] = Ev[5];
      const double detC = inv3(C, Ci);
      if (!(detC > 1e-10)) bad |= kStatusNonPositiveDetC;
      const double Jd = sqrt(detC);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Ci2[i][j] = Ci[i][0] * Ci[0][j] + Ci[i][1] * Ci[1][j] + Ci[i][2] * Ci[2][j];
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        const int i = voigt_a(v), j = voigt_b(v);
        S[v] = mu * (Jd * Ci[i][j] - Ci2[i][j]);
        Sm[i][j] = Sm[j][i] = S[v];
      }
      for (int t = sub; t < 36; t += 8) {
        const int r = t / 6, c = t % 6;
        const int i = voigt_a(r), j = voigt_b(r), k = voigt_a(c), l = voigt_b(c);
        sm[Cfg::O_C6 + t] = mu * (Jd * Ci[i][j] * Ci[k][l] - Jd * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]) +
                                  Ci[i][k] * Ci2[j][l] + Ci[i][l] * Ci2[j][k] + Ci2[i][k] * Ci[j][l] +
                                  Ci2[i][l] * Ci[j][k]);
      }
    } else {
      // NeoHooke on C = 2E + I (neohooke.hh:100-142)
      double C[3][3], Ci[3][3];
      C[0][0] = 2.0 * Ev[0] + 1.0, C[1][1] = 2.0 * Ev[1] + 1.0, C[2][2] = 2.0 * Ev[2] + 1.0;
      C[1][2] = C[2][1] = Ev[3];
      C[0][2] = C[2][0] = Ev[4];
      C[0][1] = C[1][0] = Ev[5];
      const double detC = inv3(C, Ci);
      if (!(detC > 1e-10)) bad |= kStatusNonPositiveDetC;
      const double lnJ = log(sqrt(detC));
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        const int i = voigt_a(v), j = voigt_b(v);
        S[v] = mu * ((i == j ? 1.0 : 0.0) - Ci[i][j]) + lam * lnJ * Ci[i][j];
        Sm[i][j] = Sm[j][i] = S[v];
      }
      const double cc = mu - lam * lnJ;
      for (int t = sub; t < 36; t += 8) {
        const int r = t / 6, c = t % 6;
        const int i = voigt_a(r), j = voigt_b(r), k = voigt_a(c), l = voigt_b(c);
        sm[Cfg::O_C6 + t] = lam * Ci[i][j] * Ci[k][l] + cc * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]);
      }
    }
    // nodal gradients entering B and kg (HT adds Ht dN0, displacementgradienttransposed.hh:126-140)
    double dNm[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      dNm[k] = dN[k] + (KIND == 3 ? Ht[k][0] * dN0[0] + Ht[k][1] * dN0[1] + Ht[k][2] * dN0[2] : 0.0);
#pragma unroll
    for (int k = 0; k < 3; ++k) sm[Cfg::O_DN + 3 * sub + k] = dNm[k];
    const double w = kGaussW * detJ;
    double B[6][3];
    bop(F, dNm, B);
    if (WANT_R) {
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        double t = 0.0;
#pragma unroll
        for (int r = 0; r < 6; ++r) t += B[r][b] * S[r];
        f[b] += w * t;
      }
    }
    __syncwarp();  // C6 and dNm of all nodes are in shared memory

    double V[6][3];  // C B_I
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        double t = 0.0;
#pragma unroll
        for (int x = 0; x < 6; ++x) t += sm[Cfg::O_C6 + 6 * r + x] * B[x][b];
        V[r][b] = t;
      }
    if (WANT_K) {
      double SdN[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) SdN[i] = Sm[i][0] * dNm[0] + Sm[i][1] * dNm[1] + Sm[i][2] * dNm[2];
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int Jn = (sub + d) & 7;
        double dNJ[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) dNJ[k] = sm[Cfg::O_DN + 3 * Jn + k];
        double BJ[6][3];
        bop(F, dNJ, BJ);
        const double kg = SdN[0] * dNJ[0] + SdN[1] * dNJ[1] + SdN[2] * dNJ[2];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            double t = (i == j) ? kg : 0.0;
#pragma unroll
            for (int r = 0; r < 6; ++r) t += V[r][i] * BJ[r][j];
            Kacc[d][i][j] += w * t;
          }
      }
    }

    // enhanced-strain columns owned by this lane
    for (int k = sub; k < NA; k += 8) {
      double Ea[6];
      if (KIND == 1) {
#pragma unroll
        for (int r = 0; r < 6; ++r) Ea[r] = s[k] * sm[Cfg::O_GEO + 6 * r + kRow[k]];
      } else {
        const int r = k / 3, c = k % 3;
        double v[3], coef[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          v[i] = KIND == 2 ? A0[i][r] : Fa[i][c];
          coef[i] = s[k] * (KIND == 2 ? A0[i][c] : A0[i][r]);
        }
        sym_voigt(coef, v, F, Ea);
      }
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        sm[Cfg::O_EA + 6 * k + r] = Ea[r];
        double t = 0.0;
#pragma unroll
        for (int x = 0; x < 6; ++x) t += sm[Cfg::O_C6 + 6 * r + x] * Ea[x];
        sm[Cfg::O_CEA + 6 * k + r] = t;
      }
    }
    __syncwarp();
    // L_I(k, :) += (C E_alpha(:,k))^T B_I + E_alpha,d (enhancedassumedstrains.hh:401-408)
    double SdNm[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) SdNm[i] = Sm[i][0] * dNm[0] + Sm[i][1] * dNm[1] + Sm[i][2] * dNm[2];
#pragma unroll
    for (int k = 0; k < NA; ++k) {
      double t[3];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        double x = 0.0;
#pragma unroll
        for (int r = 0; r < 6; ++r) x += sm[Cfg::O_CEA + 6 * k + r] * B[r][b];
        t[b] = x;
      }
      if (KIND != 1) {
        const int r = k / 3, c = k % 3;
        double v[3], coef[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          v[i] = KIND == 2 ? A0[i][r] : Fa[i][c];
          coef[i] = s[k] * (KIND == 2 ? A0[i][c] : A0[i][r]);
        }
        // H: v_b (coef . S dN); HT: v_b (coef . S dNm) + (F S hv)_b with hv = s a_r (a_c . dN0)
        const double cs = coef[0] * SdNm[0] + coef[1] * SdNm[1] + coef[2] * SdNm[2];
#pragma unroll
        for (int b = 0; b < 3; ++b) t[b] += v[b] * cs;
        if (KIND == 3) {
          const double ac = A0[0][c] * dN0[0] + A0[1][c] * dN0[1] + A0[2][c] * dN0[2];
          double hv[3], Shv[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) hv[i] = s[k] * A0[i][r] * ac;
#pragma unroll
          for (int i = 0; i < 3; ++i) Shv[i] = Sm[i][0] * hv[0] + Sm[i][1] * hv[1] + Sm[i][2] * hv[2];
#pragma unroll
          for (int b = 0; b < 3; ++b) t[b] += F[b][0] * Shv[0] + F[b][1] * Shv[1] + F[b][2] * Shv[2];
        }
      }
#pragma unroll
      for (int b = 0; b < 3; ++b) Lacc[k][b] += w * t[b];
    }
    // D share: (E_alpha^T C E_alpha + E_alpha,alpha) w detJ (enhancedassumedstrains.hh:400)
#pragma unroll
    for (int m = 0; m < Cfg::DSH; ++m) {
      const int t = sub + 8 * m;
      if (t < Cfg::NT) {
        int aa, bb;
        packed_index(t, NA, aa, bb);
        double x = 0.0;
#pragma unroll
        for (int r = 0; r < 6; ++r) x += sm[Cfg::O_EA + 6 * aa + r] * sm[Cfg::O_CEA + 6 * bb + r];
        if (KIND != 1) {  // (v^a . v^b)(coef^a . S coef^b)  (displacementgradient.hh:213-230)
          const int ra = aa / 3, ca = aa % 3, rb = bb / 3, cb = bb % 3;
          double va[3], vb[3], fa[3], fb[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            va[i] = KIND == 2 ? A0[i][ra] : Fa[i][ca];
            vb[i] = KIND == 2 ? A0[i][rb] : Fa[i][cb];
            fa[i] = s[aa] * (KIND == 2 ? A0[i][ca] : A0[i][ra]);
            fb[i] = s[bb] * (KIND == 2 ? A0[i][cb] : A0[i][rb]);
          }
          double Sfb[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) Sfb[i] = Sm[i][0] * fb[0] + Sm[i][1] * fb[1] + Sm[i][2] * fb[2];
          x += (va[0] * vb[0] + va[1] * vb[1] + va[2] * vb[2]) * (fa[0] * Sfb[0] + fa[1] * Sfb[1] + fa[2] * Sfb[2]);
        }
        Dacc[m] += w * x;
      }
    }
    // R~ share: E_alpha^T S w detJ (enhancedassumedstrains.hh:428)
#pragma unroll
    for (int m = 0; m < Cfg::RSH; ++m) {
      const int k = sub + 8 * m;
      if (k < NA) {
        double x = 0.0;
#pragma unroll
        for (int r = 0; r < 6; ++r) x += sm[Cfg::O_EA + 6 * k + r] * S[r];
        Racc[m] += w * x;
      }
    }
    __syncwarp();  // shared scratch is rewritten by the next Gauss point
  }

  // ---- static condensation ------------------------------------------------------------------------------
#pragma unroll
  for (int m = 0; m < Cfg::DSH; ++m) {
    const int t = sub + 8 * m;
    if (t < Cfg::NT) {
      int aa, bb;
      packed_index(t, NA, aa, bb);
      sm[Cfg::O_D + NA * aa + bb] = Dacc[m];
      sm[Cfg::O_D + NA * bb + aa] = Dacc[m];
    }
  }
#pragma unroll
  for (int m = 0; m < Cfg::RSH; ++m) {
    const int k = sub + 8 * m;
    if (k < NA) sm[Cfg::O_RT + k] = Racc[m];
  }
  __syncwarp();
  if (sub == 0) {  // LU with partial pivoting of D in place
    double* D = sm + Cfg::O_D;
    for (int k = 0; k < NA; ++k) {
      int p = k;
      double best = fabs(D[NA * k + k]);
      for (int i = k + 1; i < NA; ++i)
        if (fabs(D[NA * i + k]) > best) best = fabs(D[NA * i + k]), p = i;
      sm[Cfg::O_PIV + k] = (double)p;
      if (!(best > 0.0)) {
        bad |= kStatusSingularD;
        D[NA * k + k] = 1.0;
        continue;
      }
      if (p != k)
        for (int j = 0; j < NA; ++j) {
          const double tmp = D[NA * k + j];
          D[NA * k + j] = D[NA * p + j];
          D[NA * p + j] = tmp;
        }
      const double inv = 1.0 / D[NA * k + k];
      for (int i = k + 1; i < NA; ++i) {
        const double l = D[NA * i + k] * inv;
        D[NA * i + k] = l;
        for (int j = k + 1; j < NA; ++j) D[NA * i + j] -= l * D[NA * k + j];
      }
    }
  }
  __syncwarp();
  // solve D z = rhs with the factors (row swaps applied in order)
  auto lu_solve = [&](double* z) {
    const double* D = sm + Cfg::O_D;
    for (int k = 0; k < NA; ++k) {
      const int p = (int)sm[Cfg::O_PIV + k];
      if (p != k) {
        const double t = z[k];
        z[k] = z[p];
        z[p] = t;
      }
    }
    for (int i = 1; i < NA; ++i)
      for (int j = 0; j < i; ++j) z[i] -= D[NA * i + j] * z[j];
    for (int i = NA - 1; i >= 0; --i) {
      for (int j = i + 1; j < NA; ++j) z[i] -= D[NA * i + j] * z[j];
      z[i] /= D[NA * i + i];
    }
  };
  double y[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) y[k] = sm[Cfg::O_RT + k];
  lu_solve(y);
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    double z[NA];
#pragma unroll
    for (int k = 0; k < NA; ++k) z[k] = Lacc[k][b];
    lu_solve(z);
#pragma unroll
    for (int k = 0; k < NA; ++k) sm[Cfg::O_Y + (3 * sub + b) * NA + k] = z[k];
  }
  __syncwarp();
  if (WANT_R) {
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double t = 0.0;
#pragma unroll
      for (int k = 0; k < NA; ++k) t += Lacc[k][b] * y[k];
      f[b] -= t;
    }
  }
  if (WANT_K) {
#pragma unroll
    for (int d = 0; d < 5; ++d) {
      const int Jn = (sub + d) & 7;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double t = 0.0;
#pragma unroll
          for (int k = 0; k < NA; ++k) t += Lacc[k][i] * sm[Cfg::O_Y + (3 * Jn + j) * NA + k];
          Kacc[d][i][j] -= t;
        }
    }
  }

  if (!active) return;
  if (bad && a.status) atomicOr(a.status, bad);
  if (WANT_R && a.eas_y) {  // condensation cache for the state update
    if (sub == 0)
#pragma unroll
      for (int k = 0; k < NA; ++k) a.eas_y[(size_t)k * ne + e] = y[k];
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int k = 0; k < NA; ++k)
        a.eas_Y[(size_t)(k * 24 + 3 * sub + b) * ne + e] = sm[Cfg::O_Y + (3 * sub + b) * NA + k];
  }
  const uint8_t fmaskI = a.node_fixed ? a.node_fixed[node] : uint8_t(0);
  if (WANT_R) {
    if (a.trac_idx) {
      const int t = a.trac_idx[e];
      if (t >= 0)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          f[c] -= (a.load_factor_dev ? *a.load_factor_dev : a.load_factor) * a.trac[24 * t + 3 * sub + c];
    }
    if (a.ext) {
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] -= a.ext[24 * (size_t)e + 3 * sub + c];
    }
    if (ELEM_OUT) {
#pragma unroll
      for (int c = 0; c < 3; ++c) a.elem_vec[24 * (size_t)li + 3 * sub + c] = f[c];
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (!((fmaskI >> c) & 1)) a.R[3 * node + c] += f[c];
    }
  }
  if (WANT_K) {
    if (ELEM_OUT) {
      double* out = a.elem_mat + 576 * (size_t)li;
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int Jn = (sub + d) & 7;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            out[(3 * Jn + j) * 24 + 3 * sub + i] = Kacc[d][i][j];
            if (d >= 1 && d <= 3) out[(3 * sub + i) * 24 + 3 * Jn + j] = Kacc[d][i][j];
          }
      }
    } else {
      KT* val = static_cast<KT*>(a.Kval);
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int Jn = (sub + d) & 7;
        const uint8_t fmaskJ = a.node_fixed ? a.node_fixed[a.conn[Jn * ne + e]] : uint8_t(0);
        KT* b1 = val + block_entry(a.slot[(size_t)(sub * 8 + Jn) * ne + e], 0);  // entries 32 apart
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            if (!(((fmaskI >> i) | (fmaskJ >> j)) & 1)) b1[32 * (3 * i + j)] += KT(Kacc[d][i][j]);
        if (d >= 1 && d <= 3) {
          KT* b2 = val + block_entry(a.slot[(size_t)(Jn * 8 + sub) * ne + e], 0);
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              if (!(((fmaskI >> i) | (fmaskJ >> j)) & 1)) b2[32 * (3 * j + i)] += KT(Kacc[d][i][j]);
        }
      }
    }
  }
}

template <int NA, int KIND, int MODE, typename KT, bool HYP>
void launch_t(const ElemArgs& a, const int32_t* list, int n_list, int e_base, cudaStream_t s) {
  using Cfg = EasCfg<NA>;
  const int blocks = (n_list + Cfg::EPB - 1) / Cfg::EPB;
  const size_t shm = sizeof(double) * Cfg::PER * Cfg::EPB;
  eas_element_kernel<NA, KIND, MODE, KT, HYP><<<blocks, Cfg::EPB * 8, shm, s>>>(a, list, n_list, e_base);
}

template <int NA, int KIND, bool HYP>
void launch_kind(const ElemArgs& a, int mode, bool fp32, const int32_t* list, int n, int base, cudaStream_t s) {
  switch (mode) {
    case kWantR: launch_t<NA, KIND, kWantR, double, HYP>(a, list, n, base, s); break;
    case kWantK:
      if (fp32) launch_t<NA, KIND, kWantK, float, HYP>(a, list, n, base, s);
      else launch_t<NA, KIND, kWantK, double, HYP>(a, list, n, base, s);
      break;
    case kWantR | kElemOut: launch_t<NA, KIND, kWantR | kElemOut, double, HYP>(a, list, n, base, s); break;
    case kWantK | kElemOut: launch_t<NA, KIND, kWantK | kElemOut, double, HYP>(a, list, n, base, s); break;
    default: break;
  }
}

// the element launches of one material family (HYP: the hyperelastic framework)
template <bool HYP>
void launch_eas_family(const ElemArgs& a, int mode, bool fp32, const int32_t* list, int n, int base, cudaStream_t s) {
  if (a.eas_kind == 1 && a.n_alpha == 9) launch_kind<9, 1, HYP>(a, mode, fp32, list, n, base, s);
  else if (a.eas_kind == 1 && a.n_alpha == 21) launch_kind<21, 1, HYP>(a, mode, fp32, list, n, base, s);
  else if (a.eas_kind == 2) launch_kind<9, 2, HYP>(a, mode, fp32, list, n, base, s);
  else if (a.eas_kind == 3) launch_kind<9, 3, HYP>(a, mode, fp32, list, n, base, s);
}

}  // namespace
}  // namespace ikr
