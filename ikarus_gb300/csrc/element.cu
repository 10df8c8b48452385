// Element kernels for 3D Q1 hexahedra with the compressible Neo-Hooke law (sm_103a).
//
// Reference path: NonLinearElastic::calculateVectorImpl / calculateMatrixImpl
// (ikarus/finiteelements/mechanics/nonlinearelastic.hh:375-430) with NeoHookeT
// (materials/hyperelastic/neohooke.hh:78-142) and dead tractions (loads/traction.hh:105-138).
//
// Work decomposition: 8 lanes per element (lane = element node I), 32 elements per 256-thread block.
// Per Gauss point the lanes reduce J = sum_I X_I (x) dN_I/dxi and H = sum_I u_I (x) grad N_I with warp
// butterflies, so every lane holds F, F^{-1}, ln J.  The Neo-Hooke first elasticity tensor contracted with
// two shape-function gradients needs only g_I = F^{-T} grad N_I:
//   K_IJ = w [ mu (grad N_I . grad N_J) I + lambda g_I (x) g_J + (mu - lambda ln J) g_J (x) g_I ]
// which equals the reference's B_I^T C B_J + kg_IJ (nonlinearelastic.hh:294-322) exactly in real arithmetic,
// and the internal force f_I = w [ mu F grad N_I + (lambda ln J - mu) g_I ] equals B_I^T S w.
// Lane I owns the node blocks (I, I+d mod 8), d = 0..4, and writes d = 1..3 also transposed, so each of the
// 64 blocks is produced once and the element matrix is exactly symmetric.
// Assembly is a plain read-modify-write into the BSR values through the precomputed element-to-block slot map;
// the host launches one colour class at a time (no two elements of a class share a node), so the summation
// order is fixed and repeated runs are bit-identical.
#include <cmath>
#include <type_traits>

#include "common.cuh"
#include "hyperelastic.cuh"
#include "kernels.h"

namespace ikr {

namespace {

// B-operator of the Green-Lagrange strain variation w.r.t. a node's displacement (rows 11, 22, 33, 23, 13, 12;
// easfunctions/displacementgradient.hh:129-146): column a of row (k, l) is dN_l F_ak + dN_k F_al
template <typename T>
__device__ __forceinline__ void bop_t(const T F[3][3], const T dN[3], T B[6][3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const T g0 = F[a][0], g1 = F[a][1], g2 = F[a][2];
    B[0][a] = dN[0] * g0;
    B[1][a] = dN[1] * g1;
    B[2][a] = dN[2] * g2;
    B[3][a] = dN[2] * g1 + dN[1] * g2;
    B[4][a] = dN[2] * g0 + dN[0] * g2;
    B[5][a] = dN[1] * g0 + dN[0] * g1;
  }
}

// EPB elements per block (8 lanes each): 16, 32 or 64, chosen per element set by timing (host.cpp)
// MAT 0: NeoHooke (neohooke.hh:78-142); MAT 1: StVenantKirchhoff (svk.hh:63-163); MAT 2: BlatzKo
// (hyperelastic/deviatoric/blatzko.hh with total stretches and no volumetric part, factory.hh:34-39); MAT 3: the
// hyperelastic framework (hyperelastic/interface.hh, any deviatoric and volumetric function, hyperelastic.cuh)
template <typename KT, int MODE, int EPB, int MAT = 0>
__global__ void __launch_bounds__(EPB * 8) disp_element_kernel(ElemArgs a, const int32_t* __restrict__ list, int n_list,
                                                               int e_base) {
  constexpr bool WANT_R = MODE & kWantR;
  constexpr bool WANT_K = MODE & kWantK;
  constexpr bool WANT_E = MODE & kWantEnergy;
  constexpr bool ELEM_OUT = MODE & kElemOut;
  constexpr bool BLOCKS = MODE & kElemBlocks;
  static_assert(!(WANT_R || WANT_E) || std::is_same<KT, double>::value, "residual and energy are FP64");
  static_assert(!BLOCKS || (WANT_K && std::is_same<KT, float>::value), "element blocks: FP32 tangent only");
  __shared__ KT sh[EPB][8][6];
  __shared__ KT hm[MAT == 3 ? EPB : 1][36];  // hyperelastic: the Gauss point's material moduli (Voigt)
  // element blocks: staged per warp (4 elements x 36 blocks x 9 entries) and copied out with 16-byte stores
  __shared__ __align__(16) KT stage[BLOCKS ? EPB / 4 : 1][BLOCKS ? 4 * kElemBlockCount * 9 : 1];

  const int lane = threadIdx.x & 31;
  const int sub = threadIdx.x & 7;
  const int es = threadIdx.x >> 3;
  const int li = blockIdx.x * EPB + es;
  const bool active = li < n_list;
  const int lic = active ? li : n_list - 1;
  const int e = list ? list[lic] : e_base + lic;
  const int ne = a.n_elems;
  const int node = a.conn[sub * ne + e];

  double Xd[3], Ud[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    Xd[c] = a.X[3 * node + c];
    Ud[c] = a.u ? a.u[3 * node + c] : 0.0;
  }
  // coordinates and displacements relative to the element's first corner keep FP32 geometry accurate
  KT dX[3], dU[3];
  const int src = lane & ~7;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double x0 = __shfl_sync(0xffffffffu, Xd[c], src);
    const double u0 = __shfl_sync(0xffffffffu, Ud[c], src);
    dX[c] = KT(Xd[c] - x0);
    dU[c] = KT(Ud[c] - u0);
  }
  const KT lam = KT(a.lam_e ? a.lam_e[e] : a.lam), mu = KT(a.mu_e ? a.mu_e[e] : a.mu);

  KT Kacc[5][3][3];
  if (WANT_K) {
#pragma unroll
    for (int d = 0; d < 5; ++d)
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Kacc[d][i][j] = KT(0);
  }
  double f[3] = {0.0, 0.0, 0.0};
  double psi = 0.0;
  int bad = 0;

#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    KT dxi[3];
    ref_gradient_at_gp<KT>(sub, q, dxi);
    KT J[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) J[i][j] = sum8(dX[i] * dxi[j]);
    KT Ji[3][3];
    const KT detJ = inv3(J, Ji);
    KT dN[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dN[k] = dxi[0] * Ji[0][k] + dxi[1] * Ji[1][k] + dxi[2] * Ji[2][k];
    KT F[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] = sum8(dU[i] * dN[j]) + (i == j ? KT(1) : KT(0));
    if constexpr (MAT == 1) {
      // StVenantKirchhoff: E = (F^T F - I) / 2, S = lambda tr(E) I + 2 mu E, P = F S; first elasticity tensor
      // contracted with two gradients, g = F grad N:
      // K_IJ = w [lambda g_I (x) g_J + mu (dN_I . dN_J) F F^T + mu g_J (x) g_I + (dN_I . S dN_J) I]
      KT E[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          E[i][j] = KT(0.5) * (F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j] - (i == j ? KT(1) : KT(0)));
      const KT trE = E[0][0] + E[1][1] + E[2][2];
      KT S[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[i][j] = KT(2) * mu * E[i][j] + (i == j ? lam * trE : KT(0));
      const KT w = KT(kGaussW) * detJ;
      KT SdN[3], g[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        SdN[k] = S[k][0] * dN[0] + S[k][1] * dN[1] + S[k][2] * dN[2];
        g[k] = F[k][0] * dN[0] + F[k][1] * dN[1] + F[k][2] * dN[2];
      }
      if (WANT_R) {
#pragma unroll
        for (int i = 0; i < 3; ++i) f[i] += double(w * (F[i][0] * SdN[0] + F[i][1] * SdN[1] + F[i][2] * SdN[2]));
      }
      if (WANT_E && sub == 0) {
        KT EE = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) EE += E[i][j] * E[i][j];
        psi += double(w * (lam / KT(2) * trE * trE + mu * EE));
      }
      if (WANT_K) {
        KT FFt[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) FFt[i][j] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          sh[es][sub][k] = dN[k];
          sh[es][sub][3 + k] = g[k];
        }
        __syncwarp();
#pragma unroll
        for (int d = 0; d < 5; ++d) {
          const int Jn = (sub + d) & 7;
          KT dNJ[3], gJ[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            dNJ[k] = sh[es][Jn][k];
            gJ[k] = sh[es][Jn][3 + k];
          }
          const KT wm = w * mu * (dN[0] * dNJ[0] + dN[1] * dNJ[1] + dN[2] * dNJ[2]);
          const KT ws = w * (SdN[0] * dNJ[0] + SdN[1] * dNJ[1] + SdN[2] * dNJ[2]);
          const KT wl = w * lam, wu = w * mu;
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              Kacc[d][i][j] += wl * g[i] * gJ[j] + wm * FFt[i][j] + wu * gJ[i] * g[j] + (i == j ? ws : KT(0));
        }
        __syncwarp();
      }
      continue;
    }
    if constexpr (MAT == 3) {
      // hyperelastic framework: the material point (S and the Voigt moduli) in FP64 from C = F^T F
      // (hyper::evaluate; lanes share the moduli, 4-5 entries each), then B_I^T C B_J + (grad N_I . S grad N_J) I
      // and f_I = B_I^T S with the B-operator of F (nonlinearelastic.hh:294-342) in KT
      double Cd[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          Cd[i][j] = double(F[0][i]) * double(F[0][j]) + double(F[1][i]) * double(F[1][j]) +
                     double(F[2][i]) * double(F[2][j]);
      hyper::Point pt;
      bad |= hyper::evaluate(a.hyper, Cd, pt, WANT_K);
      const KT w = KT(kGaussW) * detJ;
      KT S[3][3];
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        const int i = voigt_a(v), j = voigt_b(v);
        S[i][j] = S[j][i] = KT(hyper::stress(pt, i, j));
      }
      KT SdN[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) SdN[k] = S[k][0] * dN[0] + S[k][1] * dN[1] + S[k][2] * dN[2];
      if (WANT_R) {
#pragma unroll
        for (int i = 0; i < 3; ++i) f[i] += double(w * (F[i][0] * SdN[0] + F[i][1] * SdN[1] + F[i][2] * SdN[2]));
      }
      if (WANT_E && sub == 0) psi += double(w) * pt.psi;
      if (WANT_K) {
        for (int t = sub; t < 36; t += 8)
          hm[es][t] = KT(hyper::modulus(pt, voigt_a(t / 6), voigt_b(t / 6), voigt_a(t % 6), voigt_b(t % 6)));
#pragma unroll
        for (int k = 0; k < 3; ++k) sh[es][sub][k] = dN[k];
        __syncwarp();
        KT BI[6][3], CB[6][3];
        bop_t(F, dN, BI);
#pragma unroll
        for (int c = 0; c < 6; ++c)
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            KT acc = KT(0);
#pragma unroll
            for (int r = 0; r < 6; ++r) acc += BI[r][i] * hm[es][6 * r + c];
            CB[c][i] = w * acc;
          }
#pragma unroll
        for (int d = 0; d < 5; ++d) {
          const int Jn = (sub + d) & 7;
          KT dNJ[3], BJ[6][3];
#pragma unroll
          for (int k = 0; k < 3; ++k) dNJ[k] = sh[es][Jn][k];
          bop_t(F, dNJ, BJ);
          const KT kg = w * (SdN[0] * dNJ[0] + SdN[1] * dNJ[1] + SdN[2] * dNJ[2]);
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              KT acc = i == j ? kg : KT(0);
#pragma unroll
              for (int c = 0; c < 6; ++c) acc += CB[c][i] * BJ[c][j];
              Kacc[d][i][j] += acc;
            }
        }
        __syncwarp();
      }
      continue;
    }
    KT Fi[3][3];
    const KT detF = inv3(F, Fi);
    // det C = det(F)^2 must exceed 1e-10 (checkPositiveOrAbort); NaN fails the test as well
    if (!(detF * detF > KT(1e-10)) || !(detF > KT(0))) bad |= kStatusNonPositiveDetC;
    const KT w = KT(kGaussW) * detJ;
    KT g[3];  // F^{-T} grad N_I
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = Fi[0][k] * dN[0] + Fi[1][k] * dN[1] + Fi[2][k] * dN[2];
    if constexpr (MAT == 2) {
      // BlatzKo, W = mu/2 (tr C^-1 + 2 J - 5) (the principal-stretch form sum 1/lambda_i^2 + 2 lambda_1 lambda_2
      // lambda_3 written with invariants): P = mu (J I - b^-1) F^-T, b^-1 = F^-T F^-1; with g = F^-T grad N:
      // K_IJ = w mu [J (g_I (x) g_J - g_J (x) g_I) + g_J (x) b^-1 g_I + (g_I . g_J) b^-1 + b^-1 g_J (x) g_I]
      KT binv[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) binv[i][k] = Fi[0][i] * Fi[0][k] + Fi[1][i] * Fi[1][k] + Fi[2][i] * Fi[2][k];
      KT bg[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) bg[i] = binv[i][0] * g[0] + binv[i][1] * g[1] + binv[i][2] * g[2];
      if (WANT_R) {
#pragma unroll
        for (int i = 0; i < 3; ++i) f[i] += double(w * mu * (detF * g[i] - bg[i]));
      }
      if (WANT_E && sub == 0) {
        const KT trCi = binv[0][0] + binv[1][1] + binv[2][2];
        psi += double(w * (mu / KT(2) * (trCi + KT(2) * detF - KT(5))));
      }
      if (WANT_K) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          sh[es][sub][k] = g[k];
          sh[es][sub][3 + k] = bg[k];
        }
        __syncwarp();
        const KT wm = w * mu, wj = w * mu * detF;
#pragma unroll
        for (int d = 0; d < 5; ++d) {
          const int Jn = (sub + d) & 7;
          KT gJ[3], bgJ[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            gJ[k] = sh[es][Jn][k];
            bgJ[k] = sh[es][Jn][3 + k];
          }
          const KT gg = wm * (g[0] * gJ[0] + g[1] * gJ[1] + g[2] * gJ[2]);
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              Kacc[d][i][j] += wj * (g[i] * gJ[j] - gJ[i] * g[j]) + wm * (gJ[i] * bg[j] + bgJ[i] * g[j]) +
                               gg * binv[i][j];
        }
        __syncwarp();
      }
      continue;
    }
    const KT lnJ = log(detF);

    if (WANT_R) {
      // P = mu (F - F^{-T}) + lambda ln J F^{-T}: written with F - F^{-T} so the undeformed state gives an
      // exactly zero internal force (no FMA rounding residue), as the reference's S = 0 does
      const KT ll = lam * lnJ;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const KT Pd = (F[i][0] - Fi[0][i]) * dN[0] + (F[i][1] - Fi[1][i]) * dN[1] + (F[i][2] - Fi[2][i]) * dN[2];
        f[i] += double(w * (mu * Pd + ll * g[i]));
      }
    }
    if (WANT_E && sub == 0) {
      KT trC = 0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) trC += F[i][j] * F[i][j];
      psi += double(w * (mu / KT(2) * (trC - KT(3) - KT(2) * lnJ) + lam / KT(2) * lnJ * lnJ));
    }
    if (WANT_K) {
      const KT c = mu - lam * lnJ;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        sh[es][sub][k] = dN[k];
        sh[es][sub][3 + k] = g[k];
      }
      __syncwarp();
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int Jn = (sub + d) & 7;
        KT dNJ[3], gJ[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          dNJ[k] = sh[es][Jn][k];
          gJ[k] = sh[es][Jn][3 + k];
        }
        const KT dd = w * mu * (dN[0] * dNJ[0] + dN[1] * dNJ[1] + dN[2] * dNJ[2]);
        const KT wl = w * lam, wc = w * c;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            Kacc[d][i][j] += wl * g[i] * gJ[j] + wc * gJ[i] * g[j] + (i == j ? dd : KT(0));
      }
      __syncwarp();
    }
  }

  const uint8_t fmaskI = a.node_fixed ? a.node_fixed[node] : uint8_t(0);
  if (WANT_R || WANT_E) {
    if (a.trac_idx) {
      const int t = a.trac_idx[e];
      if (t >= 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double tv = a.trac[24 * t + 3 * sub + c];
          const double lf = a.load_factor_dev ? *a.load_factor_dev : a.load_factor;
          f[c] -= lf * tv;
          if (WANT_E) psi -= lf * tv * Ud[c];
        }
      }
    }
    if (a.ext) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double tv = a.ext[24 * (size_t)e + 3 * sub + c];
        f[c] -= tv;
        if (WANT_E) psi -= tv * Ud[c];
      }
    }
  }
  double psi_tot = 0.0;
  if (WANT_E) psi_tot = sum8(psi);  // last warp-wide operation: inactive lanes may leave after it

  if (!active) return;
  if (bad) {
    if (a.inst_status) atomicOr(a.inst_status + a.elem_inst[e], bad);
    else if (a.status) atomicOr(a.status, bad);
  }
  if (WANT_E && ELEM_OUT && sub == 0) a.elem_energy[li] = psi_tot;
  if (WANT_R) {
    if (ELEM_OUT) {
#pragma unroll
      for (int c = 0; c < 3; ++c) a.elem_vec[24 * (size_t)li + 3 * sub + c] = f[c];
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (!((fmaskI >> c) & 1)) a.R[3 * node + c] += f[c];
    }
  }
  if constexpr (BLOCKS) {
    // lane I's blocks (I, I + d), d = 0..3, and (I, I + 4) for I < 4, into the warp's stage, then the element's 324
    // values to blk[e] (8 lanes, 16 bytes each per store)
    KT* st = stage[threadIdx.x >> 5] + (es & 3) * (kElemBlockCount * 9);
#pragma unroll
    for (int d = 0; d < 5; ++d) {
      if (d == 4 && sub >= 4) break;
      const int pb = d < 4 ? 8 * d + sub : 32 + sub;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) st[pb * 9 + 3 * i + j] = Kacc[d][i][j];
    }
    __syncwarp(0xFFu << (lane & ~7));
    const float4* src4 = reinterpret_cast<const float4*>(st);
    float4* dst4 = reinterpret_cast<float4*>(static_cast<float*>(a.blk) + (size_t)e * (kElemBlockCount * 9));
    for (int k = sub; k < kElemBlockCount * 9 / 4; k += 8) dst4[k] = src4[k];
  } else if (WANT_K) {
    if (ELEM_OUT) {
      double* out = a.elem_mat + 576 * (size_t)li;
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int Jn = (sub + d) & 7;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            out[(3 * Jn + j) * 24 + 3 * sub + i] = double(Kacc[d][i][j]);
            if (d >= 1 && d <= 3) out[(3 * sub + i) * 24 + 3 * Jn + j] = double(Kacc[d][i][j]);
          }
      }
    } else {
      KT* val = static_cast<KT*>(a.Kval);
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int Jn = (sub + d) & 7;
        const uint8_t fmaskJ = a.node_fixed ? a.node_fixed[a.conn[Jn * ne + e]] : uint8_t(0);
        const int64_t s1 = a.slot[(size_t)(sub * 8 + Jn) * ne + e];
        KT* b1 = val + block_entry(s1, 0);  // entries of a block are 32 apart
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            if (!(((fmaskI >> i) | (fmaskJ >> j)) & 1)) b1[32 * (3 * i + j)] += Kacc[d][i][j];
        if (d >= 1 && d <= 3) {
          const int64_t s2 = a.slot[(size_t)(Jn * 8 + sub) * ne + e];
          KT* b2 = val + block_entry(s2, 0);
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              if (!(((fmaskI >> i) | (fmaskJ >> j)) & 1)) b2[32 * (3 * j + i)] += Kacc[d][i][j];
        }
      }
    }
  }
}


// Tangent assembly by block rows (displacement-based NeoHooke): one thread per node row I.  For every element
// adjacent to I (ascending element index) the thread evaluates the element's 8 Gauss points and adds row a of the
// element tangent (a = I's corner), K_aJ for the 8 corners J, into its own row's blocks:
//   K_aJ += w [lambda g_a (x) g_J + (mu - lambda ln J) g_J (x) g_a + mu (dN_a . dN_J) I],  g = F^-T grad N.
// No two threads write a block, so there is no colouring and one launch; the 32 rows of a warp are one slice,
// whose blocks of equal k lie side by side in the entry-interleaved layout, so a warp's read-modify-writes
// coalesce.  The Gauss-point kinematics of an element are evaluated once per adjacent node (8 times): arithmetic
// traded for colouring-free, coalesced writes.
template <typename KT>
__global__ void __launch_bounds__(128) row_tangent_kernel(ElemArgs a, const int32_t* __restrict__ ne_ptr,
                                                        const int32_t* __restrict__ ne_elems) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= a.n_nodes) return;
  const int ne = a.n_elems;
  const uint8_t fmaskI = a.node_fixed ? a.node_fixed[I] : uint8_t(0);
  KT* val = static_cast<KT*>(a.Kval);
  for (int t = ne_ptr[I]; t < ne_ptr[I + 1]; ++t) {
    const int e = ne_elems[t];
    int nodes[8];
    int ai = 0;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      nodes[v] = a.conn[v * ne + e];
      if (nodes[v] == I) ai = v;
    }
    // coordinates and displacements relative to the element's first corner (as the element kernel does)
    KT dX[8][3], dU[8][3];
    {
      double x0[3], u0[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        x0[c] = a.X[3 * nodes[0] + c];
        u0[c] = a.u ? a.u[3 * nodes[0] + c] : 0.0;
      }
#pragma unroll
      for (int v = 0; v < 8; ++v)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          dX[v][c] = KT(a.X[3 * nodes[v] + c] - x0[c]);
          dU[v][c] = KT((a.u ? a.u[3 * nodes[v] + c] : 0.0) - u0[c]);
        }
    }
    const KT lam = KT(a.lam_e ? a.lam_e[e] : a.lam), mu = KT(a.mu_e ? a.mu_e[e] : a.mu);
    KT K[8][3][3];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) K[j][r][c] = KT(0);
    int bad = 0;
#pragma unroll 1
    for (int q = 0; q < 8; ++q) {
      KT J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        KT d[3];
        ref_gradient_at_gp<KT>(v, q, d);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) J[r][c] += dX[v][r] * d[c];
      }
      KT Ji[3][3];
      const KT detJ = inv3(J, Ji);
      KT F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        KT d[3], dn[3];
        ref_gradient_at_gp<KT>(v, q, d);
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] = d[0] * Ji[0][k] + d[1] * Ji[1][k] + d[2] * Ji[2][k];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) F[r][c] += dU[v][r] * dn[c];
      }
      KT Fi[3][3];
      const KT detF = inv3(F, Fi);
      if (!(detF * detF > KT(1e-10)) || !(detF > KT(0))) bad |= kStatusNonPositiveDetC;
      const KT lnJ = log(detF);
      const KT w = KT(kGaussW) * detJ;
      const KT wl = w * lam, wc = w * (mu - lam * lnJ), wm = w * mu;
      KT dna[3], ga[3];
      {
        KT d[3];
        ref_gradient_at_gp<KT>(ai, q, d);
#pragma unroll
        for (int k = 0; k < 3; ++k) dna[k] = d[0] * Ji[0][k] + d[1] * Ji[1][k] + d[2] * Ji[2][k];
#pragma unroll
        for (int k = 0; k < 3; ++k) ga[k] = Fi[0][k] * dna[0] + Fi[1][k] * dna[1] + Fi[2][k] * dna[2];
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        KT d[3], dn[3], gj[3];
        ref_gradient_at_gp<KT>(j, q, d);
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] = d[0] * Ji[0][k] + d[1] * Ji[1][k] + d[2] * Ji[2][k];
#pragma unroll
        for (int k = 0; k < 3; ++k) gj[k] = Fi[0][k] * dn[0] + Fi[1][k] * dn[1] + Fi[2][k] * dn[2];
        const KT dd = wm * (dna[0] * dn[0] + dna[1] * dn[1] + dna[2] * dn[2]);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) K[j][r][c] += wl * ga[r] * gj[c] + wc * gj[r] * ga[c] + (r == c ? dd : KT(0));
      }
    }
    if (bad) {
      if (a.inst_status) atomicOr(a.inst_status + a.elem_inst[e], bad);
      else if (a.status) atomicOr(a.status, bad);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint8_t fmaskJ = a.node_fixed ? a.node_fixed[nodes[j]] : uint8_t(0);
      KT* b = val + block_entry(a.slot[(size_t)(ai * 8 + j) * ne + e], 0);
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if (!(((fmaskI >> r) | (fmaskJ >> c)) & 1)) b[32 * (3 * r + c)] += K[j][r][c];
    }
  }
}

// Dead traction at load factor 1 on the element's Neumann faces, 1-point rule per face
// (loads/traction.hh:122-135: quadrature order = order() = 1 -> the face centre, weight 1):
// trac[slot][3v+c] = sum_faces N_v(centre) t_c dA.  One thread per loaded element, faces in input order.
__global__ void traction_kernel(const double* __restrict__ X, const int32_t* __restrict__ conn, int ne, int n_slots,
                                const int32_t* __restrict__ slot_elem, const int32_t* __restrict__ face_ptr,
                                const int32_t* __restrict__ face_local, const double* __restrict__ t,
                                double* __restrict__ trac) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_slots) return;
  const int e = slot_elem[s];
  double acc[24];
  for (int k = 0; k < 24; ++k) acc[k] = 0.0;
  double Xe[8][3];
  for (int v = 0; v < 8; ++v) {
    const int n = conn[v * ne + e];
    for (int c = 0; c < 3; ++c) Xe[v][c] = X[3 * n + c];
  }
  for (int k = face_ptr[s]; k < face_ptr[s + 1]; ++k) {
    const int lf = face_local[k];
    const int d = lf >> 1, side = lf & 1;
    const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
    double a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
    for (int v = 0; v < 8; ++v) {
      if (((v >> d) & 1) != side) continue;
      const double s1 = ((v >> t1) & 1) ? 0.5 : -0.5;
      const double s2 = ((v >> t2) & 1) ? 0.5 : -0.5;
      for (int c = 0; c < 3; ++c) {
        a1[c] += Xe[v][c] * s1;
        a2[c] += Xe[v][c] * s2;
      }
    }
    const double cr0 = a1[1] * a2[2] - a1[2] * a2[1];
    const double cr1 = a1[2] * a2[0] - a1[0] * a2[2];
    const double cr2 = a1[0] * a2[1] - a1[1] * a2[0];
    const double dA = sqrt(cr0 * cr0 + cr1 * cr1 + cr2 * cr2);
    for (int v = 0; v < 8; ++v) {
      if (((v >> d) & 1) != side) continue;
      for (int c = 0; c < 3; ++c) acc[3 * v + c] += 0.25 * t[3 * k + c] * 1.0 * dA;
    }
  }
  for (int k = 0; k < 24; ++k) trac[24 * (size_t)s + k] = acc[k];
}

// FP64 residual assembly with the material work spread over the Gauss points: lane q of an element's 8 lanes
// evaluates Gauss point q (geometry J, dN/dX of all 8 nodes, F, F^-1, ln J, P) once, instead of every lane
// evaluating every Gauss point; the nodal forces w P dN_v of each point are exchanged through shared memory and
// lane v sums its node's over the points in ascending order.  About a quarter of the FP64 operations of the
// node-per-lane form, which matters because GB300's FP64 rate bounds this kernel.
// HYP: the hyperelastic framework's material point (a separate instantiation keeps the other laws' registers)
template <int EPB, bool HYP>
__global__ void __launch_bounds__(EPB * 8) disp_residual_gp_kernel(ElemArgs a, const int32_t* __restrict__ list,
                                                                    int n_list, int e_base) {
  __shared__ double fs[EPB][8][8][3];  // [element][Gauss point][node][component]
  const int lane = threadIdx.x & 31;
  const int sub = threadIdx.x & 7;  // node for loads and the scatter, Gauss point for the material work
  const int es = threadIdx.x >> 3;
  const int li = blockIdx.x * EPB + es;
  const bool active = li < n_list;
  const int lic = active ? li : n_list - 1;
  const int e = list ? list[lic] : e_base + lic;
  const int ne = a.n_elems;
  const int node = a.conn[sub * ne + e];
  const int src = lane & ~7;
  double Xd[3], Ud[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    Xd[c] = a.X[3 * node + c];
    Ud[c] = a.u ? a.u[3 * node + c] : 0.0;
  }
  // coordinates and displacements relative to the element's first corner (as the node-per-lane kernel does)
  double dX[3], dU[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    dX[c] = Xd[c] - __shfl_sync(0xffffffffu, Xd[c], src);
    dU[c] = Ud[c] - __shfl_sync(0xffffffffu, Ud[c], src);
  }
  const double lam = a.lam_e ? a.lam_e[e] : a.lam, mu = a.mu_e ? a.mu_e[e] : a.mu;
  const int q = sub;
  // J = sum_v dX_v (x) dxi_v(q)
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    double xv[3], dxi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) xv[c] = __shfl_sync(0xffffffffu, dX[c], src + v);
    ref_gradient_at_gp<double>(v, q, dxi);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) J[i][j] += xv[i] * dxi[j];
  }
  double Ji[3][3];
  const double detJ = inv3(J, Ji);
  // F = I + sum_v dU_v (x) dN_v(q)
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    double uv[3], dxi[3], dN[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) uv[c] = __shfl_sync(0xffffffffu, dU[c], src + v);
    ref_gradient_at_gp<double>(v, q, dxi);
#pragma unroll
    for (int k = 0; k < 3; ++k) dN[k] = dxi[0] * Ji[0][k] + dxi[1] * Ji[1][k] + dxi[2] * Ji[2][k];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] += uv[i] * dN[j];
  }
  int bad = 0;
  const double w = kGaussW * detJ;
  double P[3][3];
  if constexpr (HYP) {
    // P = F S with S of the hyperelastic material point at C = F^T F
    double Cd[3][3], S[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Cd[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
    hyper::Point pt;
    bad |= hyper::evaluate(a.hyper, Cd, pt, false);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = hyper::stress(pt, i, j);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P[i][j] = w * (F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j]);
  } else if (a.material == 1) {
    // StVenantKirchhoff: P = F S, S = lambda tr(E) I + 2 mu E, E = (F^T F - I) / 2
    double E[3][3], S[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        E[i][j] = 0.5 * (F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j] - (i == j ? 1.0 : 0.0));
    const double trE = E[0][0] + E[1][1] + E[2][2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = 2.0 * mu * E[i][j] + (i == j ? lam * trE : 0.0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P[i][j] = w * (F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j]);
  } else if (a.material == 2) {
    // BlatzKo: P = mu (J I - b^-1) F^-T = mu (J F^-T - F^-T F^-1 F^-T)
    double Fi[3][3];
    const double detF = inv3(F, Fi);
    if (!(detF * detF > 1e-10) || !(detF > 0.0)) bad |= kStatusNonPositiveDetC;
    double binv[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) binv[i][k] = Fi[0][i] * Fi[0][k] + Fi[1][i] * Fi[1][k] + Fi[2][i] * Fi[2][k];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        P[i][j] = w * mu * (detF * Fi[j][i] - (binv[i][0] * Fi[j][0] + binv[i][1] * Fi[j][1] + binv[i][2] * Fi[j][2]));
  } else {
    double Fi[3][3];
    const double detF = inv3(F, Fi);
    // det C = det(F)^2 must exceed 1e-10 (checkPositiveOrAbort); NaN fails the test as well
    if (!(detF * detF > 1e-10) || !(detF > 0.0)) bad |= kStatusNonPositiveDetC;
    const double lnJ = log(detF);
    // P = mu (F - F^-T) + lambda ln J F^-T (F - F^-T keeps the undeformed internal force exactly zero)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P[i][j] = w * (mu * (F[i][j] - Fi[j][i]) + lam * lnJ * Fi[j][i]);
  }
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    double dxi[3], dN[3];
    ref_gradient_at_gp<double>(v, q, dxi);
#pragma unroll
    for (int k = 0; k < 3; ++k) dN[k] = dxi[0] * Ji[0][k] + dxi[1] * Ji[1][k] + dxi[2] * Ji[2][k];
#pragma unroll
    for (int i = 0; i < 3; ++i) fs[es][q][v][i] = P[i][0] * dN[0] + P[i][1] * dN[1] + P[i][2] * dN[2];
  }
  __syncwarp();
  double f[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int g = 0; g < 8; ++g)
#pragma unroll
    for (int i = 0; i < 3; ++i) f[i] += fs[es][g][sub][i];
  if (a.trac_idx) {
    const int t = a.trac_idx[e];
    if (t >= 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        f[c] -= (a.load_factor_dev ? *a.load_factor_dev : a.load_factor) * a.trac[24 * t + 3 * sub + c];
    }
  }
  if (a.ext) {
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] -= a.ext[24 * (size_t)e + 3 * sub + c];
  }
  if (!active) return;
  if (bad) {
    if (a.inst_status) atomicOr(a.inst_status + a.elem_inst[e], bad);
    else if (a.status) atomicOr(a.status, bad);
  }
  const uint8_t fmask = a.node_fixed ? a.node_fixed[node] : uint8_t(0);
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if (!((fmask >> c) & 1)) a.R[3 * node + c] += f[c];
}

template <int EPB>
void launch_residual_gp(const ElemArgs& a, const int32_t* list, int n_list, int e_base, cudaStream_t s) {
  const int blocks = (n_list + EPB - 1) / EPB;
  if (a.material == 3) disp_residual_gp_kernel<EPB, true><<<blocks, EPB * 8, 0, s>>>(a, list, n_list, e_base);
  else disp_residual_gp_kernel<EPB, false><<<blocks, EPB * 8, 0, s>>>(a, list, n_list, e_base);
}

// calculateAt<PK2Stress / kirchhoffStress / cauchyStress> (nonlinearelastic.hh:237-271) of elements
// [e0, e0 + count) at local points xi (one per element or one for all): thread per element, FP64.
// H at xi, E = GL(H), C = 2E + I, S = mu (I - C^-1) + lambda ln J C^-1, tau = F S F^T, sigma = tau / det F
// (stressconversions.hh:88-125); Voigt [11, 22, 33, 23, 13, 12] without shear factors.
__global__ void stress_at_kernel(ElemArgs a, int e0, int count, const double* __restrict__ xi, int xi_per_elem,
                                 int type, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int e = e0 + k;
  const int ne = a.n_elems;
  const double* x = xi + (xi_per_elem ? 3 * k : 0);
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double dxi[8][3], U[8][3];
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const int node = a.conn[v * ne + e];
    double f[3], df[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const bool b = (v >> d) & 1;
      f[d] = b ? x[d] : 1.0 - x[d];
      df[d] = b ? 1.0 : -1.0;
    }
    dxi[v][0] = df[0] * f[1] * f[2];
    dxi[v][1] = f[0] * df[1] * f[2];
    dxi[v][2] = f[0] * f[1] * df[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) U[v][c] = a.u ? a.u[3 * node + c] : 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) J[i][j] += a.X[3 * node + i] * dxi[v][j];
  }
  double Ji[3][3];
  inv3(J, Ji);
  double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    double dN[3];
#pragma unroll
    for (int kk = 0; kk < 3; ++kk) dN[kk] = dxi[v][0] * Ji[0][kk] + dxi[v][1] * Ji[1][kk] + dxi[v][2] * Ji[2][kk];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) H[i][j] += U[v][i] * dN[j];
  }
  double C[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double hh = H[0][i] * H[0][j] + H[1][i] * H[1][j] + H[2][i] * H[2][j];
      C[i][j] = H[i][j] + H[j][i] + hh + (i == j ? 1.0 : 0.0);
    }
  const double lam = a.lam_e ? a.lam_e[e] : a.lam, mu = a.mu_e ? a.mu_e[e] : a.mu;
  double S[3][3];
  if (a.material == 3) {  // hyperelastic framework
    hyper::Point pt;
    const int bad = hyper::evaluate(a.hyper, C, pt, false);
    if (bad && a.status) atomicOr(a.status, bad);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = hyper::stress(pt, i, j);
  } else if (a.material == 1) {  // StVenantKirchhoff: S = lambda tr(E) I + 2 mu E with E = (C - I) / 2
    const double trE = 0.5 * (C[0][0] + C[1][1] + C[2][2] - 3.0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = mu * (C[i][j] - (i == j ? 1.0 : 0.0)) + (i == j ? lam * trE : 0.0);
  } else {
    double Ci[3][3];
    const double detC = inv3(C, Ci);
    if (!(detC > 1e-10) && a.status) atomicOr(a.status, kStatusNonPositiveDetC);
    if (a.material == 2) {  // BlatzKo: S = mu (J C^-1 - C^-2)
      const double Jd = sqrt(detC);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          S[i][j] = mu * (Jd * Ci[i][j] - (Ci[i][0] * Ci[0][j] + Ci[i][1] * Ci[1][j] + Ci[i][2] * Ci[2][j]));
    } else {
      const double lnJ = log(sqrt(detC));
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[i][j] = mu * ((i == j ? 1.0 : 0.0) - Ci[i][j]) + lam * lnJ * Ci[i][j];
    }
  }
  double R[3][3];
  if (type == 0) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) R[i][j] = S[i][j];
  } else {
    double F[3][3], FS[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) FS[i][j] = F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j];
    const double sc = type == 2 ? 1.0 / det3(F) : 1.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) R[i][j] = sc * (FS[i][0] * F[j][0] + FS[i][1] * F[j][1] + FS[i][2] * F[j][2]);
  }
  double* o = out + 6 * (size_t)k;
  o[0] = R[0][0], o[1] = R[1][1], o[2] = R[2][2], o[3] = R[1][2], o[4] = R[0][2], o[5] = R[0][1];
}

// inverse of the element-to-block map, counted per padded block, filled and sorted per block
__global__ void tangent_inv_count_kernel(const int32_t* __restrict__ slot, int64_t n, int32_t* __restrict__ cnt) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n) atomicAdd(&cnt[slot[t]], 1);
}
__global__ void tangent_inv_fill_kernel(const int32_t* __restrict__ slot, int ne, const int32_t* __restrict__ ptr,
                                        int32_t* __restrict__ cursor, int32_t* __restrict__ inv) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 64LL * ne) return;
  const int pair = (int)(t / ne), e = (int)(t % ne);
  const int b = slot[t];
  const int code = tangent_block_code(pair >> 3, pair & 7);
  inv[ptr[b] + atomicAdd(&cursor[b], 1)] = ((e * kElemBlockCount + (code >> 1)) << 1) | (code & 1);
}
__global__ void tangent_inv_sort_kernel(const int32_t* __restrict__ ptr, int32_t* __restrict__ inv, int64_t n) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= n) return;
  const int c0 = ptr[b], c1 = ptr[b + 1];
  for (int i = c0 + 1; i < c1; ++i) {  // at most 8 entries: insertion sort, ascending
    const int v = inv[i];
    int j = i - 1;
    while (j >= c0 && inv[j] > v) {
      inv[j + 1] = inv[j];
      --j;
    }
    inv[j + 1] = v;
  }
}

// One thread per padded block: the sum of its element blocks in ascending order, the Full Dirichlet treatment, and
// the nine entries written to the entry-interleaved slice (a warp writes 9 x 128 contiguous bytes).
__global__ void __launch_bounds__(256) tangent_gather_kernel(Bsr A, const int32_t* __restrict__ gslice,
                                                             const int32_t* __restrict__ ptr,
                                                             const int32_t* __restrict__ inv,
                                                             const float* __restrict__ blk,
                                                             const uint8_t* __restrict__ nf, float* __restrict__ val) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= A.n_padded) return;
  const int g = (int)(b >> 5), l = (int)(b & 31);
  const int row = 32 * gslice[g] + l;
  float acc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) acc[k] = 0.f;
  const int c0 = ptr[b], c1 = ptr[b + 1];
  for (int c = c0; c < c1; ++c) {
    const int code = __ldg(inv + c);
    const float* src = blk + (size_t)(code >> 1) * 9;
    float v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] = __ldg(src + k);
    if (code & 1) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) acc[3 * i + j] += v[3 * j + i];
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] += v[k];
    }
  }
  uint8_t fr = 0, fc = 0;
  const int col = A.col_sell[b];
  if (nf && c1 > c0) fr = nf[row], fc = nf[col];
  float* out = val + (size_t)g * 288 + l;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float v = acc[3 * i + j];
      if (((fr >> i) | (fc >> j)) & 1) v = (row == col && i == j) ? 1.f : 0.f;  // getMatrixImpl's Full treatment
      out[32 * (3 * i + j)] = v;
    }
}

template <typename KT, int MODE, int EPB, int MAT = 0>
void launch_disp_epb(const ElemArgs& a, const int32_t* list, int n_list, int e_base, cudaStream_t s) {
  const int blocks = (n_list + EPB - 1) / EPB;
  disp_element_kernel<KT, MODE, EPB, MAT><<<blocks, EPB * 8, 0, s>>>(a, list, n_list, e_base);
}
// assembling modes honour a.epb; element-level outputs (tests, single elements) use 32
template <typename KT, int MODE>
void launch_disp_t(const ElemArgs& a, const int32_t* list, int n_list, int e_base, cudaStream_t s) {
  if (a.material == 1) return launch_disp_epb<KT, MODE, 32, 1>(a, list, n_list, e_base, s);  // SVK: one shape
  if (a.material == 2) return launch_disp_epb<KT, MODE, 32, 2>(a, list, n_list, e_base, s);  // BlatzKo: one shape
  if (a.material == 3) return launch_disp_epb<KT, MODE, 32, 3>(a, list, n_list, e_base, s);  // hyperelastic
  if constexpr ((MODE & kElemOut) == 0) {
    if (a.epb == 16) return launch_disp_epb<KT, MODE, 16>(a, list, n_list, e_base, s);
    if (a.epb == 64) return launch_disp_epb<KT, MODE, 64>(a, list, n_list, e_base, s);
  }
  launch_disp_epb<KT, MODE, 32>(a, list, n_list, e_base, s);
}

}  // namespace

void launch_row_tangent(const ElemArgs& a, const int32_t* ne_ptr, const int32_t* ne_elems, cudaStream_t s) {
  // FP32 only: the FP64 form of this kernel exceeds the register file (the coloured element kernel assembles it)
  row_tangent_kernel<float><<<(a.n_nodes + 127) / 128, 128, 0, s>>>(a, ne_ptr, ne_elems);
}

void launch_disp_element(const ElemArgs& a, int mode, bool fp32_tangent, const int32_t* list, int n_list, int e_base,
                         cudaStream_t s) {
  if (n_list <= 0) return;
  switch (mode) {
    case kWantR:  // assembled residual: Gauss-point-per-lane kernel (its shared exchange fits up to 32 per block)
      if (a.epb == 16) launch_residual_gp<16>(a, list, n_list, e_base, s);
      else launch_residual_gp<32>(a, list, n_list, e_base, s);
      break;
    case kWantR | kWantK: launch_disp_t<double, kWantR | kWantK>(a, list, n_list, e_base, s); break;
    case kWantK:
      if (fp32_tangent) launch_disp_t<float, kWantK>(a, list, n_list, e_base, s);
      else launch_disp_t<double, kWantK>(a, list, n_list, e_base, s);
      break;
    case kWantR | kElemOut: launch_disp_t<double, kWantR | kElemOut>(a, list, n_list, e_base, s); break;
    case kWantK | kElemOut:
      if (fp32_tangent) launch_disp_t<float, kWantK | kElemOut>(a, list, n_list, e_base, s);
      else launch_disp_t<double, kWantK | kElemOut>(a, list, n_list, e_base, s);
      break;
    case kWantEnergy | kElemOut: launch_disp_t<double, kWantEnergy | kElemOut>(a, list, n_list, e_base, s); break;
    case kWantK | kElemBlocks: launch_disp_t<float, kWantK | kElemBlocks>(a, list, n_list, e_base, s); break;
    default: break;
  }
}

void launch_tangent_inverse_count(const int32_t* slot, int n_elems, int32_t* cnt, cudaStream_t s) {
  const int64_t n = 64LL * n_elems;
  if (n > 0) tangent_inv_count_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(slot, n, cnt);
}
void launch_tangent_inverse_fill(const int32_t* slot, int n_elems, const int32_t* ptr, int32_t* cursor, int32_t* inv,
                                 int64_t n_padded, cudaStream_t s) {
  const int64_t n = 64LL * n_elems;
  if (n > 0) tangent_inv_fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(slot, n_elems, ptr, cursor, inv);
  if (n_padded > 0) tangent_inv_sort_kernel<<<(unsigned)((n_padded + 255) / 256), 256, 0, s>>>(ptr, inv, n_padded);
}
void launch_tangent_gather(const Bsr& A, const int32_t* gslice, const int32_t* inv_ptr, const int32_t* inv,
                           const float* blk, const uint8_t* node_fixed, float* val, cudaStream_t s) {
  if (A.n_padded > 0)
    tangent_gather_kernel<<<(unsigned)((A.n_padded + 255) / 256), 256, 0, s>>>(A, gslice, inv_ptr, inv, blk,
                                                                              node_fixed, val);
}

void launch_stress_at(const ElemArgs& a, int e0, int count, const double* xi, bool xi_per_elem, int type, double* out,
                      cudaStream_t s) {
  if (count <= 0) return;
  stress_at_kernel<<<(count + 127) / 128, 128, 0, s>>>(a, e0, count, xi, xi_per_elem ? 1 : 0, type, out);
}

// Gauss-point positions, one thread per element
__global__ void gauss_points_kernel(const double* __restrict__ X, const int32_t* __restrict__ conn, int ne,
                                    double* __restrict__ xgp) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double Xv[8][3];
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const int n = conn[(size_t)v * ne + e];
#pragma unroll
    for (int c = 0; c < 3; ++c) Xv[v][c] = X[3 * (size_t)n + c];
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const double N = (((v ^ q) & 1) ? kGaussLo : kGaussHi) * (((v ^ q) & 2) ? kGaussLo : kGaussHi) *
                       (((v ^ q) & 4) ? kGaussLo : kGaussHi);
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c] += N * Xv[v][c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) xgp[(8 * (size_t)e + q) * 3 + c] = x[c];
  }
}

// VolumeLoad at the element's Gauss rule, one thread per element (adds to ext)
__global__ void volume_load_kernel(const double* __restrict__ X, const int32_t* __restrict__ conn, int ne,
                                   const double* __restrict__ b, double* __restrict__ ext) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double Xv[8][3], acc[24];
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const int n = conn[(size_t)v * ne + e];
#pragma unroll
    for (int c = 0; c < 3; ++c) Xv[v][c] = X[3 * (size_t)n + c];
  }
#pragma unroll
  for (int k = 0; k < 24; ++k) acc[k] = 0.0;
  for (int q = 0; q < 8; ++q) {
    double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      double dxi[3];
      ref_gradient_at_gp<double>(v, q, dxi);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) J[i][j] += Xv[v][i] * dxi[j];
    }
    const double w = kGaussW * det3(J);
    const double* bq = b + (8 * (size_t)e + q) * 3;
    const double b0 = bq[0] * w, b1 = bq[1] * w, b2 = bq[2] * w;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const double N = (((v ^ q) & 1) ? kGaussLo : kGaussHi) * (((v ^ q) & 2) ? kGaussLo : kGaussHi) *
                       (((v ^ q) & 4) ? kGaussLo : kGaussHi);
      acc[3 * v] += N * b0;
      acc[3 * v + 1] += N * b1;
      acc[3 * v + 2] += N * b2;
    }
  }
#pragma unroll
  for (int k = 0; k < 24; ++k) ext[24 * (size_t)e + k] += acc[k];
}

__global__ void add_slot_loads_kernel(const int32_t* __restrict__ slot_elem, int n_slots,
                                      const double* __restrict__ vals, double* __restrict__ ext) {
  const int s = blockIdx.x;
  if (s >= n_slots || threadIdx.x >= 24) return;
  ext[24 * (size_t)slot_elem[s] + threadIdx.x] += vals[24 * (size_t)s + threadIdx.x];
}

void launch_gauss_points(const double* X, const int32_t* conn, int n_elems, double* xgp, cudaStream_t s) {
  if (n_elems > 0) gauss_points_kernel<<<(n_elems + 127) / 128, 128, 0, s>>>(X, conn, n_elems, xgp);
}
void launch_volume_loads(const double* X, const int32_t* conn, int n_elems, const double* b, double* ext,
                         cudaStream_t s) {
  if (n_elems > 0) volume_load_kernel<<<(n_elems + 127) / 128, 128, 0, s>>>(X, conn, n_elems, b, ext);
}
void launch_add_slot_loads(const int32_t* slot_elem, int n_slots, const double* vals, double* ext, cudaStream_t s) {
  if (n_slots > 0) add_slot_loads_kernel<<<n_slots, 32, 0, s>>>(slot_elem, n_slots, vals, ext);
}

void launch_traction_loads(const double* X, const int32_t* conn, int n_elems, int n_slots, const int32_t* slot_elem,
                           const int32_t* face_ptr, const int32_t* face_local, const double* traction, double* trac,
                           cudaStream_t s) {
  if (n_slots <= 0) return;
  traction_kernel<<<(n_slots + 127) / 128, 128, 0, s>>>(X, conn, n_elems, n_slots, slot_elem, face_ptr, face_local,
                                                          traction, trac);
}

}  // namespace ikr
