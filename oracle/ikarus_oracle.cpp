// ikarus_oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// CPU FP64 restatement of the reference (ikarus-project/ikarus v0.4.9) hot path for 3D Q1 hexahedra.
// It is the parity checker for the GPU product and the reported CPU baseline; nothing in the
// product links it.  Every routine names the reference lines it restates.  The reference's
// third-party arithmetic (dune-localfefunctions' Green-Lagrange strain, B-operator and geometric
// stiffness; Dune Q1 geometry and Gauss rules; Eigen's setFromTriplets) is restated from the
// mathematics those call sites document; parity of that part is pinned by the reference's
// end-to-end cantilever goldens (tests/src/testcantileverbeamEAS.cpp:60-96) and by
// finite-difference consistency checks in tests/.
#include "ikarus_oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

namespace {

constexpr int NN = 8;    // nodes per hexahedron
constexpr int ND = 24;   // dofs per hexahedron
constexpr int MAXA = 21; // largest EAS parameter count in 3D (E21)

// Voigt index pairs in the reference order 11,22,33,23,13,12 (tensorutils.hh:180-202).
constexpr int VA[6] = {0, 1, 2, 1, 0, 0};
constexpr int VB[6] = {0, 1, 2, 2, 2, 1};
inline int voigt(int i, int j) {
  if (i == j) return i;
  if (i + j == 3) return 3;  // (1,2)
  if (i + j == 2) return 4;  // (0,2)
  return 5;                  // (0,1)
}

struct M3 {
  double a[3][3];
};

inline double det3(const double m[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
         m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}
inline void inv3(const double m[3][3], double r[3][3], double* detOut = nullptr) {
  const double d = det3(m);
  const double id = 1.0 / d;
  r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * id;
  r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
  r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
  r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * id;
  r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
  r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
  r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * id;
  r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
  r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
  if (detOut) *detOut = d;
}

// Dense LU with partial pivoting on an n x n row-major matrix; solves for nrhs columns of B (row-major n x nrhs).
// Stands in for Eigen's D.inverse() (enhancedassumedstrains.hh:243, 294, 344).
bool lu_solve(int n, std::vector<double> A, double* B, int nrhs) {
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > best) best = std::fabs(A[i * n + k]), p = i;
    if (best == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
      for (int j = 0; j < nrhs; ++j) std::swap(B[k * nrhs + j], B[p * nrhs + j]);
    }
    const double pv = A[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double f = A[i * n + k] / pv;
      if (f == 0.0) continue;
      for (int j = k + 1; j < n; ++j) A[i * n + j] -= f * A[k * n + j];
      for (int j = 0; j < nrhs; ++j) B[i * nrhs + j] -= f * B[k * nrhs + j];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    for (int j = 0; j < nrhs; ++j) {
      double s = B[k * nrhs + j];
      for (int i = k + 1; i < n; ++i) s -= A[k * n + i] * B[i * nrhs + j];
      B[k * nrhs + j] = s / A[k * n + k];
    }
  }
  return true;
}

// Q1 shape functions on the reference cube [0,1]^3 with Dune's vertex numbering:
// vertex v sits at (v&1, (v>>1)&1, (v>>2)&1).
void shape_values(const double xi[3], double N[NN]) {
  for (int v = 0; v < NN; ++v) {
    double p = 1.0;
    for (int d = 0; d < 3; ++d) p *= ((v >> d) & 1) ? xi[d] : 1.0 - xi[d];
    N[v] = p;
  }
}
void shape_gradients(const double xi[3], double dN[NN][3]) {
  for (int v = 0; v < NN; ++v) {
    double f[3], df[3];
    for (int d = 0; d < 3; ++d) {
      const bool b = (v >> d) & 1;
      f[d] = b ? xi[d] : 1.0 - xi[d];
      df[d] = b ? 1.0 : -1.0;
    }
    dN[v][0] = df[0] * f[1] * f[2];
    dN[v][1] = f[0] * df[1] * f[2];
    dN[v][2] = f[0] * f[1] * df[2];
  }
}

// Trilinear geometry at xi: J[i][j] = dx_i/dxi_j, detJ, dN/dX = J^{-T} dN/dxi.
struct Geo {
  double J[3][3], Jinv[3][3], detJ, dNdX[NN][3];
};
void geometry(const double X[NN][3], const double xi[3], Geo& g) {
  double dN[NN][3];
  shape_gradients(xi, dN);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int v = 0; v < NN; ++v) s += X[v][i] * dN[v][j];
      g.J[i][j] = s;
    }
  inv3(g.J, g.Jinv, &g.detJ);
  for (int v = 0; v < NN; ++v)
    for (int k = 0; k < 3; ++k) g.dNdX[v][k] = dN[v][0] * g.Jinv[0][k] + dN[v][1] * g.Jinv[1][k] + dN[v][2] * g.Jinv[2][k];
}

// 2x2x2 Gauss-Legendre rule on [0,1]^3 (defaultQuadratureRule(element, 2*order), nonlinearelastic.hh:124).
struct Rule {
  double xi[8][3];
  double w[8];
};
const Rule& gauss2() {
  static Rule r = [] {
    Rule q{};
    const double a = 0.5 - 0.5 / std::sqrt(3.0), b = 0.5 + 0.5 / std::sqrt(3.0);
    const double p[2] = {a, b};
    int k = 0;
    for (int z = 0; z < 2; ++z)
      for (int y = 0; y < 2; ++y)
        for (int x = 0; x < 2; ++x, ++k) {
          q.xi[k][0] = p[x];
          q.xi[k][1] = p[y];
          q.xi[k][2] = p[z];
          q.w[k] = 0.125;
        }
    return q;
  }();
  return r;
}

// NeoHooke on C = 2E + I (neohooke.hh:78-142, strainconversions.hh:93-97, interface.hh:211-242).
struct MatState {
  double S[6];      // PK2 in Voigt [S11,S22,S33,S23,S13,S12]
  double C6[6][6];  // material tangent in Voigt
  double psi;       // stored energy
  bool ok;
};
void neohooke(double lam, double mu, const double Ev[6], MatState& m, bool wantTangent = true) {
  double C[3][3];
  for (int i = 0; i < 3; ++i) C[i][i] = 2.0 * Ev[i] + 1.0;
  C[1][2] = C[2][1] = Ev[3];
  C[0][2] = C[2][0] = Ev[4];
  C[0][1] = C[1][0] = Ev[5];
  double Ci[3][3], detC;
  inv3(C, Ci, &detC);
  m.ok = detC > 1e-10;  // checkPositiveOrAbort with FloatCmp::le(det, 0, 1e-10)
  const double lnJ = std::log(std::sqrt(detC));
  const double trC = C[0][0] + C[1][1] + C[2][2];
  m.psi = mu / 2.0 * (trC - 3.0 - 2.0 * lnJ) + lam / 2.0 * lnJ * lnJ;
  for (int v = 0; v < 6; ++v) {
    const int i = VA[v], j = VB[v];
    m.S[v] = mu * ((i == j ? 1.0 : 0.0) - Ci[i][j]) + lam * lnJ * Ci[i][j];
  }
  if (!wantTangent) return;
  const double c = mu - lam * lnJ;
  for (int r = 0; r < 6; ++r)
    for (int s = 0; s < 6; ++s) {
      const int i = VA[r], j = VB[r], k = VA[s], l = VB[s];
      m.C6[r][s] = lam * Ci[i][j] * Ci[k][l] + c * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]);
    }
}

// StVenantKirchhoff (svk.hh:63-163): psi = lambda/2 tr(E)^2 + mu E:E, S = lambda tr(E) I + 2 mu E (Voigt shear
// entries mu * 2E_ij, the strain's doubled shears), constant moduli; no determinant check in the reference.
void svk(double lam, double mu, const double Ev[6], MatState& m, bool wantTangent = true) {
  const double trE = Ev[0] + Ev[1] + Ev[2];
  m.ok = true;
  m.psi = lam / 2.0 * trE * trE + mu * (Ev[0] * Ev[0] + Ev[1] * Ev[1] + Ev[2] * Ev[2] +
                                        (Ev[3] * Ev[3] + Ev[4] * Ev[4] + Ev[5] * Ev[5]) / 2.0);
  for (int v = 0; v < 3; ++v) m.S[v] = lam * trE + 2.0 * mu * Ev[v];
  for (int v = 3; v < 6; ++v) m.S[v] = mu * Ev[v];
  if (!wantTangent) return;
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) m.C6[r][c] = (r < 3 && c < 3 ? lam : 0.0) + (r == c ? (r < 3 ? 2.0 * mu : mu) : 0.0);
}
// BlatzKo (hyperelastic/deviatoric/blatzko.hh, makeBlatzKo(mu) in factory.hh:34-39: a deviatoric function of the
// total principal stretches with no volumetric part): W = mu/2 (sum 1/lambda_i^2 + 2 lambda_1 lambda_2 lambda_3 - 5)
// = mu/2 (tr C^-1 + 2 J - 5).  S = 2 dW/dC = mu (J C^-1 - C^-2); C = 2 dS/dC =
// mu [J Ci_ij Ci_kl - J (Ci_ik Ci_jl + Ci_il Ci_jk) + Ci_ik Ci2_jl + Ci_il Ci2_jk + Ci2_ik Ci_jl + Ci2_il Ci_jk].
// The same functions of C as the reference's principal-stretch evaluation (spectral form), without the eigen
// decomposition; det C checked as in Hyperelastic::detF (hyperelastic/interface.hh:249-250).
void blatzko(double mu, const double Ev[6], MatState& m, bool wantTangent = true) {
  double C[3][3];
  for (int i = 0; i < 3; ++i) C[i][i] = 2.0 * Ev[i] + 1.0;
  C[1][2] = C[2][1] = Ev[3];
  C[0][2] = C[2][0] = Ev[4];
  C[0][1] = C[1][0] = Ev[5];
  double Ci[3][3], detC;
  inv3(C, Ci, &detC);
  m.ok = detC > 1e-10;
  const double J = std::sqrt(detC);
  double Ci2[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ci2[i][j] = Ci[i][0] * Ci[0][j] + Ci[i][1] * Ci[1][j] + Ci[i][2] * Ci[2][j];
  m.psi = mu / 2.0 * (Ci[0][0] + Ci[1][1] + Ci[2][2] + 2.0 * J - 5.0);
  for (int v = 0; v < 6; ++v) {
    const int i = VA[v], j = VB[v];
    m.S[v] = mu * (J * Ci[i][j] - Ci2[i][j]);
  }
  if (!wantTangent) return;
  for (int r = 0; r < 6; ++r)
    for (int s = 0; s < 6; ++s) {
      const int i = VA[r], j = VB[r], k = VA[s], l = VB[s];
      m.C6[r][s] = mu * (J * Ci[i][j] * Ci[k][l] - J * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]) +
                         Ci[i][k] * Ci2[j][l] + Ci[i][l] * Ci2[j][k] + Ci2[i][k] * Ci[j][l] + Ci2[i][l] * Ci[j][k]);
    }
}

// ---------------------------------------------------------------------------------------------------------------
// Hyperelastic framework (materials/hyperelastic/): W(C) = W_dev(lambda_1, lambda_2, lambda_3) + K U(J) with the
// principal stretches lambda_i = sqrt(eig_i(C)).
// ---------------------------------------------------------------------------------------------------------------

// Deviatoric invariants W1 = I1 I3^-1/3, W2 = I2 I3^-2/3 of the principal stretches with their first and second
// derivatives (deviatoric/deviatoricinvariants.hh:38-104; invariants I1, I2, I3 materialhelpers.hh:189-201).
struct DevInv {
  double W1, W2, d1[3], d2[3], dd1[3][3], dd2[3][3];
};
void deviatoric_invariants(const double l[3], DevInv& o) {
  const double l2[3] = {l[0] * l[0], l[1] * l[1], l[2] * l[2]};
  const double I1 = l2[0] + l2[1] + l2[2];
  const double I2 = l2[0] * l2[1] + l2[1] * l2[2] + l2[0] * l2[2];
  const double I3 = l2[0] * l2[1] * l2[2];
  const double c1 = std::pow(I3, 1.0 / 3.0), c2 = std::pow(I3, 2.0 / 3.0);
  o.W1 = I1 * std::pow(I3, -1.0 / 3.0);
  o.W2 = I2 * std::pow(I3, -2.0 / 3.0);
  for (int i = 0; i < 3; ++i) {
    o.d1[i] = 2.0 * (3.0 * l2[i] - I1) / (3.0 * l[i] * c1);
    o.d2[i] = -2.0 * (3.0 * I3 / l2[i] - I2) / (3.0 * l[i] * c2);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      if (i == j) {
        o.dd1[i][i] = (2.0 / 9.0) * (5.0 * I1 - 3.0 * l2[i]) / (l2[i] * c1);
        o.dd2[i][i] = (2.0 / 9.0) * (15.0 * I3 / l2[i] - I2) / (l2[i] * c2);
      } else {
        o.dd1[i][j] = (4.0 / 9.0) * (I1 - 3.0 * (l2[i] + l2[j])) / (l[i] * l[j] * c1);
        o.dd2[i][j] = (-4.0 / 9.0) * (2.0 * I2 - 3.0 * l2[i] * l2[j]) / (l[i] * l[j] * c2);
      }
    }
}

// x^p m with the reference's conventions for m = 0 and p = 0 (invariantbased.hh powerAndMultiply)
double pow_times(double x, int p, int m) {
  if (m == 0) return 0.0;
  if (p == 0) return m;
  return std::pow(x, p) * m;
}

// W, dW/dlambda_i and the "second derivative" d2W/dlambda_i dlambda_j - delta_ij (dW/dlambda_i) / lambda_i that each
// deviatoric function returns (secondDerivativeImpl of blatzko.hh, ogden.hh, invariantbased.hh, arrudaboyce.hh,
// gent.hh; the Deviatoric wrapper divides by lambda_i lambda_j, deviatoric/interface.hh:91-118).
struct DevOut {
  double W, dW[3], dS[3][3];
  bool domain_ok;  // Gent: Jm > W1 - 3 (gent.hh checkJm)
};
void deviatoric_function(const orc_hyper& h, const double l[3], DevOut& o) {
  o.W = 0.0;
  o.domain_ok = true;
  for (int i = 0; i < 3; ++i) {
    o.dW[i] = 0.0;
    for (int j = 0; j < 3; ++j) o.dS[i][j] = 0.0;
  }
  const int n = h.n_terms;
  switch (h.deviatoric) {
    case ORC_DEV_NONE: return;
    case ORC_DEV_BLATZKO: {  // blatzko.hh: W = mu/2 (sum lambda_i^-2 + 2 J - 5)
      const double mu = h.mu[0], J = l[0] * l[1] * l[2];
      o.W = mu / 2.0 * (1.0 / (l[0] * l[0]) + 1.0 / (l[1] * l[1]) + 1.0 / (l[2] * l[2]) + 2.0 * J - 5.0);
      for (int i = 0; i < 3; ++i) o.dW[i] = mu * (-1.0 / (l[i] * l[i] * l[i]) + J / l[i]);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const double li2 = l[i] * l[i];
          o.dS[i][j] = mu * (i == j ? (1.0 / li2) * (1.0 / li2 - J) + 3.0 / (li2 * li2) : J / (l[i] * l[j]));
        }
      return;
    }
    case ORC_DEV_OGDEN_TOTAL: {  // ogden.hh: W = sum mu_p / alpha_p (sum_i lambda_i^alpha_p - 3) - mu_p ln J
      const double lnJ = std::log(l[0] * l[1] * l[2]);
      for (int p = 0; p < n; ++p) {
        const double mu = h.mu[p], al = h.alpha[p];
        double s = 0.0;
        for (int i = 0; i < 3; ++i) s += std::pow(l[i], al);
        o.W += mu / al * (s - 3.0) - mu * lnJ;
        for (int i = 0; i < 3; ++i) {
          const double la = std::pow(l[i], al);
          o.dW[i] += mu * (la - 1.0) / l[i];
          o.dS[i][i] += (-2.0 * mu * (la - 1.0) + mu * la * al) / (l[i] * l[i]);
        }
      }
      return;
    }
    case ORC_DEV_OGDEN_DEVIATORIC: {  // ogden.hh with lambda_bar = J^-1/3 lambda (materialhelpers.hh:175-180)
      const double Jm13 = std::pow(l[0] * l[1] * l[2], -1.0 / 3.0);
      const double lb[3] = {Jm13 * l[0], Jm13 * l[1], Jm13 * l[2]};
      double dWdlb[3] = {0.0, 0.0, 0.0}, powsum[ORC_HYPER_MAX_TERMS];
      for (int p = 0; p < n; ++p) {
        powsum[p] = 0.0;
        for (int i = 0; i < 3; ++i) powsum[p] += std::pow(lb[i], h.alpha[p]);
        o.W += h.mu[p] / h.alpha[p] * (powsum[p] - 3.0);
        for (int i = 0; i < 3; ++i) dWdlb[i] += h.mu[p] * std::pow(lb[i], h.alpha[p] - 1.0);
      }
      const double sum = lb[0] * dWdlb[0] + lb[1] * dWdlb[1] + lb[2] * dWdlb[2];
      for (int i = 0; i < 3; ++i) o.dW[i] = (lb[i] * dWdlb[i] - sum / 3.0) / l[i];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          double v = 0.0;
          for (int p = 0; p < n; ++p) {
            const double al = h.alpha[p];
            if (a == b) v += h.mu[p] * al * (std::pow(lb[a], al) / 3.0 + powsum[p] / 9.0);
            else v += h.mu[p] * al * (-(std::pow(lb[a], al) + std::pow(lb[b], al)) / 3.0 + powsum[p] / 9.0);
          }
          v /= l[a] * l[b];
          if (a == b) v -= 2.0 / l[a] * o.dW[a];
          o.dS[a][b] = v;
        }
      return;
    }
    case ORC_DEV_INVARIANT_BASED: {  // invariantbased.hh: W = sum C_p (W1 - 3)^p_p (W2 - 3)^q_p
      DevInv d;
      deviatoric_invariants(l, d);
      const double W1 = d.W1 - 3.0, W2 = d.W2 - 3.0;
      for (int p = 0; p < n; ++p) {
        const int pe = h.p[p], qe = h.q[p];
        const double c = h.mu[p];
        const double W1p = std::pow(W1, pe), W2q = std::pow(W2, qe);
        const double W1pm1p = pow_times(W1, pe - 1, pe), W2qm1q = pow_times(W2, qe - 1, qe);
        const double W1pm2pp = pow_times(W1, pe - 2, pe * (pe - 1)), W2qm2qq = pow_times(W2, qe - 2, qe * (qe - 1));
        o.W += c * W1p * W2q;
        for (int k = 0; k < 3; ++k) o.dW[k] += c * (W1pm1p * W2q * d.d1[k] + W1p * W2qm1q * d.d2[k]);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            const double cross = d.d1[i] * d.d2[j] + d.d1[j] * d.d2[i];
            double v = (W2qm1q * cross + W2q * d.dd1[i][j]) * W1pm1p * c + W2qm1q * d.dd2[i][j] * W1p * c +
                       W1pm2pp * W2q * d.d1[i] * d.d1[j] * c + W2qm2qq * W1p * d.d2[i] * d.d2[j] * c;
            if (i == j) v -= (1.0 / l[i]) * c * (W1pm1p * W2q * d.d1[i] + W1p * W2qm1q * d.d2[i]);
            o.dS[i][j] += v;
          }
      }
      return;
    }
    case ORC_DEV_ARRUDA_BOYCE: {  // arrudaboyce.hh: W = mu sum_p a_p beta^p (W1^(p+1) - 3^(p+1)), beta = lambdaM^-2
      static const double a[5] = {0.5, 1.0 / 20.0, 11.0 / 1050.0, 19.0 / 7000.0, 519.0 / 673750.0};
      DevInv d;
      deviatoric_invariants(l, d);
      const double mu = h.mu[0], beta = 1.0 / (h.param * h.param), W1 = d.W1;
      for (int p = 0; p < 5; ++p) {
        const double f1 = mu * a[p] * std::pow(beta, p);
        o.W += a[p] * std::pow(beta, p) * (std::pow(W1, p + 1) - std::pow(3.0, p + 1));
        for (int k = 0; k < 3; ++k) o.dW[k] += f1 * std::pow(W1, p) * d.d1[k] * (p + 1);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            double v = f1 * (std::pow(W1, p) * d.dd1[i][j] * (p + 1) + std::pow(W1, p - 1) * d.d1[i] * d.d1[j] * p * (p + 1));
            if (i == j) v -= d.d1[i] / l[i] * f1 * std::pow(W1, p) * (p + 1);
            o.dS[i][j] += v;
          }
      }
      o.W *= mu;
      return;
    }
    case ORC_DEV_GENT: {  // gent.hh: W = -mu/2 Jm ln(1 - (W1 - 3) / Jm)
      DevInv d;
      deviatoric_invariants(l, d);
      const double mu = h.mu[0], Jm = h.param, W1 = d.W1;
      // checkJm: FloatCmp::le(Jm, W1 - 3, 1e-14) throws
      const double x = W1 - 3.0;
      if (Jm < x || std::fabs(Jm - x) <= 1e-14 * std::max(std::fabs(Jm), std::fabs(x))) o.domain_ok = false;
      o.W = -(mu / 2.0) * Jm * std::log(1.0 - (W1 - 3.0) / Jm);
      for (int k = 0; k < 3; ++k) o.dW[k] = (mu * d.d1[k] * Jm) / (2.0 * (Jm - W1) + 6.0);
      const double f1 = 1.0 - (W1 - 3.0) / Jm;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double v = (mu / (2.0 * f1)) * (d.dd1[i][j] + (d.d1[i] * d.d1[j] / (f1 * Jm)));
          if (i == j) v -= (mu / (2.0 * l[i] * f1)) * d.d1[i];
          o.dS[i][j] = v;
        }
      return;
    }
    default: o.domain_ok = false;
  }
}

// volumetric functions U(J), U'(J), U''(J) (volumetricfunctions.hh VF0..VF12); Volumetric multiplies them by K
void volumetric_function(int vf, double b, double J, double U[3]) {
  const double lJ = std::log(J);
  switch (vf) {
    case 1: U[0] = 0.5 * (J - 1) * (J - 1), U[1] = J - 1, U[2] = 1; break;
    case 2:
      U[0] = 0.25 * ((J - 1) * (J - 1) + lJ * lJ);
      U[1] = 0.5 * (J - 1 + 1 / J * lJ);
      U[2] = 1 / (2 * J * J) * (1 + J * J - lJ);
      break;
    case 3: U[0] = 0.5 * lJ * lJ, U[1] = 1 / J * lJ, U[2] = 1 / (J * J) * (1 - lJ); break;
    case 4:
      U[0] = (1 / (b * b)) * ((1 / std::pow(J, b)) - 1 + b * lJ);
      U[1] = (1 / b) * ((1 / J) - (1 / std::pow(J, 1 + b)));
      U[2] = (1 / b) * ((1 / std::pow(J, 2 + b)) * (1 + b - std::pow(J, b)));
      break;
    case 5: U[0] = 0.25 * (J * J - 1 - 2 * lJ), U[1] = 0.5 * (J - 1 / J), U[2] = 0.5 * (1 + 1 / (J * J)); break;
    case 6: U[0] = J - lJ - 1, U[1] = 1 - 1 / J, U[2] = 1 / (J * J); break;
    case 7:
      U[0] = std::pow(J, b) * (b * lJ - 1) + 1;
      U[1] = b * b * (1.0 / std::pow(J, 1.0 - b)) * lJ;
      U[2] = b * b * std::pow(J, b - 2.0) * (1 + (b - 1) * lJ);
      break;
    case 8: U[0] = J * lJ - J + 1, U[1] = lJ, U[2] = 1 / J; break;
    case 9:
      U[0] = (1.0 / 32.0) * (J * J - 1 / (J * J)) * (J * J - 1 / (J * J));
      U[1] = (1.0 / 8.0) * (std::pow(J, 3) - 1.0 / std::pow(J, 5));
      U[2] = (1.0 / 8.0) * (5.0 * std::pow(J, -6) + 3.0 * J * J);
      break;
    case 10:
      U[0] = (J / b) * (1 - (std::pow(J, -b) / (1 - b))) + (1.0 / (b - 1));
      U[1] = (1 / b) * (1 - std::pow(J, -b));
      U[2] = std::pow(J, -1 - b);
      break;
    case 11:
      U[0] = (1.0 / 50.0) * (std::pow(J, 5.0) + std::pow(J, -5.0) - 2.0);
      U[1] = (1.0 / 10.0) * (std::pow(J, 4.0) - std::pow(J, -6.0));
      U[2] = (1.0 / 10.0) * (4 * std::pow(J, 3.0) + 6 * std::pow(J, -7.0));
      break;
    case 12: U[0] = J - 1, U[1] = 1, U[2] = 0; break;
    default: U[0] = U[1] = U[2] = 0; break;  // VF0
  }
}

// Eigen decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations (Jacobi 1846; Golub & Van Loan,
// "Matrix Computations", sec. 8.5: the stable choice t = sign(theta) / (|theta| + sqrt(theta^2 + 1))).  The
// reference calls Eigen's SelfAdjointEigenSolver (materialhelpers.hh:139-152), whose algorithm is not part of the
// reference; any backward-stable solver gives the same stresses and moduli up to rounding, since these are
// functions of C alone.  Eigenvalues ascending (as Eigen returns them), eigenvectors in the columns of V.
void sym_eig3(const double A[3][3], double ev[3], double V[3][3]) {
  double a[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      a[i][j] = A[i][j];
      V[i][j] = i == j ? 1.0 : 0.0;
    }
  static const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
  for (int sweep = 0; sweep < 32; ++sweep) {
    if (a[0][1] == 0.0 && a[0][2] == 0.0 && a[1][2] == 0.0) break;
    for (int r = 0; r < 3; ++r) {
      const int p = P[r], q = Q[r];
      const double apq = a[p][q];
      if (apq == 0.0) continue;
      if (std::fabs(a[p][p]) + 100.0 * std::fabs(apq) == std::fabs(a[p][p]) &&
          std::fabs(a[q][q]) + 100.0 * std::fabs(apq) == std::fabs(a[q][q])) {
        a[p][q] = a[q][p] = 0.0;  // below the diagonal's resolution
        continue;
      }
      const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
      double t = 1.0 / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      if (std::fabs(theta) > 1e150) t = 0.5 / std::fabs(theta);
      if (theta < 0.0) t = -t;
      const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
      const int o = 3 - p - q;  // the third index
      const double aop = a[o][p], aoq = a[o][q];
      a[p][p] -= t * apq;
      a[q][q] += t * apq;
      a[p][q] = a[q][p] = 0.0;
      a[o][p] = a[p][o] = c * aop - s * aoq;
      a[o][q] = a[q][o] = s * aop + c * aoq;
      for (int k = 0; k < 3; ++k) {
        const double vkp = V[k][p], vkq = V[k][q];
        V[k][p] = c * vkp - s * vkq;
        V[k][q] = s * vkp + c * vkq;
      }
    }
  }
  for (int i = 0; i < 3; ++i) ev[i] = a[i][i];
  // ascending order, columns of V along
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (ev[j] > ev[j + 1]) {
        std::swap(ev[j], ev[j + 1]);
        for (int k = 0; k < 3; ++k) std::swap(V[k][j], V[k][j + 1]);
      }
}

// Hyperelastic::stressesImpl / tangentModuliImpl / storedEnergyImpl (hyperelastic/interface.hh:106-160, 180-214):
// S = sum_i (dW_i / lambda_i) N_i (x) N_i + J U' C^-1; moduli = sum_ik L_iikk (N_i N_i)(N_k N_k) +
// sum_{i != k} L_ikik (N_i N_k)(N_i N_k + N_k N_i) + J (U' + J U'') C^-1 (x) C^-1 - J U' (C^-1 (.) C^-1 sym), with
// L_iikk = dS_ik / (lambda_i lambda_k) and L_ikik = (S_i - S_k) / (lambda_i^2 - lambda_k^2), or
// (L_iiii - L_iikk) / 2 for equal stretches (FloatCmp::eq with 1e-8; deviatoric/interface.hh:91-118).
void hyperelastic(const orc_hyper& h, const double Ev[6], MatState& m, bool wantTangent, bool* domain_ok = nullptr) {
  double C[3][3];
  for (int i = 0; i < 3; ++i) C[i][i] = 2.0 * Ev[i] + 1.0;
  C[1][2] = C[2][1] = Ev[3];
  C[0][2] = C[2][0] = Ev[4];
  C[0][1] = C[1][0] = Ev[5];
  double ev[3], N[3][3];
  sym_eig3(C, ev, N);
  const double l[3] = {std::sqrt(ev[0]), std::sqrt(ev[1]), std::sqrt(ev[2])};
  const double J = l[0] * l[1] * l[2];  // detF from the principal values (interface.hh:245-253)
  m.ok = J * J > 1e-10 && J > 0.0;
  DevOut d;
  deviatoric_function(h, l, d);
  if (domain_ok) *domain_ok = d.domain_ok;
  double U[3];
  volumetric_function(h.volumetric, h.beta, J, U);
  const double K = h.K;
  m.psi = d.W + K * U[0];
  double Ci[3][3];
  inv3(C, Ci);
  const double Sp[3] = {d.dW[0] / l[0], d.dW[1] / l[1], d.dW[2] / l[2]};
  // Voigt dyads of the principal directions: nn[i][v] = N_Ai N_Bi
  double nn[3][6];
  for (int v = 0; v < 6; ++v)
    for (int i = 0; i < 3; ++i) nn[i][v] = N[VA[v]][i] * N[VB[v]][i];
  const double vs = J * K * U[1];
  for (int v = 0; v < 6; ++v) m.S[v] = Sp[0] * nn[0][v] + Sp[1] * nn[1][v] + Sp[2] * nn[2][v] + vs * Ci[VA[v]][VB[v]];
  if (!wantTangent) return;
  double L[3][3], Lo[3][3];  // L_iikk and, off the diagonal, L_ikik
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) L[i][k] = d.dS[i][k] / (l[i] * l[k]);
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      if (i == k) {
        Lo[i][k] = 0.0;
        continue;
      }
      if (std::fabs(l[i] - l[k]) <= 1e-8 * std::max(std::fabs(l[i]), std::fabs(l[k])))
        Lo[i][k] = 0.5 * (L[i][i] - L[i][k]);
      else Lo[i][k] = (Sp[i] - Sp[k]) / (l[i] * l[i] - l[k] * l[k]);
    }
  const double v1 = J * K * (U[1] + J * U[2]), v2 = J * K * U[1];
  for (int r = 0; r < 6; ++r)
    for (int s = 0; s < 6; ++s) {
      const int A = VA[r], B = VB[r], Cc = VA[s], D = VB[s];
      double c = 0.0;
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
          c += L[i][k] * nn[i][r] * nn[k][s];
          if (i != k) c += Lo[i][k] * N[A][i] * N[B][k] * (N[Cc][i] * N[D][k] + N[Cc][k] * N[D][i]);
        }
      c += v1 * Ci[A][B] * Ci[Cc][D] - v2 * (Ci[A][Cc] * Ci[B][D] + Ci[A][D] * Ci[B][Cc]);
      m.C6[r][s] = c;
    }
}

void material_law(int material, double lam, double mu, const orc_hyper* h, const double Ev[6], MatState& m,
                  bool wantTangent = true) {
  if (material == ORC_MATERIAL_SVK) svk(lam, mu, Ev, m, wantTangent);
  else if (material == ORC_MATERIAL_BLATZKO) blatzko(mu, Ev, m, wantTangent);
  else if (material == ORC_MATERIAL_HYPERELASTIC) {
    bool dom = true;
    hyperelastic(*h, Ev, m, wantTangent, &dom);
    if (!dom) m.ok = false;
  } else neohooke(lam, mu, Ev, m, wantTangent);
}

// Green-Lagrange strain of a displacement gradient, Voigt with doubled shears
// (dune-localfefunctions greenLagrangeStrains; easfunctions/displacementgradient.hh:86-87).
void gl_strain(const double H[3][3], double Ev[6]) {
  double E[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double hh = 0;
      for (int k = 0; k < 3; ++k) hh += H[k][i] * H[k][j];
      E[i][j] = 0.5 * (H[i][j] + H[j][i] + hh);
    }
  for (int v = 0; v < 6; ++v) Ev[v] = (v < 3 ? 1.0 : 2.0) * E[VA[v]][VB[v]];
}

// B-operator row layout of the Green-Lagrange strain variation w.r.t. node displacement
// (easfunctions/displacementgradient.hh:129-146): g_k = F e_k, dN = nodal gradient.
void bop(const double F[3][3], const double dN[3], double B[6][3]) {
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

// Strain transformation matrix of tensorutils.hh:438-465 written from its defining rule:
// T[(a,b)][(c,d)] = (a==b ? 1/2 : 1) * (Jt[a][c] Jt[b][d] + Jt[b][c] Jt[a][d]) with Jt = J^T.
void transformation_matrix(const double J[3][3], double T[6][6]) {
  for (int r = 0; r < 6; ++r)
    for (int s = 0; s < 6; ++s) {
      const int a = VA[r], b = VB[r], c = VA[s], d = VB[s];
      const double v = J[c][a] * J[d][b] + J[c][b] * J[d][a];
      T[r][s] = (a == b) ? 0.5 * v : v;
    }
}

// E9 / E21 ansatz before transformation (easvariants/linearandglstrains.hh:252-327):
// each entry is (row, column, product of the listed (2 xi_k - 1) factors).
struct AnsatzEntry {
  int row, col, f1, f2;  // f2 = -1 for a single factor
};
constexpr AnsatzEntry kE21[] = {
    {0, 0, 0, -1},  {1, 1, 1, -1},  {2, 2, 2, -1},  {3, 3, 1, -1},  {3, 4, 2, -1},  {4, 5, 0, -1},
    {4, 6, 2, -1},  {5, 7, 0, -1},  {5, 8, 1, -1},  {3, 9, 0, 1},   {3, 10, 0, 2},  {4, 11, 0, 1},
    {4, 12, 1, 2},  {5, 13, 0, 2},  {5, 14, 1, 2},  {0, 15, 0, 1},  {0, 16, 0, 2},  {1, 17, 0, 1},
    {1, 18, 1, 2},  {2, 19, 0, 2},  {2, 20, 1, 2}};

}  // namespace

struct orc_problem {
  int nn = 0, ne = 0;
  std::vector<double> X;      // nn*3
  std::vector<int32_t> conn;  // ne*8
  double lam = 0, mu = 0;
  int material = 0;  // ORC_MATERIAL_*
  orc_hyper hyper{};  // the functions of ORC_MATERIAL_HYPERELASTIC
  int eas = 0, na = 0;
  bool faithful = false;
  std::vector<uint8_t> fixed;   // n dofs
  std::vector<double> alpha;    // ne*na
  // Neumann faces grouped per element
  std::vector<std::vector<std::pair<int, std::array<double, 3>>>> faces;
  // loads given as functions f(X, lambda): volume loads on every element, Neumann faces with a function
  struct PointFn {
    orc_point_fn f;
    void* user;
  };
  std::vector<PointFn> volume_fns;
  std::vector<std::vector<std::pair<int, PointFn>>> fn_faces;  // per element: (local face, function)
  std::vector<int32_t> pl_dof;
  std::vector<double> pl_val;
  // inhomogeneous Dirichlet values u_D(lambda) = lambda * idbc_rate on constrained dofs (empty: none); with a value
  // function, u_D(lambda) = idbc_value(X, lambda) interpolated at every node and idbc_rate its lambda-derivative at 1
  std::vector<double> idbc_rate;
  orc_point_fn idbc_value = nullptr;
  void* idbc_user = nullptr;
  // u_D at the load factor into v (n dofs)
  void idbc_values(double lambda, std::vector<double>& v) const {
    v.assign(3 * (size_t)nn, 0.0);
    if (idbc_value) idbc_value(nn, X.data(), lambda, v.data(), idbc_user);
    else
      for (size_t i = 0; i < v.size(); ++i) v[i] = lambda * idbc_rate[i];
  }
  // pattern caches
  std::vector<std::vector<int32_t>> nodeAdj;
  int ndof() const { return 3 * nn; }
};

namespace {

struct ElemOut {
  double f[ND];
  double K[ND][ND];
  double D[MAXA * MAXA];
  double L[MAXA * ND];
  double Rt[MAXA];
  double energy;
  bool ok;
};

void gather(const orc_problem& p, int e, const double* u, double X[NN][3], double ue[NN][3]) {
  for (int v = 0; v < NN; ++v) {
    const int n = p.conn[8 * e + v];
    for (int c = 0; c < 3; ++c) {
      X[v][c] = p.X[3 * n + c];
      ue[v][c] = u ? u[3 * n + c] : 0.0;
    }
  }
}

// Element-centre data of the enhanced-strain ansatz (helperfunctions.hh:19-36, linearandglstrains.hh:238-250,
// displacementgradienttransposed.hh:336-369): centre geometry, T0^{-1} / detJ0 (GL), J0^{-T} (H, HT) and the
// compatible deformation gradient at the centre (HT).
struct EasCentre {
  Geo g0;
  double T0inv[6][6] = {};
  double JIT0[3][3];
  double Fc0[3][3];
};
void eas_centre(int kind, const double X[NN][3], const double ue[NN][3], EasCentre& ec) {
  const double xc[3] = {0.5, 0.5, 0.5};
  geometry(X, xc, ec.g0);
  const Geo& g0 = ec.g0;
  if (kind == ORC_EAS_GL) {
    double T[6][6];
    transformation_matrix(g0.J, T);
    std::vector<double> A(36), B(36, 0.0);
    for (int r = 0; r < 6; ++r)
      for (int s = 0; s < 6; ++s) A[r * 6 + s] = T[r][s] * g0.detJ;
    for (int r = 0; r < 6; ++r) B[r * 6 + r] = 1.0;
    lu_solve(6, A, B.data(), 6);
    for (int r = 0; r < 6; ++r)
      for (int s = 0; s < 6; ++s) ec.T0inv[r][s] = B[r * 6 + s];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ec.JIT0[i][j] = g0.Jinv[j][i];  // jacobianInverseTransposed at the centre
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = (i == j) ? 1.0 : 0.0;
      for (int v = 0; v < NN; ++v) s += ue[v][i] * g0.dNdX[v][j];
      ec.Fc0[i][j] = s;
    }
}

// Enhanced-strain element at the current (u, alpha): internal force, tangent, D, L, R~ and energy.
// Restates NonLinearElastic::calculate{Vector,Matrix}Impl (nonlinearelastic.hh:375-430) and
// EnhancedAssumedStrains::calculate{Vector,Matrix}Impl / calculateDAndLMatrix / calculateRtilde
// (enhancedassumedstrains.hh:258-434) with the strain functions of easfunctions/*.hh.
void element_internal(const orc_problem& p, int e, const double* u, bool wantK, ElemOut& out) {
  double X[NN][3], ue[NN][3];
  gather(p, e, u, X, ue);
  const int na = p.na;
  const int kind = na > 0 ? p.eas : ORC_EAS_NONE;
  const double* al = na > 0 ? &p.alpha[(size_t)e * na] : nullptr;
  std::memset(&out, 0, sizeof(out));
  out.ok = true;

  // centre data (helperfunctions.hh:19-36, displacementgradienttransposed.hh:336-369)
  EasCentre ec;
  eas_centre(kind, X, ue, ec);
  const Geo& g0 = ec.g0;
  const auto& T0inv = ec.T0inv;
  const auto& JIT0 = ec.JIT0;
  const auto& Fc0 = ec.Fc0;

  const Rule& R = gauss2();
  for (int q = 0; q < 8; ++q) {
    Geo g;
    geometry(X, R.xi[q], g);
    const double wdJ = R.w[q] * g.detJ;
    double Hc[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0;
        for (int v = 0; v < NN; ++v) s += ue[v][i] * g.dNdX[v][j];
        Hc[i][j] = s;
      }

    // EAS ansatz at this Gauss point
    double M[6][MAXA] = {};      // GL: E~ = M alpha
    double Hp[MAXA][3][3] = {};  // H, HT: enhancement matrices (transformed)
    if (kind == ORC_EAS_GL) {
      double M0[6][MAXA] = {};
      for (int k = 0; k < na; ++k) {
        const AnsatzEntry& a = kE21[k];
        double v = 2.0 * R.xi[q][a.f1] - 1.0;
        if (a.f2 >= 0) v *= 2.0 * R.xi[q][a.f2] - 1.0;
        M0[a.row][a.col] = v;
      }
      for (int r = 0; r < 6; ++r)
        for (int k = 0; k < na; ++k) {
          double s = 0;
          for (int t = 0; t < 6; ++t) s += T0inv[r][t] * M0[t][k];
          M[r][k] = s / g.detJ;
        }
    } else if (kind == ORC_EAS_H || kind == ORC_EAS_HT) {
      // H9 (easvariants/displacementgradient.hh:136-161): mode p = 3r+c has entry (r,c) = 2 xi_c - 1,
      // transformed by (detJ0/detJ) J0^{-T} H J0^{-1} (helperfunctions.hh:27-36).
      const double sc = g0.detJ / g.detJ;
      for (int pm = 0; pm < na; ++pm) {
        const int r = pm / 3, c = pm % 3;
        const double val = 2.0 * R.xi[q][c] - 1.0;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Hp[pm][i][j] = sc * JIT0[i][r] * val * JIT0[j][c];
      }
    }

    // displacement gradient actually used, F, modified nodal gradients
    double H[3][3];
    std::memcpy(H, Hc, sizeof(H));
    double Ht[3][3] = {};  // sum_p alpha_p H_p
    if (kind == ORC_EAS_H || kind == ORC_EAS_HT) {
      for (int pm = 0; pm < na; ++pm)
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Ht[i][j] += Hp[pm][i][j] * al[pm];
      if (kind == ORC_EAS_H) {
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) H[i][j] += Ht[i][j];
      } else {  // H = Hc + Fc0 Ht^T (displacementgradienttransposed.hh:353-368)
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += Fc0[i][k] * Ht[j][k];
            H[i][j] += s;
          }
      }
    }
    double F[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
    double Ev[6];
    gl_strain(H, Ev);
    if (kind == ORC_EAS_GL)
      for (int r = 0; r < 6; ++r)
        for (int k = 0; k < na; ++k) Ev[r] += M[r][k] * al[k];

    MatState m;
    material_law(p.material, p.lam, p.mu, &p.hyper, Ev, m, true);
    if (!m.ok) out.ok = false;
    out.energy += m.psi * wdJ;
    double Smat[3][3];
    for (int v = 0; v < 6; ++v) Smat[VA[v]][VB[v]] = Smat[VB[v]][VA[v]] = m.S[v];

    // nodal gradients entering B and kg (HT modifies them: displacementgradienttransposed.hh:126-140)
    double dN[NN][3];
    for (int v = 0; v < NN; ++v)
      for (int k = 0; k < 3; ++k) {
        dN[v][k] = g.dNdX[v][k];
        if (kind == ORC_EAS_HT)
          dN[v][k] += Ht[k][0] * g0.dNdX[v][0] + Ht[k][1] * g0.dNdX[v][1] + Ht[k][2] * g0.dNdX[v][2];
      }
    double B[NN][6][3];
    for (int v = 0; v < NN; ++v) bop(F, dN[v], B[v]);

    // internal forces f_I += B_I^T S w detJ (nonlinearelastic.hh:335-342)
    for (int v = 0; v < NN; ++v)
      for (int a = 0; a < 3; ++a) {
        double s = 0;
        for (int r = 0; r < 6; ++r) s += B[v][r][a] * m.S[r];
        out.f[3 * v + a] += s * wdJ;
      }

    if (wantK) {
      // K_IJ += (B_I^T C B_J + kg_IJ) w detJ (nonlinearelastic.hh:294-322, 387-398)
      for (int I = 0; I < NN; ++I)
        for (int Jn = 0; Jn < NN; ++Jn) {
          MatState mm;
          const MatState* mp = &m;
          if (p.faithful) {  // the reference evaluates the moduli inside the (i,j) loop
            material_law(p.material, p.lam, p.mu, &p.hyper, Ev, mm, true);
            mp = &mm;
          }
          double CB[6][3];
          for (int r = 0; r < 6; ++r)
            for (int b = 0; b < 3; ++b) {
              double s = 0;
              for (int t = 0; t < 6; ++t) s += mp->C6[r][t] * B[Jn][t][b];
              CB[r][b] = s;
            }
          double kg = 0;
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) kg += dN[I][i] * Smat[i][j] * dN[Jn][j];
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
              double s = 0;
              for (int r = 0; r < 6; ++r) s += B[I][r][a] * CB[r][b];
              if (a == b) s += kg;
              out.K[3 * I + a][3 * Jn + b] += s * wdJ;
            }
        }
    }

    if (na > 0) {
      // E_alpha (6 x na)
      double Ea[6][MAXA] = {};
      double Haux[MAXA][3][3];  // H~_p used by H / HT
      if (kind == ORC_EAS_GL) {
        std::memcpy(Ea, M, sizeof(Ea));
      } else {
        for (int pm = 0; pm < na; ++pm) {
          if (kind == ORC_EAS_H) {
            std::memcpy(Haux[pm], Hp[pm], sizeof(Haux[pm]));
          } else {  // Fc0 H_p^T (displacementgradienttransposed.hh:155-158)
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int k = 0; k < 3; ++k) s += Fc0[i][k] * Hp[pm][j][k];
                Haux[pm][i][j] = s;
              }
          }
          // M(v,p) = sym(F^T Haux_p) in Voigt (displacementgradient.hh:153-166)
          const double(*h)[3] = Haux[pm];
          auto col_dot = [&](int ci, int gj) { return h[0][ci] * F[0][gj] + h[1][ci] * F[1][gj] + h[2][ci] * F[2][gj]; };
          Ea[0][pm] = col_dot(0, 0);
          Ea[1][pm] = col_dot(1, 1);
          Ea[2][pm] = col_dot(2, 2);
          Ea[3][pm] = col_dot(2, 1) + col_dot(1, 2);
          Ea[4][pm] = col_dot(2, 0) + col_dot(0, 2);
          Ea[5][pm] = col_dot(1, 0) + col_dot(0, 1);
        }
      }
      // C Ea
      double CEa[6][MAXA];
      for (int r = 0; r < 6; ++r)
        for (int k = 0; k < na; ++k) {
          double s = 0;
          for (int t = 0; t < 6; ++t) s += m.C6[r][t] * Ea[t][k];
          CEa[r][k] = s;
        }
      // D += (Ea^T C Ea + E_aa) w detJ (enhancedassumedstrains.hh:400)
      for (int a = 0; a < na; ++a)
        for (int b = 0; b < na; ++b) {
          double s = 0;
          for (int r = 0; r < 6; ++r) s += Ea[r][a] * CEa[r][b];
          if (kind != ORC_EAS_GL) {  // E_aa (displacementgradient.hh:213-230)
            double kgab = 0;
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j) {
                const double sij = 0.5 * Smat[i][j];
                double c1 = 0, c2 = 0;
                for (int k = 0; k < 3; ++k) {
                  c1 += Haux[a][k][i] * Haux[b][k][j];
                  c2 += Haux[a][k][j] * Haux[b][k][i];
                }
                kgab += sij * (c1 + c2);
              }
            s += kgab;
          }
          out.D[a * na + b] += s * wdJ;
        }
      // R~ += Ea^T S w detJ (enhancedassumedstrains.hh:428)
      for (int a = 0; a < na; ++a) {
        double s = 0;
        for (int r = 0; r < 6; ++r) s += Ea[r][a] * m.S[r];
        out.Rt[a] += s * wdJ;
      }
      // L(:, 3I..3I+2) += (Ea^T C B_I + E_ad) w detJ (enhancedassumedstrains.hh:401-408)
      for (int I = 0; I < NN; ++I)
        for (int a = 0; a < na; ++a)
          for (int b = 0; b < 3; ++b) {
            double s = 0;
            for (int r = 0; r < 6; ++r) s += CEa[r][a] * B[I][r][b];
            if (kind == ORC_EAS_H) {  // displacementgradient.hh:231-254
              double kad = 0;
              for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                  kad += 0.5 * Smat[i][j] * (Haux[a][b][i] * g.dNdX[I][j] + Haux[a][b][j] * g.dNdX[I][i]);
              s += kad;
            } else if (kind == ORC_EAS_HT) {  // displacementgradienttransposed.hh:272-319
              double hv[3];  // H_a dN0_I
              for (int i = 0; i < 3; ++i)
                hv[i] = Hp[a][i][0] * g0.dNdX[I][0] + Hp[a][i][1] * g0.dNdX[I][1] + Hp[a][i][2] * g0.dNdX[I][2];
              double kad = 0;
              for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                  kad += 0.5 * Smat[i][j] *
                         (Haux[a][b][i] * dN[I][j] + Haux[a][b][j] * dN[I][i] + hv[i] * F[b][j] + hv[j] * F[b][i]);
              s += kad;
            }
            out.L[a * ND + 3 * I + b] += s * wdJ;
          }
    }
  }
}

// Dead traction on the element's Neumann faces, 1-point rule (loads/traction.hh:105-138): lambda t for the faces
// with fixed values, f(X_quadrature point, lambda) for the faces with a function.
void element_traction(const orc_problem& p, int e, double lambda, double f[ND], const double* u, double* energy) {
  const bool fixed_faces = !p.faces.empty() && !p.faces[e].empty();
  const bool fn_faces = !p.fn_faces.empty() && !p.fn_faces[e].empty();
  if (!fixed_faces && !fn_faces) return;
  double X[NN][3], ue[NN][3];
  gather(p, e, u, X, ue);
  std::vector<std::pair<int, std::array<double, 3>>> list;
  if (fixed_faces)
    for (const auto& fc : p.faces[e])
      list.push_back({fc.first, {lambda * fc.second[0], lambda * fc.second[1], lambda * fc.second[2]}});
  if (fn_faces)
    for (const auto& ff : p.fn_faces[e]) {
      const int d = ff.first / 2;
      double xi[3] = {0.5, 0.5, 0.5};
      xi[d] = (ff.first % 2) ? 1.0 : 0.0;
      double N[NN], Xq[3] = {0, 0, 0}, t[3];
      shape_values(xi, N);
      for (int v = 0; v < NN; ++v)
        for (int c = 0; c < 3; ++c) Xq[c] += N[v] * X[v][c];
      ff.second.f(1, Xq, lambda, t, ff.second.user);
      list.push_back({ff.first, {t[0], t[1], t[2]}});
    }
  for (const auto& fc : list) {
    const int lf = fc.first;
    const int d = lf / 2;
    double xi[3] = {0.5, 0.5, 0.5};
    xi[d] = (lf % 2) ? 1.0 : 0.0;
    double N[NN], dN[NN][3];
    shape_values(xi, N);
    shape_gradients(xi, dN);
    int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
    double a[3], b[3];
    for (int c = 0; c < 3; ++c) {
      a[c] = b[c] = 0;
      for (int v = 0; v < NN; ++v) a[c] += X[v][c] * dN[v][t1], b[c] += X[v][c] * dN[v][t2];
    }
    const double cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const double dA = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    const double t[3] = {fc.second[0], fc.second[1], fc.second[2]};
    if (f)
      for (int v = 0; v < NN; ++v)
        for (int c = 0; c < 3; ++c) f[3 * v + c] -= N[v] * t[c] * 1.0 * dA;
    if (energy) {
      double uv[3] = {0, 0, 0};
      for (int v = 0; v < NN; ++v)
        for (int c = 0; c < 3; ++c) uv[c] += N[v] * ue[v][c];
      *energy -= (t[0] * uv[0] + t[1] * uv[1] + t[2] * uv[2]) * dA;
    }
  }
}

// VolumeLoad (loads/volume.hh:86-106): f_I -= N_I b(X(xi_q), lambda) w_q detJ(xi_q) over the element's Gauss rule,
// energy -= u(xi_q) . b w_q detJ (:63-80).
void element_volume_load(const orc_problem& p, int e, double lambda, double f[ND], const double* u, double* energy) {
  if (p.volume_fns.empty()) return;
  double X[NN][3], ue[NN][3];
  gather(p, e, u, X, ue);
  const Rule& R = gauss2();
  for (int q = 0; q < 8; ++q) {
    Geo g;
    geometry(X, R.xi[q], g);
    double N[NN], Xq[3] = {0, 0, 0}, uq[3] = {0, 0, 0};
    shape_values(R.xi[q], N);
    for (int v = 0; v < NN; ++v)
      for (int c = 0; c < 3; ++c) Xq[c] += N[v] * X[v][c], uq[c] += N[v] * ue[v][c];
    const double wdJ = R.w[q] * g.detJ;
    for (const auto& vf : p.volume_fns) {
      double b[3];
      vf.f(1, Xq, lambda, b, vf.user);
      if (f)
        for (int v = 0; v < NN; ++v)
          for (int c = 0; c < 3; ++c) f[3 * v + c] -= N[v] * b[c] * wdJ;
      if (energy) *energy -= (uq[0] * b[0] + uq[1] * b[1] + uq[2] * b[2]) * wdJ;
    }
  }
}

// Condensed element vector / matrix (enhancedassumedstrains.hh:291-296, 336-345).
int element_vector(const orc_problem& p, int e, const double* u, double lambda, double out[ND]) {
  ElemOut eo;
  element_internal(p, e, u, false, eo);
  if (!eo.ok) return ORC_ERR_NONPOSITIVE_DETC;
  std::memcpy(out, eo.f, sizeof(eo.f));
  const int na = p.na;
  if (na > 0) {
    std::vector<double> Dm(eo.D, eo.D + na * na), y(eo.Rt, eo.Rt + na);
    if (!lu_solve(na, Dm, y.data(), 1)) return ORC_ERR_SINGULAR;
    for (int k = 0; k < ND; ++k) {
      double s = 0;
      for (int a = 0; a < na; ++a) s += eo.L[a * ND + k] * y[a];
      out[k] -= s;
    }
  }
  element_traction(p, e, lambda, out, nullptr, nullptr);
  element_volume_load(p, e, lambda, out, nullptr, nullptr);
  return ORC_OK;
}

int element_matrix(const orc_problem& p, int e, const double* u, double K[ND][ND]) {
  static thread_local ElemOut eo;
  element_internal(p, e, u, true, eo);
  if (!eo.ok) return ORC_ERR_NONPOSITIVE_DETC;
  std::memcpy(K, eo.K, sizeof(eo.K));
  const int na = p.na;
  if (na > 0) {
    std::vector<double> Dm(eo.D, eo.D + na * na), Y(eo.L, eo.L + na * ND);
    if (!lu_solve(na, Dm, Y.data(), ND)) return ORC_ERR_SINGULAR;
    for (int r = 0; r < ND; ++r)
      for (int c = r; c < ND; ++c) {
        double s = 0;
        for (int a = 0; a < na; ++a) s += eo.L[a * ND + r] * Y[a * ND + c];
        K[r][c] -= s;
      }
    for (int r = 0; r < ND; ++r)
      for (int c = 0; c < r; ++c) K[r][c] = K[c][r];
  }
  return ORC_OK;
}

// sparsity: node adjacency (nodes sharing an element), sorted
void build_adjacency(orc_problem& p) {
  if (!p.nodeAdj.empty()) return;
  p.nodeAdj.assign(p.nn, {});
  for (int e = 0; e < p.ne; ++e)
    for (int a = 0; a < NN; ++a)
      for (int b = 0; b < NN; ++b) p.nodeAdj[p.conn[8 * e + a]].push_back(p.conn[8 * e + b]);
  for (auto& v : p.nodeAdj) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
}

std::vector<int32_t> constraints_below(const orc_problem& p) {
  // FlatAssemblerBase ctor (assembler/interface.hh:50-62)
  std::vector<int32_t> cb(p.ndof());
  int32_t c = 0;
  for (int i = 0; i < p.ndof(); ++i) {
    cb[i] = c;
    if (p.fixed[i]) ++c;
  }
  return cb;
}

struct CSC {
  int n = 0;
  std::vector<int64_t> cp;
  std::vector<int32_t> ri;
  std::vector<double> v;
};

// createOccupationPattern / createReducedOccupationPattern + setFromTriplets (simpleassemblers.inl:206-251):
// column-major, row indices sorted, duplicates merged.
void build_pattern(orc_problem& p, int dbc, CSC& A) {
  build_adjacency(p);
  const bool red = dbc == ORC_DBC_REDUCED;
  auto cb = constraints_below(p);
  const int n = red ? p.ndof() - (p.ndof() ? cb[p.ndof() - 1] + p.fixed[p.ndof() - 1] : 0) : p.ndof();
  A.n = n;
  A.cp.assign(n + 1, 0);
  A.ri.clear();
  for (int J = 0; J < p.nn; ++J)
    for (int b = 0; b < 3; ++b) {
      const int gc = 3 * J + b;
      if (red && p.fixed[gc]) continue;
      for (int I : p.nodeAdj[J])
        for (int a = 0; a < 3; ++a) {
          const int gr = 3 * I + a;
          if (red && p.fixed[gr]) continue;
          A.ri.push_back(red ? gr - cb[gr] : gr);
        }
      const int col = red ? gc - cb[gc] : gc;
      A.cp[col + 1] = (int64_t)A.ri.size();
    }
  A.v.assign(A.ri.size(), 0.0);
}

int64_t linear_index(const CSC& A, int r, int c) {
  const int32_t* b = A.ri.data() + A.cp[c];
  const int32_t* e = A.ri.data() + A.cp[c + 1];
  const int32_t* it = std::lower_bound(b, e, r);
  return (int64_t)(it - A.ri.data());
}

int assemble_matrix(orc_problem& p, const double* u, int dbc, CSC& A) {
  build_pattern(p, dbc, A);
  auto cb = constraints_below(p);
  static thread_local double K[ND][ND];
  for (int e = 0; e < p.ne; ++e) {
    int st = element_matrix(p, e, u, K);
    if (st) return st;
    int dofs[ND];
    for (int v = 0; v < NN; ++v)
      for (int c = 0; c < 3; ++c) dofs[3 * v + c] = 3 * p.conn[8 * e + v] + c;
    // column-major scatter through linear indices (simpleassemblers.inl:120-137, 253-265)
    for (int c = 0; c < ND; ++c)
      for (int r = 0; r < ND; ++r) {
        int gr = dofs[r], gc = dofs[c];
        if (dbc == ORC_DBC_REDUCED) {
          if (p.fixed[gr] || p.fixed[gc]) continue;
          gr -= cb[gr];
          gc -= cb[gc];
        }
        A.v[linear_index(A, gr, gc)] += K[r][c];
      }
  }
  if (dbc == ORC_DBC_FULL) {  // simpleassemblers.inl:159-167 (explicit zeros stay stored)
    for (int c = 0; c < A.n; ++c)
      for (int64_t k = A.cp[c]; k < A.cp[c + 1]; ++k) {
        const int r = A.ri[k];
        if (p.fixed[c] || p.fixed[r]) A.v[k] = (r == c) ? 1.0 : 0.0;
      }
  }
  return ORC_OK;
}

int assemble_vector(orc_problem& p, const double* u, double lambda, int dbc, std::vector<double>& out) {
  auto cb = constraints_below(p);
  const int n = p.ndof();
  std::vector<double> full(n, 0.0);
  double fe[ND];
  for (int e = 0; e < p.ne; ++e) {
    int st = element_vector(p, e, u, lambda, fe);
    if (st) return st;
    for (int v = 0; v < NN; ++v)
      for (int c = 0; c < 3; ++c) full[3 * p.conn[8 * e + v] + c] += fe[3 * v + c];
  }
  if (dbc == ORC_DBC_REDUCED) {
    out.assign(n - (n ? cb[n - 1] + p.fixed[n - 1] : 0), 0.0);
    for (int i = 0; i < n; ++i)
      if (!p.fixed[i]) out[i - cb[i]] = full[i];
    for (size_t k = 0; k < p.pl_dof.size(); ++k)
      if (!p.fixed[p.pl_dof[k]]) out[p.pl_dof[k] - cb[p.pl_dof[k]]] += lambda * p.pl_val[k];
  } else {
    if (dbc == ORC_DBC_FULL)
      for (int i = 0; i < n; ++i)
        if (p.fixed[i]) full[i] = 0.0;
    for (size_t k = 0; k < p.pl_dof.size(); ++k) full[p.pl_dof[k]] += lambda * p.pl_val[k];
    out.swap(full);
  }
  return ORC_OK;
}

// Banded LDL^T (no pivoting) for the symmetric Full-DBC tangent; stands in for the reference's
// sparse direct solvers (UmfPackLU / SimplicialLDLT).
bool banded_ldlt_solve(const CSC& A, const std::vector<double>& b, std::vector<double>& x) {
  const int n = A.n;
  int bw = 0;
  for (int c = 0; c < n; ++c)
    for (int64_t k = A.cp[c]; k < A.cp[c + 1]; ++k) bw = std::max(bw, std::abs(A.ri[k] - c));
  const int w = bw + 1;
  // lower band storage: Lb[i*w + (i-j)] for j in [i-bw, i]
  std::vector<double> Lb((size_t)n * w, 0.0);
  for (int c = 0; c < n; ++c)
    for (int64_t k = A.cp[c]; k < A.cp[c + 1]; ++k) {
      const int r = A.ri[k];
      if (r >= c) Lb[(size_t)r * w + (r - c)] = A.v[k];
    }
  std::vector<double> d(n);
  for (int j = 0; j < n; ++j) {
    double dj = Lb[(size_t)j * w];
    const int k0 = std::max(0, j - bw);
    for (int k = k0; k < j; ++k) {
      const double l = Lb[(size_t)j * w + (j - k)];
      dj -= l * l * d[k];
    }
    if (dj == 0.0 || !std::isfinite(dj)) return false;
    d[j] = dj;
    const int iend = std::min(n - 1, j + bw);
    for (int i = j + 1; i <= iend; ++i) {
      double s = Lb[(size_t)i * w + (i - j)];
      const int kk0 = std::max(k0, i - bw);
      for (int k = kk0; k < j; ++k) s -= Lb[(size_t)i * w + (i - k)] * Lb[(size_t)j * w + (j - k)] * d[k];
      Lb[(size_t)i * w + (i - j)] = s / dj;
    }
  }
  x = b;
  for (int i = 0; i < n; ++i) {
    double s = x[i];
    for (int k = std::max(0, i - bw); k < i; ++k) s -= Lb[(size_t)i * w + (i - k)] * x[k];
    x[i] = s;
  }
  for (int i = 0; i < n; ++i) x[i] /= d[i];
  for (int i = n - 1; i >= 0; --i) {
    double s = x[i];
    for (int k = i + 1; k <= std::min(n - 1, i + bw); ++k) s -= Lb[(size_t)k * w + (k - i)] * x[k];
    x[i] = s;
  }
  return true;
}

// Jacobi-preconditioned CG (the reference's si_ConjugateGradient: Eigen ConjugateGradient with its
// default diagonal preconditioner, linearsolver.cpp:23-25), relative tolerance on ||r||/||b||.
// Fork-join pool for the CG's vector work: task t of T covers the rows [t n / T, (t + 1) n / T), and partial sums
// are added in task order, so results depend only on the thread count (one thread: the plain serial loops).
// Eigen runs ConjugateGradient<SparseMatrix, Lower | Upper> -- the reference's si_ConjugateGradient
// (solver/linearsolver/linearsolver.cpp:24) -- with a multithreaded matrix-vector product when OpenMP is on; this
// pool stands in for that.  Element assembly stays serial, as in the reference's assembler.
int g_threads = 1;
class Pool {
 public:
  explicit Pool(int n) : n_(n) {
    for (int t = 1; t < n_; ++t) th_.emplace_back([this, t] { loop(t); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> l(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  int size() const { return n_; }
  // runs f(t) for t = 0..n-1 (t = 0 on the calling thread) and waits for all
  void run(const std::function<void(int)>& f) {
    {
      std::lock_guard<std::mutex> l(m_);
      job_ = &f;
      pending_ = n_ - 1;
      ++gen_;
    }
    cv_.notify_all();
    f(0);
    std::unique_lock<std::mutex> l(m_);
    done_.wait(l, [this] { return pending_ == 0; });
  }

 private:
  void loop(int t) {
    int seen = 0;
    for (;;) {
      const std::function<void(int)>* job;
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        job = job_;
      }
      (*job)(t);
      {
        std::lock_guard<std::mutex> l(m_);
        if (--pending_ == 0) done_.notify_one();
      }
    }
  }
  int n_;
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int pending_ = 0, gen_ = 0;
  bool stop_ = false;
};

bool cg_jacobi_solve(const CSC& A, const std::vector<double>& b, std::vector<double>& x, double rtol, int maxit,
                     int* iterations = nullptr) {
  const int n = A.n;
  const int T = std::max(1, std::min(g_threads, n));
  Pool pool(T);
  auto lo = [&](int t) { return (int)((int64_t)n * t / T); };
  std::vector<double> part(T);
  auto reduce = [&] {
    double s = 0;
    for (double v : part) s += v;
    return s;
  };
  std::vector<double> diag(n, 1.0), r(b), z(n), pv(n), q(n);
  for (int c = 0; c < n; ++c)
    for (int64_t k = A.cp[c]; k < A.cp[c + 1]; ++k)
      if (A.ri[k] == c && A.v[k] != 0.0) diag[c] = A.v[k];
  x.assign(n, 0.0);
  double bn = 0;
  for (double v : b) bn += v * v;
  bn = std::sqrt(bn);
  if (bn == 0) return true;
  for (int i = 0; i < n; ++i) z[i] = r[i] / diag[i];
  pv = z;
  double rz = 0;
  for (int i = 0; i < n; ++i) rz += r[i] * z[i];
  for (int it = 0; it < maxit; ++it) {
    // q = A p (A symmetric: column i of the CSC is row i) and p.q
    pool.run([&](int t) {
      double pq = 0;
      for (int i = lo(t); i < lo(t + 1); ++i) {
        double acc = 0;
        for (int64_t k = A.cp[i]; k < A.cp[i + 1]; ++k) acc += A.v[k] * pv[A.ri[k]];
        q[i] = acc;
        pq += pv[i] * acc;
      }
      part[t] = pq;
    });
    const double al = rz / reduce();
    pool.run([&](int t) {
      double rn = 0;
      for (int i = lo(t); i < lo(t + 1); ++i) {
        x[i] += al * pv[i];
        r[i] -= al * q[i];
        rn += r[i] * r[i];
      }
      part[t] = rn;
    });
    const double rn = reduce();
    if (iterations) *iterations = it + 1;
    if (std::sqrt(rn) <= rtol * bn) return true;
    pool.run([&](int t) {
      double rzn = 0;
      for (int i = lo(t); i < lo(t + 1); ++i) {
        z[i] = r[i] / diag[i];
        rzn += r[i] * z[i];
      }
      part[t] = rzn;
    });
    const double rzn = reduce();
    const double be = rzn / rz;
    rz = rzn;
    pool.run([&](int t) {
      for (int i = lo(t); i < lo(t + 1); ++i) pv[i] = z[i] + be * pv[i];
    });
  }
  return false;
}

// EAS internal-state update at the old displacement (enhancedassumedstrains.hh:225-248).
int update_state(orc_problem& p, const double* u, const double* corr) {
  if (p.na == 0) return ORC_OK;
  const int na = p.na;
  std::vector<double> newAlpha(p.alpha);
  for (int e = 0; e < p.ne; ++e) {
    ElemOut eo;
    element_internal(p, e, u, false, eo);
    if (!eo.ok) return ORC_ERR_NONPOSITIVE_DETC;
    std::vector<double> rhs(na);
    for (int a = 0; a < na; ++a) {
      double s = eo.Rt[a];
      for (int v = 0; v < NN; ++v)
        for (int c = 0; c < 3; ++c) s += eo.L[a * ND + 3 * v + c] * corr[3 * p.conn[8 * e + v] + c];
      rhs[a] = s;
    }
    std::vector<double> Dm(eo.D, eo.D + na * na);
    if (!lu_solve(na, Dm, rhs.data(), 1)) return ORC_ERR_SINGULAR;
    for (int a = 0; a < na; ++a) newAlpha[(size_t)e * na + a] -= rhs[a];
  }
  p.alpha.swap(newAlpha);
  return ORC_OK;
}

double norm2(const std::vector<double>& v) {
  double s = 0;
  for (double x : v) s += x * x;
  return std::sqrt(s);
}

}  // namespace

extern "C" {

orc_problem* orc_problem_create(int n_nodes, const double* coords, int n_elems, const int32_t* conn, double lambda,
                                double mu, int eas_kind, int n_alpha) {
  if (n_nodes <= 0 || n_elems <= 0 || !coords || !conn) return nullptr;
  if (eas_kind < 0 || eas_kind > 3) return nullptr;
  if (n_alpha != 0) {
    if (eas_kind == ORC_EAS_NONE) return nullptr;
    if (eas_kind == ORC_EAS_GL && n_alpha != 9 && n_alpha != 21) return nullptr;
    if ((eas_kind == ORC_EAS_H || eas_kind == ORC_EAS_HT) && n_alpha != 9) return nullptr;
  }
  auto* p = new orc_problem;
  p->nn = n_nodes;
  p->ne = n_elems;
  p->X.assign(coords, coords + 3 * (size_t)n_nodes);
  p->conn.assign(conn, conn + 8 * (size_t)n_elems);
  p->lam = lambda;
  p->mu = mu;
  p->eas = eas_kind;
  p->na = n_alpha;
  p->fixed.assign(3 * (size_t)n_nodes, 0);
  p->alpha.assign((size_t)n_elems * n_alpha, 0.0);
  return p;
}
void orc_problem_destroy(orc_problem* p) { delete p; }
int orc_set_material(orc_problem* p, int material) {
  if (!p || material < ORC_MATERIAL_NEOHOOKE || material > ORC_MATERIAL_BLATZKO) return ORC_ERR_ARG;
  p->material = material;
  return ORC_OK;
}

namespace {
bool hyper_valid(const orc_hyper* h) {
  if (!h || h->deviatoric < ORC_DEV_NONE || h->deviatoric > ORC_DEV_GENT) return false;
  if (h->volumetric < 0 || h->volumetric > 12) return false;
  const bool terms = h->deviatoric == ORC_DEV_OGDEN_TOTAL || h->deviatoric == ORC_DEV_OGDEN_DEVIATORIC ||
                     h->deviatoric == ORC_DEV_INVARIANT_BASED;
  if (terms && (h->n_terms < 1 || h->n_terms > ORC_HYPER_MAX_TERMS)) return false;
  if (h->deviatoric == ORC_DEV_INVARIANT_BASED)
    for (int i = 0; i < h->n_terms; ++i)  // checkExponents (invariantbased.hh): p_i = q_i = 0 throws
      if (h->p[i] < 0 || h->q[i] < 0 || (h->p[i] == 0 && h->q[i] == 0)) return false;
  if ((h->deviatoric == ORC_DEV_ARRUDA_BOYCE || h->deviatoric == ORC_DEV_GENT) && !(h->param > 0.0)) return false;
  return true;
}
}  // namespace

int orc_set_hyperelastic(orc_problem* p, const orc_hyper* h) {
  if (!p || !hyper_valid(h)) return ORC_ERR_ARG;
  p->hyper = *h;
  p->material = ORC_MATERIAL_HYPERELASTIC;
  return ORC_OK;
}

int orc_hyper_deviatoric(const orc_hyper* h, const double* lambda, double* out13) {
  if (!hyper_valid(h) || !lambda || !out13) return ORC_ERR_ARG;
  DevOut d;
  deviatoric_function(*h, lambda, d);
  out13[0] = d.W;
  for (int i = 0; i < 3; ++i) out13[1 + i] = d.dW[i];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out13[4 + 3 * i + j] = d.dS[i][j];
  return d.domain_ok ? ORC_OK : ORC_ERR_ARG;
}

int orc_hyper_volumetric(int vf, double beta, double J, double* out3) {
  if (vf < 0 || vf > 12 || !out3) return ORC_ERR_ARG;
  volumetric_function(vf, beta, J, out3);
  return ORC_OK;
}

int orc_material_point(int material, double lambda, double mu, const orc_hyper* h, const double* C, double* out43) {
  if (!C || !out43 || material < ORC_MATERIAL_NEOHOOKE || material > ORC_MATERIAL_HYPERELASTIC) return ORC_ERR_ARG;
  if (material == ORC_MATERIAL_HYPERELASTIC && !hyper_valid(h)) return ORC_ERR_ARG;
  double Ev[6];
  for (int i = 0; i < 3; ++i) Ev[i] = 0.5 * (C[4 * i] - 1.0);
  Ev[3] = C[5], Ev[4] = C[2], Ev[5] = C[1];  // doubled shears 2 E_ij = C_ij
  MatState m;
  material_law(material, lambda, mu, h, Ev, m, true);
  out43[0] = m.psi;
  for (int v = 0; v < 6; ++v) out43[1 + v] = m.S[v];
  for (int r = 0; r < 6; ++r)
    for (int s = 0; s < 6; ++s) out43[7 + 6 * r + s] = m.C6[r][s];
  return m.ok ? ORC_OK : ORC_ERR_NONPOSITIVE_DETC;
}
int orc_set_dirichlet(orc_problem* p, const uint8_t* f) {
  if (!p || !f) return ORC_ERR_ARG;
  for (int i = 0; i < p->ndof(); ++i) p->fixed[i] = f[i] ? 1 : 0;
  return ORC_OK;
}
// DirichletValues::storeInhomogeneousBoundaryCondition (dirichletvalues.hh:213-222) for prescribed values linear
// in the load factor: u_D(lambda) = lambda * rate, derivative rate; rate must vanish on free dofs.
int orc_set_dirichlet_function(orc_problem* p, orc_point_fn value, orc_point_fn derivative, void* user) {
  if (!p || !value || !derivative) return ORC_ERR_ARG;
  // storeInhomogeneousBoundaryCondition (dirichletvalues.hh:213-222): the value and its lambda-derivative; the IDBC
  // force uses the derivative at lambda = 1 interpolated at every node (functionhelper.hh:170-184)
  p->idbc_rate.assign(3 * (size_t)p->nn, 0.0);
  derivative(p->nn, p->X.data(), 1.0, p->idbc_rate.data(), user);
  p->idbc_value = value;
  p->idbc_user = user;
  return ORC_OK;
}
int orc_set_dirichlet_values(orc_problem* p, const double* rate) {
  if (!p) return ORC_ERR_ARG;
  p->idbc_value = nullptr;
  if (!rate) {
    p->idbc_rate.clear();
    return ORC_OK;
  }
  for (int i = 0; i < p->ndof(); ++i)
    if ((rate[i] != 0.0 && !p->fixed[i]) || !std::isfinite(rate[i])) return ORC_ERR_ARG;
  p->idbc_rate.assign(rate, rate + p->ndof());
  return ORC_OK;
}
int orc_add_volume_load(orc_problem* p, orc_point_fn f, void* user) {
  if (!p || !f) return ORC_ERR_ARG;
  p->volume_fns.push_back({f, user});
  return ORC_OK;
}
int orc_add_neumann_function(orc_problem* p, int nf, const int32_t* fe, const int32_t* fl, orc_point_fn f,
                             void* user) {
  if (!p || nf < 0 || !f || (nf > 0 && (!fe || !fl))) return ORC_ERR_ARG;
  if (p->fn_faces.empty()) p->fn_faces.assign(p->ne, {});
  for (int k = 0; k < nf; ++k) {
    if (fe[k] < 0 || fe[k] >= p->ne || fl[k] < 0 || fl[k] > 5) return ORC_ERR_ARG;
    p->fn_faces[fe[k]].push_back({fl[k], {f, user}});
  }
  return ORC_OK;
}
int orc_add_neumann(orc_problem* p, int nf, const int32_t* fe, const int32_t* fl, const double* t) {
  if (!p || nf < 0) return ORC_ERR_ARG;
  if (p->faces.empty()) p->faces.assign(p->ne, {});
  for (int k = 0; k < nf; ++k) {
    if (fe[k] < 0 || fe[k] >= p->ne || fl[k] < 0 || fl[k] > 5) return ORC_ERR_ARG;
    p->faces[fe[k]].push_back({fl[k], {t[3 * k], t[3 * k + 1], t[3 * k + 2]}});
  }
  return ORC_OK;
}
int orc_add_point_loads(orc_problem* p, int n, const int32_t* dofs, const double* vals) {
  if (!p || n < 0) return ORC_ERR_ARG;
  for (int k = 0; k < n; ++k) {
    if (dofs[k] < 0 || dofs[k] >= p->ndof()) return ORC_ERR_ARG;
    p->pl_dof.push_back(dofs[k]);
    p->pl_val.push_back(vals[k]);
  }
  return ORC_OK;
}
int orc_set_faithful_moduli(orc_problem* p, int on) {
  if (!p) return ORC_ERR_ARG;
  p->faithful = on != 0;
  return ORC_OK;
}
int orc_get_alpha(const orc_problem* p, double* a) {
  if (!p || !a) return ORC_ERR_ARG;
  std::copy(p->alpha.begin(), p->alpha.end(), a);
  return ORC_OK;
}
int orc_set_alpha(orc_problem* p, const double* a) {
  if (!p || !a) return ORC_ERR_ARG;
  std::copy(a, a + p->alpha.size(), p->alpha.begin());
  return ORC_OK;
}
int orc_element_vector(orc_problem* p, int e, const double* u, double lambda, double* out) {
  if (!p || e < 0 || e >= p->ne || !out) return ORC_ERR_ARG;
  return element_vector(*p, e, u, lambda, out);
}
int orc_element_matrix(orc_problem* p, int e, const double* u, double lambda, double* out) {
  (void)lambda;
  if (!p || e < 0 || e >= p->ne || !out) return ORC_ERR_ARG;
  static thread_local double K[ND][ND];
  int st = element_matrix(*p, e, u, K);
  if (st) return st;
  for (int c = 0; c < ND; ++c)
    for (int r = 0; r < ND; ++r) out[c * ND + r] = K[r][c];
  return ORC_OK;
}
int orc_element_energy(orc_problem* p, int e, const double* u, double lambda, double* energy) {
  if (!p || e < 0 || e >= p->ne || !energy) return ORC_ERR_ARG;
  if (p->na > 0) return ORC_ERR_NOT_IMPLEMENTED;  // enhancedassumedstrains.hh:305-309
  ElemOut eo;
  element_internal(*p, e, u, false, eo);
  if (!eo.ok) return ORC_ERR_NONPOSITIVE_DETC;
  double en = eo.energy;
  element_traction(*p, e, lambda, nullptr, u, &en);
  element_volume_load(*p, e, lambda, nullptr, u, &en);
  *energy = en;
  return ORC_OK;
}
// calculateAt<PK2Stress / kirchhoffStress / cauchyStress> of the displacement-based element at a local point
// (nonlinearelastic.hh:237-271): H at xi, E = GL(H), S = NeoHooke PK2, tau = F S F^T, sigma = tau / det F
// (stressconversions.hh:88-125); result in Voigt without shear factors [11, 22, 33, 23, 13, 12].
int orc_calculate_at(orc_problem* p, int e, const double* u, int type, const double* xi, double* out6) {
  if (!p || e < 0 || e >= p->ne || !xi || !out6 || type < 0 || type > 2) return ORC_ERR_ARG;
  double X[NN][3], ue[NN][3];
  gather(*p, e, u, X, ue);
  Geo g;
  geometry(X, xi, g);
  double H[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int v = 0; v < NN; ++v) s += ue[v][i] * g.dNdX[v][j];
      H[i][j] = s;
    }
  double Ev[6];
  const int na = p->na;
  const int kind = na > 0 ? p->eas : ORC_EAS_NONE;
  if (kind == ORC_EAS_NONE) {
    gl_strain(H, Ev);
  } else {
    // EnhancedAssumedStrains::calculateAtImpl (enhancedassumedstrains.hh:127-188) with the stored alpha: GL adds
    // M(xi) alpha to the strain of the compatible gradient (F stays compatible); H / HT enhance the gradient
    const double* al = &p->alpha[(size_t)e * na];
    EasCentre ec;
    eas_centre(kind, X, ue, ec);
    if (kind == ORC_EAS_GL) {
      gl_strain(H, Ev);
      for (int k = 0; k < na; ++k) {
        const AnsatzEntry& a = kE21[k];
        double v = 2.0 * xi[a.f1] - 1.0;
        if (a.f2 >= 0) v *= 2.0 * xi[a.f2] - 1.0;
        for (int r = 0; r < 6; ++r) Ev[r] += ec.T0inv[r][a.row] * v / g.detJ * al[k];
      }
    } else {
      const double sc = ec.g0.detJ / g.detJ;
      double Ht[3][3] = {};
      for (int pm = 0; pm < na; ++pm) {
        const int r = pm / 3, c = pm % 3;
        const double val = 2.0 * xi[c] - 1.0;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Ht[i][j] += sc * ec.JIT0[i][r] * val * ec.JIT0[j][c] * al[pm];
      }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double add = Ht[i][j];
          if (kind == ORC_EAS_HT) {
            add = 0.0;
            for (int k = 0; k < 3; ++k) add += ec.Fc0[i][k] * Ht[j][k];
          }
          H[i][j] += add;
        }
      gl_strain(H, Ev);
    }
  }
  MatState m;
  material_law(p->material, p->lam, p->mu, &p->hyper, Ev, m, false);
  if (!m.ok) return ORC_ERR_NONPOSITIVE_DETC;
  if (type == 0) {
    std::copy(m.S, m.S + 6, out6);
    return ORC_OK;
  }
  double S[3][3], F[3][3], FS[3][3], tau[3][3];
  for (int v = 0; v < 6; ++v) S[VA[v]][VB[v]] = S[VB[v]][VA[v]] = m.S[v];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += F[i][k] * S[k][j];
      FS[i][j] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += FS[i][k] * F[j][k];
      tau[i][j] = s;
    }
  const double sc = type == 2 ? 1.0 / det3(F) : 1.0;
  for (int v = 0; v < 6; ++v) out6[v] = sc * tau[VA[v]][VB[v]];
  return ORC_OK;
}
int orc_update_state(orc_problem* p, const double* u, double lambda, const double* corr) {
  (void)lambda;
  if (!p || !corr) return ORC_ERR_ARG;
  return update_state(*p, u, corr);
}
int orc_assemble_vector(orc_problem* p, const double* u, double lambda, int dbc, double* out) {
  if (!p || !out || dbc < 0 || dbc > 2) return ORC_ERR_ARG;
  std::vector<double> v;
  int st = assemble_vector(*p, u, lambda, dbc, v);
  if (st) return st;
  std::copy(v.begin(), v.end(), out);
  return ORC_OK;
}
int64_t orc_pattern_nnz(orc_problem* p, int dbc) {
  if (!p || dbc < 0 || dbc > 2) return ORC_ERR_ARG;
  CSC A;
  build_pattern(*p, dbc, A);
  return (int64_t)A.ri.size();
}
int orc_cg_jacobi_csc(int n, const int64_t* col_ptr, const int32_t* row_idx, const double* values, const double* b,
                      double* x, double rtol, int max_iter, int* iterations) {
  if (n <= 0 || !col_ptr || !row_idx || !values || !b || !x) return ORC_ERR_ARG;
  CSC A;
  A.n = n;
  A.cp.assign(col_ptr, col_ptr + n + 1);
  A.ri.assign(row_idx, row_idx + col_ptr[n]);
  A.v.assign(values, values + col_ptr[n]);
  std::vector<double> bv(b, b + n), xv;
  int its = 0;
  const bool ok = cg_jacobi_solve(A, bv, xv, rtol, max_iter, &its);
  std::copy(xv.begin(), xv.end(), x);
  if (iterations) *iterations = its;
  return ok ? ORC_OK : ORC_ERR_NOT_CONVERGED;
}
int orc_reduced_size(orc_problem* p) {
  if (!p) return ORC_ERR_ARG;
  int c = 0;
  for (auto f : p->fixed) c += f;
  return p->ndof() - c;
}
int orc_assemble_matrix_csc(orc_problem* p, const double* u, double lambda, int dbc, int64_t* cp, int32_t* ri,
                            double* v) {
  (void)lambda;
  if (!p || dbc < 0 || dbc > 2) return ORC_ERR_ARG;
  CSC A;
  int st = assemble_matrix(*p, u, dbc, A);
  if (st) return st;
  if (cp) std::copy(A.cp.begin(), A.cp.end(), cp);
  if (ri) std::copy(A.ri.begin(), A.ri.end(), ri);
  if (v) std::copy(A.v.begin(), A.v.end(), v);
  return ORC_OK;
}

// FlatAssemblerBase constructor (assembler/interface.hh:50-62): constraintsBelow[i] = constrained dofs below i
int orc_constraints_below(const orc_problem* p, int32_t* out) {
  if (!p || !out) return ORC_ERR_ARG;
  int32_t counter = 0;
  for (int i = 0; i < p->ndof(); ++i) {
    out[i] = counter;
    if (p->fixed[i]) ++counter;
  }
  return ORC_OK;
}

int orc_set_threads(int n) {
  if (n < 1) return ORC_ERR_ARG;
  g_threads = n;
  return ORC_OK;
}

int orc_load_step(orc_problem* p, double dlambda, double tol, int tol_mode, int max_iter, int solver, double cg_rtol,
                  double* u, double* lambda, double* stats) {
  if (!p || !u || !lambda || !stats || !p->idbc_rate.empty()) return ORC_ERR_ARG;
  using clk = std::chrono::steady_clock;
  auto secs = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
  const int n = p->ndof();
  std::vector<double> x(u, u + n), R, dx;
  CSC K;
  double t_res = 0, t_mat = 0, t_sol = 0;
  int64_t cg_total = 0;
  *lambda += dlambda;  // LoadControl::predictor (loadcontrol.inl:54-57)
  auto t0 = clk::now();
  int st = assemble_vector(*p, x.data(), *lambda, ORC_DBC_FULL, R);
  t_res += secs(t0, clk::now());
  if (st) return st;
  double rn = norm2(R);
  const double thr = tol_mode == 1 ? tol * rn : tol;
  int it = 0;
  while (rn > thr && it < max_iter) {  // newtonraphson.hh:219-247
    t0 = clk::now();
    st = assemble_matrix(*p, x.data(), ORC_DBC_FULL, K);
    t_mat += secs(t0, clk::now());
    if (st) return st;
    std::vector<double> b(n);
    for (int i = 0; i < n; ++i) b[i] = -R[i];
    t0 = clk::now();
    int its = 0;
    const bool ok = solver == ORC_SOLVER_CG_JACOBI ? cg_jacobi_solve(K, b, dx, cg_rtol, 20 * n, &its)
                                                   : banded_ldlt_solve(K, b, dx);
    t_sol += secs(t0, clk::now());
    cg_total += its;
    if (!ok) return ORC_ERR_SINGULAR;
    st = update_state(*p, x.data(), dx.data());
    if (st) return st;
    for (int i = 0; i < n; ++i) x[i] += dx[i];
    t0 = clk::now();
    st = assemble_vector(*p, x.data(), *lambda, ORC_DBC_FULL, R);
    t_res += secs(t0, clk::now());
    if (st) return st;
    rn = norm2(R);
    ++it;
  }
  std::copy(x.begin(), x.end(), u);
  stats[0] = it;
  stats[1] = (double)cg_total;
  stats[2] = t_res;
  stats[3] = t_mat;
  stats[4] = t_sol;
  stats[5] = rn;
  return it == max_iter ? ORC_ERR_NOT_CONVERGED : ORC_OK;
}

int orc_load_control(orc_problem* p, int steps, double t0, double t1, double tol, int tol_mode, int max_iter,
                     int solver, double cg_rtol, double* u, double* lambda, int32_t* iterations, double* res_norms,
                     int* n_solves, int* total_iterations) {
  if (!p || !u || !lambda || steps <= 0) return ORC_ERR_ARG;
  const int n = p->ndof();
  std::vector<double> x(u, u + n), R, dx;
  const double step = (t1 - t0) / steps;  // loadcontrol.hh:77
  int total = 0, solves = 0;
  CSC K;
  const bool idbc = !p->idbc_rate.empty();
  // syncParameterAndGlobalSolution with the inhomogeneous values (nonlinearsolverfactory.hh:45-52): entries whose
  // prescribed value is nonzero take it
  std::vector<double> vd;
  auto sync = [&]() {
    if (!idbc) return;
    p->idbc_values(*lambda, vd);
    for (int i = 0; i < n; ++i)
      if (vd[i] != 0.0) x[i] = vd[i];
  };
  for (int s = 0; s <= steps; ++s) {
    if (s > 0) *lambda += step;  // LoadControl::predictor (loadcontrol.inl:54-57)
    const double step_size = s > 0 ? step : 0.0;  // solve(x) for the initial check, solve(x, stepSize) after
    int st = assemble_vector(*p, x.data(), *lambda, ORC_DBC_FULL, R);
    if (st) return st;
    if (idbc && step_size != 0.0) {
      // rx += idbcForce(x) * stepSize (newtonraphson.hh:212-215) with obtainForcesDueToIDBC
      // (functionhelper.hh:170-184): K_raw * du_D/dlambda, zero at constrained dofs
      st = assemble_matrix(*p, x.data(), ORC_DBC_RAW, K);
      if (st) return st;
      std::vector<double> F(n, 0.0);
      for (int c = 0; c < n; ++c)
        for (int64_t k = K.cp[c]; k < K.cp[c + 1]; ++k) F[K.ri[k]] += K.v[k] * p->idbc_rate[c];
      for (int i = 0; i < n; ++i)
        if (!p->fixed[i]) R[i] += F[i] * step_size;
    }
    double rn = norm2(R);
    const double thr = tol_mode == 1 ? tol * rn : tol;
    int it = 0;
    while (rn > thr && it < max_iter) {  // newtonraphson.hh:219
      st = assemble_matrix(*p, x.data(), ORC_DBC_FULL, K);
      if (st) return st;
      std::vector<double> b(n);
      for (int i = 0; i < n; ++i) b[i] = -R[i];
      bool ok = solver == ORC_SOLVER_CG_JACOBI ? cg_jacobi_solve(K, b, dx, cg_rtol, 20 * n)
                                               : banded_ldlt_solve(K, b, dx);
      if (!ok) return ORC_ERR_SINGULAR;
      st = update_state(*p, x.data(), dx.data());  // CORRECTION_UPDATED before x += dx (newtonraphson.hh:230-233)
      if (st) return st;
      for (int i = 0; i < n; ++i) x[i] += dx[i];
      sync();  // newtonraphson.hh:235-236
      st = assemble_vector(*p, x.data(), *lambda, ORC_DBC_FULL, R);
      if (st) return st;
      rn = norm2(R);
      ++it;
    }
    if (it == 0) sync();  // loadcontrol.inl:43-44
    if (iterations) iterations[s] = it;
    if (res_norms) res_norms[s] = rn;
    total += it;
    ++solves;
    if (n_solves) *n_solves = solves;
    if (total_iterations) *total_iterations = total;
    std::copy(x.begin(), x.end(), u);
    if (it == max_iter) return ORC_ERR_NOT_CONVERGED;  // success = (iter != maxIter)
  }
  return ORC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------------
// Path following: Newton-Raphson with a scalar subsidiary function (newtonraphsonwithscalarsubsidiaryfunction.hh
// :207-316) under PathFollowing::run (pathfollowing.inl:25-73), with the subsidiary functions ArcLength,
// LoadControlSubsidiaryFunction and DisplacementControl (pathfollowingfunctions.hh:88-368), idbcIncrement
// (common.hh:38-51) and the IterationBased step-size adaptation (adaptivestepsizing.hh:36-57).  The core is
// written over callbacks so that the same code runs the reference's two-dof test operator (golden values of
// tests/src/testpathfollowing.cpp) and the finite-element problem.
namespace {

using Vec = std::vector<double>;

double dotv(const Vec& a, const Vec& b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

struct PFOps {
  int nx = 0;  // size of the global solution
  int nr = 0;  // size of the residual / correction
  std::function<int(const Vec& x, double lam, Vec& R)> residual;
  std::function<int(const Vec& x, double lam)> tangent;   // assemble (and factor) K at (x, lam)
  std::function<int(const Vec& b, Vec& sol)> solve;         // K^{-1} b with the last tangent
  bool has_idbc = false;
  std::function<int(const Vec& x, double lam, Vec& F)> idbc_force;
  std::function<void(Vec& x, const Vec& dx)> update;       // updateFunction(x, dx)
  std::function<void(Vec& x, double lam)> sync;            // syncParameterAndGlobalSolution
  std::function<int(const Vec& x, const Vec& corr)> on_correction;  // CORRECTION_UPDATED (EAS state)
};

struct PFArgs {  // SubsidiaryArgs (pathfollowingfunctions.hh:30-69)
  double step_size = 0;
  Vec DD;
  double Dlambda = 0, f = 0;
  Vec dfdDD;
  double dfdDlambda = 0;
  int current_step = 0;
};

struct PFType {
  int kind = ORC_PF_ARC_LENGTH;
  double psi = 0;
  bool computed = false;
  std::vector<int> ci;  // DisplacementControl's controlled indices
};

// idbcIncrement (common.hh:38-51): the change of the synchronised solution when the load factor grows by Dlambda
Vec idbc_increment(const PFOps& o, const Vec& x, double lam, double Dlambda) {
  Vec d(o.nx, 0.0);
  if (!o.has_idbc) return d;
  Vec y = x;
  o.sync(y, lam + Dlambda);
  for (int i = 0; i < o.nx; ++i) d[i] = y[i] - x[i];
  return d;
}

void subsidiary(const PFOps& o, PFType& t, const Vec& x, double lam, PFArgs& a) {
  if (t.kind == ORC_PF_ARC_LENGTH) {  // ArcLength::operator() (pathfollowingfunctions.hh:102-115)
    const Vec d = idbc_increment(o, x, lam, a.Dlambda);
    const double dd2 = dotv(d, d);
    const double root = std::sqrt(dotv(a.DD, a.DD) + dd2 + t.psi * t.psi * a.Dlambda * a.Dlambda);
    a.f = root - a.step_size;
    if (!t.computed) {
      std::fill(a.dfdDD.begin(), a.dfdDD.end(), 0.0);
      a.dfdDlambda = 0.0;
    } else {
      for (int i = 0; i < o.nr; ++i) a.dfdDD[i] = a.DD[i] / root;
      const double dhat02 = dd2 / (a.Dlambda * a.Dlambda);  // Dhat0 = idbcDelta / Dlambda
      a.dfdDlambda = ((dhat02 + t.psi * t.psi) * a.Dlambda) / root;
    }
  } else if (t.kind == ORC_PF_LOAD_CONTROL) {  // LoadControlSubsidiaryFunction::operator() (:230-236)
    a.f = a.Dlambda - a.step_size;
    std::fill(a.dfdDD.begin(), a.dfdDD.end(), 0.0);
    a.dfdDlambda = 1.0;
  } else {  // DisplacementControl::operator() (:316-324)
    double s = 0;
    for (int i : t.ci) s += a.DD[i] * a.DD[i];
    const double nrm = std::sqrt(s);
    a.f = nrm - a.step_size;
    a.dfdDlambda = 0.0;
    std::fill(a.dfdDD.begin(), a.dfdDD.end(), 0.0);
    for (int i : t.ci) a.dfdDD[i] = a.DD[i] / nrm;
  }
}

struct PFSolveInfo {
  int iterations = 0;
  double residual_norm = 0, correction_norm = 0;
  bool success = true;
};

// NewtonRaphsonWithSubsidiaryFunction::solve (newtonraphsonwithscalarsubsidiaryfunction.hh:207-316)
int pf_nr_solve(const PFOps& o, PFType& t, Vec& x, double& lam, PFArgs& a, double tol, int max_iter,
                PFSolveInfo& info) {
  info = PFSolveInfo{};
  // Fext0 = -R(x = 0, lambda = 1): the load is taken as lambda * Fext0 (:225-232)
  Vec zero(o.nx, 0.0), R, fext0(o.nr);
  int st = o.residual(zero, 1.0, R);
  if (st) return st;
  for (int i = 0; i < o.nr; ++i) fext0[i] = -R[i];
  Vec rx;
  st = o.residual(x, lam, rx);
  if (st) return st;
  a.dfdDD.assign(o.nr, 0.0);
  if ((int)a.DD.size() != o.nr) a.DD.assign(o.nr, 0.0);
  subsidiary(o, t, x, lam, a);
  double rnorm = std::sqrt(dotv(rx, rx));
  info.residual_norm = rnorm;
  int iter = 0;
  Vec b1(o.nr), b2(o.nr), dR, dL, dD(o.nr), F;
  while (rnorm > tol && iter < max_iter) {
    st = o.tangent(x, lam);
    if (st) return st;
    for (int i = 0; i < o.nr; ++i) b1[i] = -rx[i];
    b2 = fext0;
    if (o.has_idbc) {  // second column Fext0 - idbcForce(req) (:260-263)
      st = o.idbc_force(x, lam, F);
      if (st) return st;
      for (int i = 0; i < o.nr; ++i) b2[i] -= F[i];
    }
    if ((st = o.solve(b1, dR)) || (st = o.solve(b2, dL))) return st;
    const double dlam = (-a.f - dotv(a.dfdDD, dR)) / (dotv(a.dfdDD, dL) + a.dfdDlambda);  // :275-276
    for (int i = 0; i < o.nr; ++i) dD[i] = dR[i] + dlam * dL[i];
    if (o.on_correction && (st = o.on_correction(x, dD))) return st;
    o.update(x, dD);
    for (int i = 0; i < o.nr; ++i) a.DD[i] += dD[i];
    lam += dlam;
    a.Dlambda += dlam;
    if (o.has_idbc) o.sync(x, lam);
    info.correction_norm = std::sqrt(dotv(dD, dD) + dlam * dlam);
    st = o.residual(x, lam, rx);
    if (st) return st;
    subsidiary(o, t, x, lam, a);
    rnorm = std::sqrt(dotv(rx, rx) + a.f * a.f);  // :298
    info.residual_norm = rnorm;
    ++iter;
    if (!std::isfinite(rnorm)) break;
  }
  info.iterations = iter;
  info.success = iter != max_iter && std::isfinite(rnorm);
  return ORC_OK;
}

// ArcLength::initialPrediction (pathfollowingfunctions.hh:132-174) and the other kinds' initial predictions
int pf_initial_prediction(const PFOps& o, PFType& t, Vec& x, double& lam, PFArgs& a) {
  if (t.kind == ORC_PF_LOAD_CONTROL) {  // :249-255
    a.Dlambda = a.step_size;
    lam = a.Dlambda;
  } else if (t.kind == ORC_PF_DISPLACEMENT_CONTROL) {  // :330-336
    for (int i : t.ci) a.DD[i] = a.step_size;
    for (int i = 0; i < o.nx; ++i) x[i] = a.DD[i];
  } else {
    const double dlambda = 1.0;
    Vec idbc_delta = idbc_increment(o, x, lam, dlambda);
    const double dhat02 = dotv(idbc_delta, idbc_delta) / (dlambda * dlambda);
    lam = dlambda;
    Vec R, F;
    int st = o.residual(x, lam, R);
    if (st) return st;
    if ((st = o.tangent(x, lam))) return st;
    if (o.has_idbc) {
      if ((st = o.idbc_force(x, lam, F))) return st;
      for (int i = 0; i < o.nr; ++i) R[i] += F[i];
    }
    for (double& v : R) v = -v;
    if ((st = o.solve(R, a.DD))) return st;
    const double dd2 = dotv(a.DD, a.DD);
    t.psi = std::sqrt(dd2 + dhat02);
    const double s = std::sqrt(dd2 + dhat02 + t.psi * t.psi * dlambda * dlambda);
    for (double& v : a.DD) v *= a.step_size / s;
    a.Dlambda = a.step_size / s;
    for (double& v : idbc_delta) v *= a.Dlambda / dlambda;
    o.update(x, a.DD);
    lam = a.Dlambda;
    if (o.has_idbc) o.sync(x, lam);
    t.psi = std::sqrt((dotv(idbc_delta, idbc_delta) + dotv(a.DD, a.DD)) / (a.Dlambda * a.Dlambda));
  }
  t.computed = true;
  return ORC_OK;
}

// intermediatePrediction of the three kinds (:188-195, :269-274, :339-344)
void pf_intermediate_prediction(const PFOps& o, PFType& t, Vec& x, double& lam, PFArgs& a) {
  if (t.kind == ORC_PF_LOAD_CONTROL) {
    lam += a.Dlambda;
    return;
  }
  if (t.kind == ORC_PF_DISPLACEMENT_CONTROL) {
    for (int i = 0; i < o.nx; ++i) x[i] += a.DD[i];
    return;
  }
  o.update(x, a.DD);
  lam += a.Dlambda;
  if (o.has_idbc) o.sync(x, lam);
}

// PathFollowing::run (pathfollowing.inl:25-73); infos receive steps + 1 entries (load step -1 first)
int pf_run(const PFOps& o, PFType& t, int steps, double step_size, int target_iterations, double tol, int max_iter,
           Vec& x, double& lam, int32_t* iterations, double* res_norms, double* lambdas, double* psi_out,
           int* n_solves, int* total, double* x_steps = nullptr) {
  PFArgs a;
  a.DD.assign(o.nr, 0.0);
  a.dfdDD.assign(o.nr, 0.0);
  a.step_size = step_size;
  PFSolveInfo info;
  int solves = 0, tot = 0;
  auto record = [&]() {
    if (iterations) iterations[solves] = info.iterations;
    if (res_norms) res_norms[solves] = info.residual_norm;
    if (lambdas) lambdas[solves] = lam;
    if (x_steps) std::copy(x.begin(), x.end(), x_steps + (size_t)solves * o.nx);
    tot += info.iterations;
    ++solves;
    if (n_solves) *n_solves = solves;
    if (total) *total = tot;
    if (psi_out) *psi_out = t.psi;
  };
  int st = pf_nr_solve(o, t, x, lam, a, tol, max_iter, info);  // load step -1
  if (st) return st;
  record();
  if (!info.success) return ORC_ERR_NOT_CONVERGED;
  if ((st = pf_initial_prediction(o, t, x, lam, a))) return st;
  if ((st = pf_nr_solve(o, t, x, lam, a, tol, max_iter, info))) return st;
  record();
  if (!info.success) return ORC_ERR_NOT_CONVERGED;
  for (int ls = 1; ls < steps; ++ls) {
    a.current_step = ls;
    // AdaptiveStepSizing::IterationBased (adaptivestepsizing.hh:36-47); 0 = NoOp
    if (target_iterations > 0 && info.iterations > target_iterations)
      a.step_size = std::sqrt((double)target_iterations / info.iterations) * a.step_size;
    pf_intermediate_prediction(o, t, x, lam, a);
    if ((st = pf_nr_solve(o, t, x, lam, a, tol, max_iter, info))) return st;
    record();
    if (!info.success) return ORC_ERR_NOT_CONVERGED;
  }
  return ORC_OK;
}

// The two-dof operator of the reference's path-following tests (tests/src/testpathfollowing.cpp:26-40), D = (u, w)
void toy_residual(double u, double w, double lam, double R[2]) {
  R[0] = 16.0 * u - 3 * w - w * w * w - (2.0 / 3.0) * lam;
  R[1] = -3 * u + 4 * w - 3 * u * w * w - (9.0 / 4.0) * lam;
}
void toy_stiffness(double u, double w, double K[2][2]) {
  K[0][0] = 16.0;
  K[0][1] = -3.0 * w * w - 3;
  K[1][0] = -3 * w * w - 3;
  K[1][1] = -6 * u * w + 4;
}

}  // namespace

extern "C" {

int orc_path_following(orc_problem* p, int kind, int steps, double step_size, int n_controlled,
                       const int32_t* controlled, int target_iterations, double tol, int max_iter, int solver,
                       double cg_rtol, double* u, double* lambda, int32_t* iterations, double* res_norms,
                       double* lambdas, double* psi, int* n_solves, int* total_iterations) {
  if (p && p->idbc_value) return ORC_ERR_NOT_IMPLEMENTED;  // prescribed-value functions: load control only
  if (!p || !u || !lambda || steps <= 0 || kind < 0 || kind > 2) return ORC_ERR_ARG;
  const int n = p->ndof();
  const bool idbc = !p->idbc_rate.empty();
  if (idbc && kind != ORC_PF_ARC_LENGTH) return ORC_ERR_NOT_IMPLEMENTED;  // checkHasNoValidIDBCForceFunction
  PFType t;
  t.kind = kind;
  if (kind == ORC_PF_DISPLACEMENT_CONTROL) {
    if (n_controlled <= 0 || !controlled) return ORC_ERR_ARG;
    for (int k = 0; k < n_controlled; ++k) {
      if (controlled[k] < 0 || controlled[k] >= n) return ORC_ERR_ARG;
      t.ci.push_back(controlled[k]);
    }
  }
  CSC K;
  PFOps o;
  o.nx = o.nr = n;
  o.residual = [&](const Vec& x, double lam, Vec& R) -> int { return assemble_vector(*p, x.data(), lam, ORC_DBC_FULL, R); };
  o.tangent = [&](const Vec& x, double) -> int { return assemble_matrix(*p, x.data(), ORC_DBC_FULL, K); };
  o.solve = [&](const Vec& b, Vec& sol) -> int {
    const bool ok = solver == ORC_SOLVER_CG_JACOBI ? cg_jacobi_solve(K, b, sol, cg_rtol, 20 * n)
                                                   : banded_ldlt_solve(K, b, sol);
    return ok ? ORC_OK : ORC_ERR_SINGULAR;
  };
  o.has_idbc = idbc;
  o.idbc_force = [&](const Vec& x, double, Vec& F) -> int {  // obtainForcesDueToIDBC (functionhelper.hh:170-184)
    CSC Kr;
    int st = assemble_matrix(*p, x.data(), ORC_DBC_RAW, Kr);
    if (st) return st;
    F.assign(n, 0.0);
    for (int c = 0; c < n; ++c)
      for (int64_t k = Kr.cp[c]; k < Kr.cp[c + 1]; ++k) F[Kr.ri[k]] += Kr.v[k] * p->idbc_rate[c];
    for (int i = 0; i < n; ++i)
      if (p->fixed[i]) F[i] = 0.0;
    return ORC_OK;
  };
  o.update = [](Vec& x, const Vec& dx) {
    for (size_t i = 0; i < x.size(); ++i) x[i] += dx[i];
  };
  o.sync = [&](Vec& x, double lam) {  // entries whose prescribed value is nonzero take it
    for (int i = 0; i < n; ++i) {
      const double v = lam * p->idbc_rate[i];
      if (v != 0.0) x[i] = v;
    }
  };
  o.on_correction = [&](const Vec& x, const Vec& corr) -> int { return update_state(*p, x.data(), corr.data()); };
  Vec x(u, u + n);
  double lam = *lambda;
  const int st = pf_run(o, t, steps, step_size, target_iterations, tol, max_iter, x, lam, iterations, res_norms,
                        lambdas, psi, n_solves, total_iterations);
  std::copy(x.begin(), x.end(), u);
  *lambda = lam;
  return st;
}

int orc_path_following_toy(int kind, int idbc, int steps, double step_size, int target_iterations, double tol,
                           int max_iter, double* d2, double* lambda, int32_t* iterations, double* lambdas,
                           double* d_steps, int* n_solves) {
  if (!d2 || !lambda || steps <= 0 || kind < 0 || kind > 2) return ORC_ERR_ARG;
  if (idbc && kind != ORC_PF_ARC_LENGTH) return ORC_ERR_NOT_IMPLEMENTED;
  PFType t;
  t.kind = kind;
  if (kind == ORC_PF_DISPLACEMENT_CONTROL) t.ci = {0};  // testpathfollowing.cpp:356
  double Kd[2][2] = {{0, 0}, {0, 0}};
  PFOps o;
  o.nx = 2;
  if (!idbc) {
    o.nr = 2;
    o.residual = [](const Vec& x, double lam, Vec& R) -> int {
      R.assign(2, 0.0);
      toy_residual(x[0], x[1], lam, R.data());
      return ORC_OK;
    };
    o.tangent = [&](const Vec& x, double) -> int {
      toy_stiffness(x[0], x[1], Kd);
      return ORC_OK;
    };
    o.solve = [&](const Vec& b, Vec& s) -> int {  // dense 2x2 solve
      const double det = Kd[0][0] * Kd[1][1] - Kd[0][1] * Kd[1][0];
      if (det == 0.0) return ORC_ERR_SINGULAR;
      s = {(Kd[1][1] * b[0] - Kd[0][1] * b[1]) / det, (Kd[0][0] * b[1] - Kd[1][0] * b[0]) / det};
      return ORC_OK;
    };
    o.update = [](Vec& x, const Vec& dx) {
      x[0] += dx[0];
      x[1] += dx[1];
    };
  } else {  // w free, u = 0.1 lambda prescribed (testpathfollowing.cpp:80-94, 358-365)
    o.nr = 1;
    o.has_idbc = true;
    o.residual = [](const Vec& x, double lam, Vec& R) -> int {
      double r[2];
      toy_residual(x[0], x[1], lam, r);
      R.assign(1, r[1]);
      return ORC_OK;
    };
    o.tangent = [&](const Vec& x, double) -> int {
      toy_stiffness(x[0], x[1], Kd);
      return ORC_OK;
    };
    o.solve = [&](const Vec& b, Vec& s) -> int {
      if (Kd[1][1] == 0.0) return ORC_ERR_SINGULAR;
      s.assign(1, b[0] / Kd[1][1]);
      return ORC_OK;
    };
    o.idbc_force = [&](const Vec& x, double, Vec& F) -> int {
      double K[2][2];
      toy_stiffness(x[0], x[1], K);
      F.assign(1, K[1][0] * 0.1);
      return ORC_OK;
    };
    o.update = [](Vec& x, const Vec& dx) { x[1] += dx[0]; };
    o.sync = [](Vec& x, double lam) { x[0] = 0.1 * lam; };
  }
  Vec x(d2, d2 + 2);
  double lam = *lambda;
  const int st = pf_run(o, t, steps, step_size, target_iterations, tol, max_iter, x, lam, iterations, nullptr,
                        lambdas, nullptr, n_solves, nullptr, d_steps);
  d2[0] = x[0];
  d2[1] = x[1];
  *lambda = lam;
  return st;
}

}  // extern "C"
