// Hyperelastic<Deviatoric<DF>, Volumetric<VF>> material point on the device (FP64).
//
// Reference: materials/hyperelastic/interface.hh (stressesImpl, tangentModuliImpl, storedEnergyImpl and the
// transformations of :120-160), deviatoric/interface.hh:91-118 (principal stresses and moduli L_iikk, L_ikik),
// the deviatoric functions deviatoric/{blatzko,ogden,invariantbased,arrudaboyce,gent}.hh with
// deviatoric/deviatoricinvariants.hh, and the volumetric functions volumetric/volumetricfunctions.hh.
//
// W(C) = W_dev(lambda_1, lambda_2, lambda_3) + K U(J), lambda_i = sqrt(eig_i(C)), J = lambda_1 lambda_2 lambda_3.
// S = sum_i (W_i / lambda_i) N_i (x) N_i + J K U' C^-1.  Material moduli (Voigt entry (A B, C D)):
//   sum_ik L_iikk N_Ai N_Bi N_Ck N_Dk + sum_{i != k} L_ikik N_Ai N_Bk (N_Ci N_Dk + N_Ck N_Di)
//   + J K (U' + J U'') Ci_AB Ci_CD - J K U' (Ci_AC Ci_BD + Ci_AD Ci_BC)
// with L_iikk = dS_ik / (lambda_i lambda_k) (dS = the function's secondDerivativeImpl) and L_ikik =
// (S_i - S_k) / (lambda_i^2 - lambda_k^2), or (L_iiii - L_iikk) / 2 where lambda_i, lambda_k agree to 1e-8.
// The eigen decomposition is cyclic Jacobi (stable rotation of Golub & Van Loan, sec. 8.5), eigenvalues ascending;
// the reference calls Eigen's SelfAdjointEigenSolver, and the stresses and moduli are functions of C alone.
// Everything indexes registers with compile-time constants (the rotations are templates over the index pair).
#pragma once
#include <cmath>

#include "common.cuh"
#include "kernels.h"

namespace ikr {
namespace hyper {

template <int P, int Q>
__device__ __forceinline__ void jacobi_rotate(double a[3][3], double V[3][3]) {
  constexpr int O = 3 - P - Q;
  const double apq = a[P][Q];
  if (apq == 0.0) return;
  const double app = a[P][P], aqq = a[Q][Q];
  if (fabs(app) + 100.0 * fabs(apq) == fabs(app) && fabs(aqq) + 100.0 * fabs(apq) == fabs(aqq)) {
    a[P][Q] = a[Q][P] = 0.0;  // below the diagonal's resolution
    return;
  }
  const double theta = (aqq - app) / (2.0 * apq);
  double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
  if (fabs(theta) > 1e150) t = 0.5 / fabs(theta);
  if (theta < 0.0) t = -t;
  const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
  const double aop = a[O][P], aoq = a[O][Q];
  a[P][P] = app - t * apq;
  a[Q][Q] = aqq + t * apq;
  a[P][Q] = a[Q][P] = 0.0;
  a[O][P] = a[P][O] = c * aop - s * aoq;
  a[O][Q] = a[Q][O] = s * aop + c * aoq;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double vkp = V[k][P], vkq = V[k][Q];
    V[k][P] = c * vkp - s * vkq;
    V[k][Q] = s * vkp + c * vkq;
  }
}

template <int I, int J>
__device__ __forceinline__ void sort_pair(double ev[3], double V[3][3]) {
  if (ev[I] > ev[J]) {
    const double t = ev[I];
    ev[I] = ev[J];
    ev[J] = t;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double v = V[k][I];
      V[k][I] = V[k][J];
      V[k][J] = v;
    }
  }
}

// symmetric 3x3 eigen decomposition: ev ascending, eigenvectors in the columns of V (at most 32 sweeps)
__device__ __forceinline__ void sym_eig3(const double A[3][3], double ev[3], double V[3][3]) {
  double a[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      a[i][j] = A[i][j];
      V[i][j] = i == j ? 1.0 : 0.0;
    }
#pragma unroll 1
  for (int sweep = 0; sweep < 32; ++sweep) {
    if (a[0][1] == 0.0 && a[0][2] == 0.0 && a[1][2] == 0.0) break;
    jacobi_rotate<0, 1>(a, V);
    jacobi_rotate<0, 2>(a, V);
    jacobi_rotate<1, 2>(a, V);
  }
  ev[0] = a[0][0], ev[1] = a[1][1], ev[2] = a[2][2];
  sort_pair<0, 1>(ev, V);
  sort_pair<1, 2>(ev, V);
  sort_pair<0, 1>(ev, V);
}

// deviatoric invariants W1 = I1 I3^-1/3, W2 = I2 I3^-2/3 with first and second derivatives
struct DevInv {
  double W1, W2, d1[3], d2[3], dd1[3][3], dd2[3][3];
};
__device__ __forceinline__ void deviatoric_invariants(const double l[3], DevInv& o) {
  double l2[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) l2[i] = l[i] * l[i];
  const double I1 = l2[0] + l2[1] + l2[2];
  const double I2 = l2[0] * l2[1] + l2[1] * l2[2] + l2[0] * l2[2];
  const double I3 = l2[0] * l2[1] * l2[2];
  const double c1 = pow(I3, 1.0 / 3.0), c2 = pow(I3, 2.0 / 3.0);
  o.W1 = I1 * pow(I3, -1.0 / 3.0);
  o.W2 = I2 * pow(I3, -2.0 / 3.0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    o.d1[i] = 2.0 * (3.0 * l2[i] - I1) / (3.0 * l[i] * c1);
    o.d2[i] = -2.0 * (3.0 * I3 / l2[i] - I2) / (3.0 * l[i] * c2);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
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

__device__ __forceinline__ double pow_times(double x, int p, int m) {
  if (m == 0) return 0.0;
  if (p == 0) return m;
  return pow(x, (double)p) * m;
}

// W, dW/dlambda_i and dS_ij = d2W/dlambda_i dlambda_j - delta_ij W_i / lambda_i of the deviatoric function; returns
// false outside its domain (Gent: Jm <= W1 - 3)
static __device__ __noinline__ bool deviatoric_function(const HyperParams& h, const double l[3], double& W, double dW[3],
                                                        double dS[3][3]) {
  W = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dW[i] = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) dS[i][j] = 0.0;
  }
  const int n = h.n;
  switch (h.dev) {
    case kDevBlatzKo: {
      const double mu = h.mu[0], J = l[0] * l[1] * l[2];
      W = mu / 2.0 * (1.0 / (l[0] * l[0]) + 1.0 / (l[1] * l[1]) + 1.0 / (l[2] * l[2]) + 2.0 * J - 5.0);
#pragma unroll
      for (int i = 0; i < 3; ++i) dW[i] = mu * (-1.0 / (l[i] * l[i] * l[i]) + J / l[i]);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const double li2 = l[i] * l[i];
          dS[i][j] = mu * (i == j ? (1.0 / li2) * (1.0 / li2 - J) + 3.0 / (li2 * li2) : J / (l[i] * l[j]));
        }
      return true;
    }
    case kDevOgdenTotal: {
      const double lnJ = log(l[0] * l[1] * l[2]);
#pragma unroll
      for (int p = 0; p < kHyperMaxTerms; ++p) {
        if (p >= n) break;
        const double mu = h.mu[p], al = h.alpha[p];
        double la[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) la[i] = pow(l[i], al);
        W += mu / al * (la[0] + la[1] + la[2] - 3.0) - mu * lnJ;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          dW[i] += mu * (la[i] - 1.0) / l[i];
          dS[i][i] += (-2.0 * mu * (la[i] - 1.0) + mu * la[i] * al) / (l[i] * l[i]);
        }
      }
      return true;
    }
    case kDevOgdenDeviatoric: {
      const double Jm13 = pow(l[0] * l[1] * l[2], -1.0 / 3.0);
      const double lb[3] = {Jm13 * l[0], Jm13 * l[1], Jm13 * l[2]};
      double dWdlb[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int p = 0; p < kHyperMaxTerms; ++p) {
        if (p >= n) break;
        double ps = 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) ps += pow(lb[i], h.alpha[p]);
        W += h.mu[p] / h.alpha[p] * (ps - 3.0);
#pragma unroll
        for (int i = 0; i < 3; ++i) dWdlb[i] += h.mu[p] * pow(lb[i], h.alpha[p] - 1.0);
      }
      const double sum = lb[0] * dWdlb[0] + lb[1] * dWdlb[1] + lb[2] * dWdlb[2];
#pragma unroll
      for (int i = 0; i < 3; ++i) dW[i] = (lb[i] * dWdlb[i] - sum / 3.0) / l[i];
#pragma unroll
      for (int p = 0; p < kHyperMaxTerms; ++p) {
        if (p >= n) break;
        const double al = h.alpha[p], c = h.mu[p] * al;
        double lba[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) lba[i] = pow(lb[i], al);
        const double ps = lba[0] + lba[1] + lba[2];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b)
            dS[a][b] += a == b ? c * (lba[a] / 3.0 + ps / 9.0) : c * (-(lba[a] + lba[b]) / 3.0 + ps / 9.0);
      }
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          dS[a][b] /= l[a] * l[b];
          if (a == b) dS[a][b] -= 2.0 / l[a] * dW[a];
        }
      return true;
    }
    case kDevInvariantBased: {
      DevInv d;
      deviatoric_invariants(l, d);
      const double W1 = d.W1 - 3.0, W2 = d.W2 - 3.0;
#pragma unroll
      for (int p = 0; p < kHyperMaxTerms; ++p) {
        if (p >= n) break;
        const int pe = h.p[p], qe = h.q[p];
        const double c = h.mu[p];
        const double W1p = pow(W1, (double)pe), W2q = pow(W2, (double)qe);
        const double W1pm1p = pow_times(W1, pe - 1, pe), W2qm1q = pow_times(W2, qe - 1, qe);
        const double W1pm2pp = pow_times(W1, pe - 2, pe * (pe - 1)), W2qm2qq = pow_times(W2, qe - 2, qe * (qe - 1));
        W += c * W1p * W2q;
#pragma unroll
        for (int k = 0; k < 3; ++k) dW[k] += c * (W1pm1p * W2q * d.d1[k] + W1p * W2qm1q * d.d2[k]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const double cross = d.d1[i] * d.d2[j] + d.d1[j] * d.d2[i];
            double v = (W2qm1q * cross + W2q * d.dd1[i][j]) * W1pm1p * c + W2qm1q * d.dd2[i][j] * W1p * c +
                       W1pm2pp * W2q * d.d1[i] * d.d1[j] * c + W2qm2qq * W1p * d.d2[i] * d.d2[j] * c;
            if (i == j) v -= (1.0 / l[i]) * c * (W1pm1p * W2q * d.d1[i] + W1p * W2qm1q * d.d2[i]);
            dS[i][j] += v;
          }
      }
      return true;
    }
    case kDevArrudaBoyce: {
      constexpr double a[5] = {0.5, 1.0 / 20.0, 11.0 / 1050.0, 19.0 / 7000.0, 519.0 / 673750.0};
      DevInv d;
      deviatoric_invariants(l, d);
      const double mu = h.mu[0], beta = 1.0 / (h.param * h.param), W1 = d.W1;
#pragma unroll
      for (int p = 0; p < 5; ++p) {
        const double bp = pow(beta, (double)p);
        const double f1 = mu * a[p] * bp;
        const double W1p = pow(W1, (double)p), W1pm1 = pow(W1, (double)(p - 1));
        W += a[p] * bp * (pow(W1, (double)(p + 1)) - pow(3.0, (double)(p + 1)));
#pragma unroll
        for (int k = 0; k < 3; ++k) dW[k] += f1 * W1p * d.d1[k] * (p + 1);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            double v = f1 * (W1p * d.dd1[i][j] * (p + 1) + W1pm1 * d.d1[i] * d.d1[j] * p * (p + 1));
            if (i == j) v -= d.d1[i] / l[i] * f1 * W1p * (p + 1);
            dS[i][j] += v;
          }
      }
      W *= mu;
      return true;
    }
    case kDevGent: {
      DevInv d;
      deviatoric_invariants(l, d);
      const double mu = h.mu[0], Jm = h.param, W1 = d.W1, x = W1 - 3.0;
      const bool ok = !(Jm < x || fabs(Jm - x) <= 1e-14 * fmax(fabs(Jm), fabs(x)));
      W = -(mu / 2.0) * Jm * log(1.0 - (W1 - 3.0) / Jm);
#pragma unroll
      for (int k = 0; k < 3; ++k) dW[k] = (mu * d.d1[k] * Jm) / (2.0 * (Jm - W1) + 6.0);
      const double f1 = 1.0 - (W1 - 3.0) / Jm;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double v = (mu / (2.0 * f1)) * (d.dd1[i][j] + (d.d1[i] * d.d1[j] / (f1 * Jm)));
          if (i == j) v -= (mu / (2.0 * l[i] * f1)) * d.d1[i];
          dS[i][j] = v;
        }
      return ok;
    }
    default: return true;  // NoDev
  }
}

// U, U', U'' of volumetric function VF<vf> (without the factor K)
static __device__ __noinline__ void volumetric_function(int vf, double b, double J, double U[3]) {
  const double lJ = log(J);
  switch (vf) {
    case 1: U[0] = 0.5 * (J - 1) * (J - 1), U[1] = J - 1, U[2] = 1; break;
    case 2:
      U[0] = 0.25 * ((J - 1) * (J - 1) + lJ * lJ);
      U[1] = 0.5 * (J - 1 + 1 / J * lJ);
      U[2] = 1 / (2 * J * J) * (1 + J * J - lJ);
      break;
    case 3: U[0] = 0.5 * lJ * lJ, U[1] = 1 / J * lJ, U[2] = 1 / (J * J) * (1 - lJ); break;
    case 4:
      U[0] = (1 / (b * b)) * ((1 / pow(J, b)) - 1 + b * lJ);
      U[1] = (1 / b) * ((1 / J) - (1 / pow(J, 1 + b)));
      U[2] = (1 / b) * ((1 / pow(J, 2 + b)) * (1 + b - pow(J, b)));
      break;
    case 5: U[0] = 0.25 * (J * J - 1 - 2 * lJ), U[1] = 0.5 * (J - 1 / J), U[2] = 0.5 * (1 + 1 / (J * J)); break;
    case 6: U[0] = J - lJ - 1, U[1] = 1 - 1 / J, U[2] = 1 / (J * J); break;
    case 7:
      U[0] = pow(J, b) * (b * lJ - 1) + 1;
      U[1] = b * b * (1.0 / pow(J, 1.0 - b)) * lJ;
      U[2] = b * b * pow(J, b - 2.0) * (1 + (b - 1) * lJ);
      break;
    case 8: U[0] = J * lJ - J + 1, U[1] = lJ, U[2] = 1 / J; break;
    case 9: {
      const double t = J * J - 1 / (J * J);
      U[0] = (1.0 / 32.0) * t * t;
      U[1] = (1.0 / 8.0) * (pow(J, 3.0) - 1.0 / pow(J, 5.0));
      U[2] = (1.0 / 8.0) * (5.0 * pow(J, -6.0) + 3.0 * J * J);
      break;
    }
    case 10:
      U[0] = (J / b) * (1 - (pow(J, -b) / (1 - b))) + (1.0 / (b - 1));
      U[1] = (1 / b) * (1 - pow(J, -b));
      U[2] = pow(J, -1 - b);
      break;
    case 11:
      U[0] = (1.0 / 50.0) * (pow(J, 5.0) + pow(J, -5.0) - 2.0);
      U[1] = (1.0 / 10.0) * (pow(J, 4.0) - pow(J, -6.0));
      U[2] = (1.0 / 10.0) * (4 * pow(J, 3.0) + 6 * pow(J, -7.0));
      break;
    case 12: U[0] = J - 1, U[1] = 1, U[2] = 0; break;
    default: U[0] = U[1] = U[2] = 0; break;
  }
}

// The spectral ingredients of one material point: stresses and any modulus entry follow from them.
struct Point {
  double N[3][3];   // principal directions (columns)
  double Sp[3];     // principal deviatoric stresses W_i / lambda_i
  double L[3][3];   // L_iikk
  double Lo[3][3];  // L_ikik (i != k)
  double Ci[3][3];  // C^-1
  double vs, v1, v2;  // J K U', J K (U' + J U''), J K U'
  double psi;
};

// returns the status bits of the point (non-positive det C, outside the deviatoric function's domain)
__device__ __forceinline__ int evaluate(const HyperParams& h, const double C[3][3], Point& pt, bool want_moduli) {
  double ev[3];
  sym_eig3(C, ev, pt.N);
  const double l[3] = {sqrt(ev[0]), sqrt(ev[1]), sqrt(ev[2])};
  const double J = l[0] * l[1] * l[2];
  int bad = (J * J > 1e-10 && J > 0.0) ? 0 : kStatusNonPositiveDetC;
  double W, dW[3], dS[3][3];
  if (!deviatoric_function(h, l, W, dW, dS)) bad |= kStatusMaterialDomain;
  double U[3];
  volumetric_function(h.vol, h.beta, J, U);
  pt.psi = W + h.K * U[0];
  inv3(C, pt.Ci);
#pragma unroll
  for (int i = 0; i < 3; ++i) pt.Sp[i] = dW[i] / l[i];
  pt.vs = J * h.K * U[1];
  pt.v1 = J * h.K * (U[1] + J * U[2]);
  pt.v2 = pt.vs;
  if (want_moduli) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) pt.L[i][k] = dS[i][k] / (l[i] * l[k]);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (i == k) {
          pt.Lo[i][k] = 0.0;
        } else if (fabs(l[i] - l[k]) <= 1e-8 * fmax(fabs(l[i]), fabs(l[k]))) {
          pt.Lo[i][k] = 0.5 * (pt.L[i][i] - pt.L[i][k]);
        } else {
          pt.Lo[i][k] = (pt.Sp[i] - pt.Sp[k]) / (l[i] * l[i] - l[k] * l[k]);
        }
      }
  }
  return bad;
}

// PK2 stress entry (A, B)
__device__ __forceinline__ double stress(const Point& pt, int A, int B) {
  return pt.Sp[0] * pt.N[A][0] * pt.N[B][0] + pt.Sp[1] * pt.N[A][1] * pt.N[B][1] +
         pt.Sp[2] * pt.N[A][2] * pt.N[B][2] + pt.vs * pt.Ci[A][B];
}

// material modulus entry (A B, C D)
__device__ __forceinline__ double modulus(const Point& pt, int A, int B, int Cc, int D) {
  double c = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      c += pt.L[i][k] * (pt.N[A][i] * pt.N[B][i]) * (pt.N[Cc][k] * pt.N[D][k]);
      if (i != k) c += pt.Lo[i][k] * pt.N[A][i] * pt.N[B][k] * (pt.N[Cc][i] * pt.N[D][k] + pt.N[Cc][k] * pt.N[D][i]);
    }
  return c + pt.v1 * pt.Ci[A][B] * pt.Ci[Cc][D] - pt.v2 * (pt.Ci[A][Cc] * pt.Ci[B][D] + pt.Ci[A][D] * pt.Ci[B][Cc]);
}

}  // namespace hyper
}  // namespace ikr
