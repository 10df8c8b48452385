// Enhanced-assumed-strain Q1 hexahedra: centre data, state update, stresses and the element launches for the
// NeoHooke, StVenantKirchhoff and BlatzKo laws (the kernel template is in element_eas.cuh).
#include "element_eas.cuh"

namespace ikr {

namespace {

// Per-element centre data (helperfunctions.hh:19-36): GL: (T(J0) detJ0)^{-1} (36, row-major);
// H / HT: J0^{-T} (9, row-major), detJ0; HT also grad N_v at the centre (24).
__global__ void eas_geometry_kernel(const double* __restrict__ X, const int32_t* __restrict__ conn, int ne, int kind,
                                    double* __restrict__ geo, int* status) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double Xe[8][3];
  for (int v = 0; v < 8; ++v) {
    const int n = conn[v * ne + e];
    for (int c = 0; c < 3; ++c) Xe[v][c] = X[3 * n + c];
  }
  double J[3][3] = {};
  for (int v = 0; v < 8; ++v) {
    double d[3];
    ref_gradient_at_center<double>(v, d);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) J[i][j] += Xe[v][i] * d[j];
  }
  double Ji[3][3];
  const double detJ0 = inv3(J, Ji);
  if (kind == 1) {
    // strain transformation T[(a,b)][(c,d)] = (a==b ? 1/2 : 1)(Jt[a][c] Jt[b][d] + Jt[b][c] Jt[a][d]), Jt = J^T
    // (tensorutils.hh:438-465), scaled by detJ0 and inverted
    double A[6][12];
    for (int r = 0; r < 6; ++r) {
      const int a = voigt_a(r), b = voigt_b(r);
      for (int s = 0; s < 6; ++s) {
        const int c = voigt_a(s), d = voigt_b(s);
        const double v = J[c][a] * J[d][b] + J[c][b] * J[d][a];
        A[r][s] = (a == b ? 0.5 * v : v) * detJ0;
        A[r][6 + s] = (r == s) ? 1.0 : 0.0;
      }
    }
    for (int k = 0; k < 6; ++k) {  // Gauss-Jordan with partial pivoting
      int p = k;
      for (int i = k + 1; i < 6; ++i)
        if (fabs(A[i][k]) > fabs(A[p][k])) p = i;
      if (!(fabs(A[p][k]) > 0.0)) {
        atomicOr(status, kStatusSingularD);
        return;
      }
      if (p != k)
        for (int j = 0; j < 12; ++j) {
          const double t = A[k][j];
          A[k][j] = A[p][j];
          A[p][j] = t;
        }
      const double inv = 1.0 / A[k][k];
      for (int j = 0; j < 12; ++j) A[k][j] *= inv;
      for (int i = 0; i < 6; ++i) {
        if (i == k) continue;
        const double l = A[i][k];
        if (l == 0.0) continue;
        for (int j = 0; j < 12; ++j) A[i][j] -= l * A[k][j];
      }
    }
    for (int r = 0; r < 6; ++r)
      for (int s = 0; s < 6; ++s) geo[(size_t)(6 * r + s) * ne + e] = A[r][6 + s];
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) geo[(size_t)(3 * i + j) * ne + e] = Ji[j][i];
    geo[(size_t)9 * ne + e] = detJ0;
    if (kind == 3)
      for (int v = 0; v < 8; ++v) {
        double d[3];
        ref_gradient_at_center<double>(v, d);
        for (int k = 0; k < 3; ++k)
          geo[(size_t)(10 + 3 * v + k) * ne + e] = d[0] * Ji[0][k] + d[1] * Ji[1][k] + d[2] * Ji[2][k];
      }
  }
}

// alpha_e -= D^{-1} R~ + D^{-1} L dd_e (enhancedassumedstrains.hh:243), 8 lanes per element
template <int NA>
__global__ void eas_update_kernel(ElemArgs a, double* __restrict__ alpha, const double* __restrict__ corr) {
  const int sub = threadIdx.x & 7;
  const int e0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int ne = a.n_elems;
  const bool active = e0 < ne;
  const int e = active ? e0 : ne - 1;
  const int node = a.conn[sub * ne + e];
  double dd[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) dd[c] = corr[3 * node + c];
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    double t = 0.0;
#pragma unroll
    for (int b = 0; b < 3; ++b) t += a.eas_Y[(size_t)(k * 24 + 3 * sub + b) * ne + e] * dd[b];
    t = sum8(t);
    if (active && sub == 0) alpha[(size_t)k * ne + e] -= a.eas_y[(size_t)k * ne + e] + t;
  }
}

// calculateAt of EAS elements (enhancedassumedstrains.hh:127-188), one thread per element, FP64: the stored alpha
// enhances the strain at the local point xi.  GL (E9/E21): E = E(H_c) + M(xi) alpha, F = I + H_c; H9 / H9T: the
// displacement gradient H = H_c + H~ (or H_c + F_c0 H~^T), F = I + H, E = E(H).  type 0 PK2, 1 Kirchhoff, 2 Cauchy.
__global__ void eas_stress_at_kernel(ElemArgs a, int e0, int count, const double* __restrict__ xi, int xi_per_elem,
                                     int type, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int e = e0 + k;
  const int ne = a.n_elems;
  const int kind = a.eas_kind, na = a.n_alpha;
  const double* x = xi + (xi_per_elem ? 3 * k : 0);
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double dxi[8][3], U[8][3];
  for (int v = 0; v < 8; ++v) {
    const int node = a.conn[v * ne + e];
    double f[3], df[3];
    for (int d = 0; d < 3; ++d) {
      const bool b = (v >> d) & 1;
      f[d] = b ? x[d] : 1.0 - x[d];
      df[d] = b ? 1.0 : -1.0;
    }
    dxi[v][0] = df[0] * f[1] * f[2];
    dxi[v][1] = f[0] * df[1] * f[2];
    dxi[v][2] = f[0] * f[1] * df[2];
    for (int c = 0; c < 3; ++c) U[v][c] = a.u ? a.u[3 * node + c] : 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) J[i][j] += a.X[3 * node + i] * dxi[v][j];
  }
  double Ji[3][3];
  const double detJ = inv3(J, Ji);
  double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int v = 0; v < 8; ++v) {
    double dN[3];
    for (int kk = 0; kk < 3; ++kk) dN[kk] = dxi[v][0] * Ji[0][kk] + dxi[v][1] * Ji[1][kk] + dxi[v][2] * Ji[2][kk];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) H[i][j] += U[v][i] * dN[j];
  }
  if (kind != 1) {  // H9 / H9T enhancement of the gradient
    double A0[3][3], Ht[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) A0[i][j] = a.eas_geo[(size_t)(3 * i + j) * ne + e];
    const double sc = a.eas_geo[(size_t)9 * ne + e] / detJ;
    for (int p = 0; p < na; ++p) {
      const int r = p / 3, c = p % 3;
      const double w = a.alpha[(size_t)p * ne + e] * sc * (2.0 * x[c] - 1.0);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Ht[i][j] += w * A0[i][r] * A0[j][c];
    }
    if (kind == 2) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[i][j] += Ht[i][j];
    } else {
      double Fc0[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double t = (i == j) ? 1.0 : 0.0;
          for (int v = 0; v < 8; ++v) t += U[v][i] * a.eas_geo[(size_t)(10 + 3 * v + j) * ne + e];
          Fc0[i][j] = t;
        }
      double add[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) add[i][j] = Fc0[i][0] * Ht[j][0] + Fc0[i][1] * Ht[j][1] + Fc0[i][2] * Ht[j][2];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[i][j] += add[i][j];
    }
  }
  double Ev[6];
  {
    double E[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        E[i][j] = 0.5 * (H[i][j] + H[j][i] + H[0][i] * H[0][j] + H[1][i] * H[1][j] + H[2][i] * H[2][j]);
    Ev[0] = E[0][0], Ev[1] = E[1][1], Ev[2] = E[2][2];
    Ev[3] = 2.0 * E[1][2], Ev[4] = 2.0 * E[0][2], Ev[5] = 2.0 * E[0][1];
  }
  if (kind == 1) {  // GL: E += (T0^{-1} / detJ) M0(xi) alpha
    for (int q = 0; q < na; ++q) {
      double v = 2.0 * x[kF1[q]] - 1.0;
      if (kF2[q] >= 0) v *= 2.0 * x[kF2[q]] - 1.0;
      const double w = v / detJ * a.alpha[(size_t)q * ne + e];
      for (int r = 0; r < 6; ++r) Ev[r] += w * a.eas_geo[(size_t)(6 * r + kRow[q]) * ne + e];
    }
  }
  const double lam = a.lam_e ? a.lam_e[e] : a.lam, mu = a.mu_e ? a.mu_e[e] : a.mu;
  double S[3][3];
  double C[3][3];
  C[0][0] = 2.0 * Ev[0] + 1.0, C[1][1] = 2.0 * Ev[1] + 1.0, C[2][2] = 2.0 * Ev[2] + 1.0;
  C[1][2] = C[2][1] = Ev[3];
  C[0][2] = C[2][0] = Ev[4];
  C[0][1] = C[1][0] = Ev[5];
  if (a.material == 1) {
    const double trE = Ev[0] + Ev[1] + Ev[2];
    for (int v = 0; v < 6; ++v) {
      const int i = voigt_a(v), j = voigt_b(v);
      S[i][j] = S[j][i] = v < 3 ? lam * trE + 2.0 * mu * Ev[v] : mu * Ev[v];
    }
  } else if (a.material == 3) {  // hyperelastic framework
    hyper::Point pt;
    const int bad = hyper::evaluate(a.hyper, C, pt, false);
    if (bad && a.status) atomicOr(a.status, bad);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] = hyper::stress(pt, i, j);
  } else {
    double Ci[3][3];
    const double detC = inv3(C, Ci);
    if (!(detC > 1e-10) && a.status) atomicOr(a.status, kStatusNonPositiveDetC);
    if (a.material == 2) {  // BlatzKo
      const double Jd = sqrt(detC);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          S[i][j] = mu * (Jd * Ci[i][j] - (Ci[i][0] * Ci[0][j] + Ci[i][1] * Ci[1][j] + Ci[i][2] * Ci[2][j]));
    } else {
      const double lnJ = log(sqrt(detC));
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) S[i][j] = mu * ((i == j ? 1.0 : 0.0) - Ci[i][j]) + lam * lnJ * Ci[i][j];
    }
  }
  double R[3][3];
  if (type == 0) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[i][j] = S[i][j];
  } else {
    double F[3][3], FS[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) FS[i][j] = F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j];
    const double scl = type == 2 ? 1.0 / det3(F) : 1.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[i][j] = scl * (FS[i][0] * F[j][0] + FS[i][1] * F[j][1] + FS[i][2] * F[j][2]);
  }
  double* o = out + 6 * (size_t)k;
  o[0] = R[0][0], o[1] = R[1][1], o[2] = R[2][2], o[3] = R[1][2], o[4] = R[0][2], o[5] = R[0][1];
}

}  // namespace

void launch_eas_stress_at(const ElemArgs& a, int e0, int count, const double* xi, bool xi_per_elem, int type,
                          double* out, cudaStream_t s) {
  if (count <= 0) return;
  eas_stress_at_kernel<<<(count + 127) / 128, 128, 0, s>>>(a, e0, count, xi, xi_per_elem ? 1 : 0, type, out);
}

int eas_geo_stride(int kind) { return kind == 1 ? 36 : (kind == 3 ? 34 : 10); }

void launch_eas_element(const ElemArgs& a, int mode, bool fp32, const int32_t* list, int n, int base,
                        cudaStream_t s) {
  if (n <= 0) return;
  if (a.material == 3) launch_eas_element_hyper(a, mode, fp32, list, n, base, s);  // element_eas_hyper.cu
  else launch_eas_family<false>(a, mode, fp32, list, n, base, s);
}

void launch_eas_geometry(const ElemArgs& a, double* geo_out, cudaStream_t s) {
  eas_geometry_kernel<<<(a.n_elems + 127) / 128, 128, 0, s>>>(a.X, a.conn, a.n_elems, a.eas_kind, geo_out, a.status);
}

void launch_eas_update(const ElemArgs& a, double* alpha, const double* corr, cudaStream_t s) {
  const int blocks = (int)((8LL * a.n_elems + 255) / 256);
  if (a.n_alpha == 9) eas_update_kernel<9><<<blocks, 256, 0, s>>>(a, alpha, corr);
  else if (a.n_alpha == 21) eas_update_kernel<21><<<blocks, 256, 0, s>>>(a, alpha, corr);
}

}  // namespace ikr
