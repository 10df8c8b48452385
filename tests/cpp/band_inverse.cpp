// Host check of the coarse operator's band Cholesky inverse (ikr_ls_s::band_spd_inverse, host_internal.h):
// a random symmetric positive definite block-tridiagonal matrix of 6x6 blocks, with one aggregate whose six
// modes have no stiffness and one mode that repeats another.  Prints the largest |A inv - I| over the kept
// modes, the largest entry of the dropped rows and columns, and the number of dropped modes.
#include <cstdio>
#include <random>

#include "../../ikarus_gb300/csrc/host_internal.h"

int main() {
  const int S = 12, n = 6 * S, bw = 11;
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  // A = B B^T + n I restricted to the block band, B random in the band
  std::vector<double> B((size_t)n * n, 0.0), A((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = std::max(0, i - 5); j <= i; ++j) B[(size_t)i * n + j] = u(rng);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += B[(size_t)i * n + k] * B[(size_t)j * n + k];
      A[(size_t)i * n + j] = (std::abs(i / 6 - j / 6) <= 1 ? s : 0.0) + (i == j ? 4.0 : 0.0);
    }
  // aggregate 0 has no free dof: zero rows and columns; mode 6 * 5 + 1 repeats mode 6 * 5
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 6; ++j) A[(size_t)i * n + j] = A[(size_t)j * n + i] = 0.0;
  const int m0 = 30, m1 = 31;
  for (int i = 0; i < n; ++i) A[(size_t)i * n + m1] = A[(size_t)m1 * n + i] = A[(size_t)i * n + m0];
  A[(size_t)m1 * n + m1] = A[(size_t)m0 * n + m0];
  std::vector<double> L, inv;
  const int dropped = ikr_ls_s::band_spd_inverse(A, n, bw, L, inv);
  std::vector<char> keep(n, 1);
  for (int j = 0; j < 6; ++j) keep[j] = 0;
  keep[m1] = 0;
  double err = 0.0, dropped_max = 0.0, asym = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      asym = std::max(asym, std::abs(inv[(size_t)i * n + j] - inv[(size_t)j * n + i]));
      if (!keep[i] || !keep[j]) {
        dropped_max = std::max(dropped_max, std::abs(inv[(size_t)i * n + j]));
        continue;
      }
      double s = 0.0;
      for (int k = 0; k < n; ++k)
        if (keep[k]) s += A[(size_t)i * n + k] * inv[(size_t)k * n + j];
      err = std::max(err, std::abs(s - (i == j ? 1.0 : 0.0)));
    }
  std::printf("%.3e %.3e %.3e %d\n", err, dropped_max, asym, dropped);
  return 0;
}
