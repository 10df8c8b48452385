// Device helpers shared by the element, sparse and solver kernels (sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ikr {

// 2-point Gauss-Legendre abscissae on [0,1]: 1/2 -+ 1/(2 sqrt 3).  With them every Q1 shape-function
// factor at a Gauss point is one of these two numbers (1 - lo == hi).
constexpr double kGaussLo = 0.21132486540518711775;
constexpr double kGaussHi = 0.78867513459481288225;
constexpr double kGaussW = 0.125;  // 2x2x2 rule on the unit cube

// Gauss point q = x + 2y + 4z; Dune vertex v = (v&1, v>>1&1, v>>2&1).
// dN_v/dxi_d at Gauss point q = s_d(v) * prod_{d' != d} (bit_d'(v) == bit_d'(q) ? hi : lo).
template <typename T>
__device__ __forceinline__ void ref_gradient_at_gp(int v, int q, T dxi[3]) {
  const T f0 = (((v ^ q) & 1) == 0) ? T(kGaussHi) : T(kGaussLo);
  const T f1 = (((v ^ q) & 2) == 0) ? T(kGaussHi) : T(kGaussLo);
  const T f2 = (((v ^ q) & 4) == 0) ? T(kGaussHi) : T(kGaussLo);
  dxi[0] = ((v & 1) ? T(1) : T(-1)) * f1 * f2;
  dxi[1] = ((v & 2) ? T(1) : T(-1)) * f0 * f2;
  dxi[2] = ((v & 4) ? T(1) : T(-1)) * f0 * f1;
}
// dN_v/dxi at the element centre (1/2,1/2,1/2)
template <typename T>
__device__ __forceinline__ void ref_gradient_at_center(int v, T dxi[3]) {
  dxi[0] = ((v & 1) ? T(0.25) : T(-0.25));
  dxi[1] = ((v & 2) ? T(0.25) : T(-0.25));
  dxi[2] = ((v & 4) ? T(0.25) : T(-0.25));
}

template <typename T>
__device__ __forceinline__ T det3(const T m[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
         m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}
// inverse of a 3x3 by cofactors; returns the determinant
template <typename T>
__device__ __forceinline__ T inv3(const T m[3][3], T r[3][3]) {
  const T c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  const T c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  const T c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  const T d = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
  const T id = T(1) / d;
  r[0][0] = c00 * id;
  r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
  r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
  r[1][0] = c01 * id;
  r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
  r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
  r[2][0] = c02 * id;
  r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
  r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
  return d;
}

// butterfly sum over the 8 lanes that share an element (lanes 8k..8k+7 of a warp)
template <typename T>
__device__ __forceinline__ T sum8(T v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Voigt pairs in the order 11,22,33,23,13,12
__device__ __forceinline__ int voigt_a(int v) { return v < 3 ? v : (v == 3 ? 1 : 0); }
__device__ __forceinline__ int voigt_b(int v) { return v < 3 ? v : (v == 5 ? 1 : 2); }

}  // namespace ikr
