// Device helpers shared by the batched eigensolver (eig_f64.cu) and the bidiagonal SVD
// (svd_bidiag.cu): warp reductions and inverse iteration on a shifted tridiagonal matrix (partially
// pivoted LU, Wilkinson, The Algebraic Eigenvalue Problem, chapter 5).  Each translation unit gets
// its own copy (internal linkage).
#pragma once
#include <cfloat>
#include <cstdint>

namespace mpsg {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

__device__ __forceinline__ double hash_unit(uint32_t a, uint32_t b) {  // deterministic value in [-1, 1)
  uint64_t z = ((uint64_t)a << 32) ^ b ^ 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// Partially pivoted LU of T - lam I (rows i, i+1 swapped when the subdiagonal entry is larger than the
// pivot); zero pivots are replaced by eps * tnorm.  u0 holds the reciprocal pivots, u1, u2 the first
// and second superdiagonals of U, mul the multipliers, piv the interchange flags.
// d == nullptr: zero diagonal (the Golub-Kahan matrix of a bidiagonal)
__device__ void tri_shift_factor(const double* d, const double* e, int n, double lam, double tnorm, double* u0,
                                 double* u1, double* u2, double* mul, unsigned char* piv) {
  const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  double dd = (d ? d[0] : 0.0) - lam, du = n > 1 ? e[0] : 0.0;
  for (int i = 0; i + 1 < n; ++i) {
    const double sub = e[i];
    const double dnext = (d ? d[i + 1] : 0.0) - lam;
    const double dunext = i + 2 < n ? e[i + 1] : 0.0;
    if (fabs(dd) >= fabs(sub)) {
      if (dd == 0.0) dd = tiny;
      const double inv = 1.0 / dd;
      const double l = sub * inv;
      u0[i] = inv; u1[i] = du; u2[i] = 0.0; mul[i] = l; piv[i] = 0;
      dd = dnext - l * du;
      du = dunext;
    } else {
      const double l = dd / sub;
      u0[i] = 1.0 / sub; u1[i] = dnext; u2[i] = dunext; mul[i] = l; piv[i] = 1;
      dd = du - l * dnext;
      du = -l * dunext;
    }
  }
  if (dd == 0.0) dd = tiny;
  u0[n - 1] = 1.0 / dd;
}
// x <- c (T - lam I)^-1 x with the factors of tri_shift_factor, for some c > 0: whenever an entry
// passes 2^166 (~1e50) the whole vector is scaled by 2^-166, so that products of reciprocal tiny
// pivots (near-singular shifts, clusters) cannot overflow (the caller normalises the result).
__device__ __forceinline__ void tri_rescale(int n, double* x, double v) {
  if (fabs(v) > 0x1p+166)
    for (int k = 0; k < n; ++k) x[k] *= 0x1p-166;
}
__device__ void tri_shift_solve(int n, double* x, const double* u0, const double* u1, const double* u2,
                                const double* mul, const unsigned char* piv) {
  for (int i = 0; i + 1 < n; ++i) {
    if (piv[i]) {
      const double t = x[i];
      x[i] = x[i + 1];
      x[i + 1] = t - mul[i] * x[i];
    } else {
      x[i + 1] -= mul[i] * x[i];
    }
    tri_rescale(n, x, x[i + 1]);
  }
  x[n - 1] *= u0[n - 1];
  tri_rescale(n, x, x[n - 1]);
  if (n >= 2) {
    x[n - 2] = (x[n - 2] - u1[n - 2] * x[n - 1]) * u0[n - 2];
    tri_rescale(n, x, x[n - 2]);
  }
  for (int i = n - 3; i >= 0; --i) {
    x[i] = (x[i] - u1[i] * x[i + 1] - u2[i] * x[i + 2]) * u0[i];
    tri_rescale(n, x, x[i]);
  }
}

}  // namespace
}  // namespace mpsg
