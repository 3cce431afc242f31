// The single-population genotype estimators of moments: the DD numerator
// polynomial, the Dz quartic and 16 x the pi2 correction (genotype_kernels.py:
// 27-71, 235-279, 364-398), expanded into canonical monomials over the
// moments-order counts g1..g9 (g[0..8]; g[9] = 1) and regrouped as
//   sum_a g[a] * (sum_b g[b] * (sum_c coef_abc * g[c])),
// innermost sums in 32-bit and outer sums in 64-bit integers: exact for
// populations below 32,768 individuals.  Generated by
// tests/golden/make_geno_tables.py.
#pragma once

namespace pgld {
namespace geno {

__host__ __device__ __forceinline__ long long dd_poly(const int* g) {
  return (long long)g[0] * (
        (long long)g[0] * (-16 * g[8] - 4 * g[7] - 4 * g[5] - 1 * g[4]) +
        (long long)g[1] * (-16 * g[8] - 4 * g[5]) +
        (long long)g[2] * (8 * g[7] + 2 * g[4]) +
        (long long)g[3] * (-16 * g[8] - 4 * g[7]) +
        (long long)g[4] * (1 - 18 * g[8] - 4 * g[7] + 2 * g[6] - 4 * g[5] - 1 * g[4]) +
        (long long)g[5] * (4 - 16 * g[8] + 8 * g[6] - 4 * g[5]) +
        (long long)g[7] * (4 - 16 * g[8] - 4 * g[7]) +
        (long long)g[8] * (16 - 16 * g[8])) +
      (long long)g[1] * (
        (long long)g[1] * (-4 * g[8] - 4 * g[6] - 1 * g[5] - 1 * g[3]) +
        (long long)g[2] * (-16 * g[6] - 4 * g[3]) +
        (long long)g[3] * (1 + 2 * g[7] - 4 * g[6] + 2 * g[5] - 1 * g[3]) +
        (long long)g[4] * (-4 * g[8] - 4 * g[6]) +
        (long long)g[5] * (1 - 4 * g[8] + 2 * g[7] - 1 * g[5]) +
        (long long)g[6] * (4 + 8 * g[8] - 4 * g[6]) +
        (long long)g[8] * (4 - 4 * g[8])) +
      (long long)g[2] * (
        (long long)g[2] * (-4 * g[7] - 16 * g[6] - 1 * g[4] - 4 * g[3]) +
        (long long)g[3] * (4 + 8 * g[8] - 16 * g[6] - 4 * g[4] - 4 * g[3]) +
        (long long)g[4] * (1 + 2 * g[8] - 4 * g[7] - 18 * g[6] - 1 * g[4]) +
        (long long)g[5] * (-4 * g[7] - 16 * g[6]) +
        (long long)g[6] * (16 - 16 * g[7] - 16 * g[6]) +
        (long long)g[7] * (4 - 4 * g[7])) +
      (long long)g[3] * (
        (long long)g[3] * (-4 * g[8] - 1 * g[7]) +
        (long long)g[4] * (-4 * g[8]) +
        (long long)g[5] * (2 * g[7]) +
        (long long)g[7] * (1 - 4 * g[8] - 1 * g[7]) +
        (long long)g[8] * (4 - 4 * g[8])) +
      (long long)g[4] * (
        (long long)g[4] * (-1 * g[8] - 1 * g[6]) +
        (long long)g[5] * (-4 * g[6]) +
        (long long)g[6] * (1 + 2 * g[8] - 1 * g[6]) +
        (long long)g[8] * (1 - 1 * g[8])) +
      (long long)g[5] * (
        (long long)g[5] * (-1 * g[7] - 4 * g[6]) +
        (long long)g[6] * (4 - 4 * g[7] - 4 * g[6]) +
        (long long)g[7] * (1 - 1 * g[7]));
}

__host__ __device__ __forceinline__ long long dz_quartic(const int* g) {
  return (long long)g[0] * (
        (long long)g[0] * (-4 * g[8] - 4 * g[7] - 4 * g[5] - 3 * g[4]) +
        (long long)g[1] * (-2 * g[7] + 4 * g[6] - 1 * g[5] - 1 * g[4] + 3 * g[3]) +
        (long long)g[2] * (4 * g[8] + 4 * g[6] + 4 * g[5] + 2 * g[4] + 4 * g[3]) +
        (long long)g[3] * (-1 * g[7] - 2 * g[5] - 1 * g[4]) +
        (long long)g[4] * (2 + 2 * g[8] + 1 * g[7] + 2 * g[6] + 1 * g[5]) +
        (long long)g[5] * (2 - 1 * g[7] + 2 * g[5]) +
        (long long)g[6] * (4 * g[8] + 4 * g[7]) +
        (long long)g[7] * (2 + 2 * g[7]) +
        (long long)g[8] * (8 - 4 * g[8])) +
      (long long)g[1] * (
        (long long)g[1] * (2 * g[8] + 2 * g[6] + 1 * g[5] + 1 * g[3]) +
        (long long)g[2] * (4 * g[8] - 2 * g[7] + 3 * g[5] - 1 * g[4] - 1 * g[3]) +
        (long long)g[3] * (-1 - 1 * g[8] - 2 * g[7] - 1 * g[6] - 2 * g[5] + 1 * g[3]) +
        (long long)g[4] * (1 * g[8] + 1 * g[6]) +
        (long long)g[5] * (-1 - 1 * g[8] - 2 * g[7] - 1 * g[6] + 1 * g[5]) +
        (long long)g[6] * (2 - 2 * g[7] - 4 * g[6]) +
        (long long)g[7] * (-2 * g[8]) +
        (long long)g[8] * (2 - 4 * g[8])) +
      (long long)g[2] * (
        (long long)g[2] * (-4 * g[7] - 4 * g[6] - 3 * g[4] - 4 * g[3]) +
        (long long)g[3] * (2 - 1 * g[7] - 2 * g[5] + 1 * g[4] + 2 * g[3]) +
        (long long)g[4] * (2 + 2 * g[8] + 1 * g[7] + 2 * g[6] - 1 * g[5]) +
        (long long)g[5] * (-1 * g[7]) +
        (long long)g[6] * (8 + 4 * g[8] - 4 * g[6]) +
        (long long)g[7] * (2 + 4 * g[8] + 2 * g[7])) +
      (long long)g[3] * (
        (long long)g[3] * (2 * g[8] + 1 * g[7]) +
        (long long)g[4] * (1 * g[8] - 1 * g[6]) +
        (long long)g[5] * (-2 * g[8] - 2 * g[7] - 2 * g[6]) +
        (long long)g[6] * (4 * g[8] + 3 * g[7]) +
        (long long)g[7] * (-1 - 1 * g[8] + 1 * g[7]) +
        (long long)g[8] * (2 - 4 * g[8])) +
      (long long)g[4] * (
        (long long)g[5] * (-1 * g[8] + 1 * g[6]) +
        (long long)g[6] * (2 + 2 * g[8] - 1 * g[7] - 3 * g[6]) +
        (long long)g[7] * (-1 * g[8]) +
        (long long)g[8] * (2 - 3 * g[8])) +
      (long long)g[5] * (
        (long long)g[5] * (1 * g[7] + 2 * g[6]) +
        (long long)g[6] * (2 + 4 * g[8] - 1 * g[7] - 4 * g[6]) +
        (long long)g[7] * (-1 + 3 * g[8] + 1 * g[7]));
}

__host__ __device__ __forceinline__ long long pi2_corr(const int* g) {
  return (long long)g[0] * (
        (long long)g[0] * (-16 * g[8] - 8 * g[7] - 8 * g[5] - 4 * g[4]) +
        (long long)g[1] * (-44 * g[8] - 36 * g[7] - 28 * g[6] - 24 * g[5] - 20 * g[4] - 16 * g[3]) +
        (long long)g[2] * (-48 * g[8] - 48 * g[7] - 48 * g[6] - 28 * g[5] - 28 * g[4] - 28 * g[3]) +
        (long long)g[3] * (-44 * g[8] - 24 * g[7] - 36 * g[5] - 20 * g[4]) +
        (long long)g[4] * (12 - 48 * g[8] - 40 * g[7] - 28 * g[6] - 40 * g[5] - 16 * g[4]) +
        (long long)g[5] * (16 - 44 * g[8] - 48 * g[7] - 48 * g[6] - 20 * g[5]) +
        (long long)g[6] * (-48 * g[8] - 28 * g[7]) +
        (long long)g[7] * (16 - 44 * g[8] - 20 * g[7]) +
        (long long)g[8] * (16 - 16 * g[8])) +
      (long long)g[1] * (
        (long long)g[1] * (-20 * g[8] - 20 * g[7] - 20 * g[6] - 11 * g[5] - 11 * g[4] - 11 * g[3]) +
        (long long)g[2] * (-28 * g[8] - 36 * g[7] - 44 * g[6] - 16 * g[5] - 20 * g[4] - 24 * g[3]) +
        (long long)g[3] * (13 - 48 * g[8] - 38 * g[7] - 24 * g[6] - 38 * g[5] - 32 * g[4] - 11 * g[3]) +
        (long long)g[4] * (17 - 40 * g[8] - 42 * g[7] - 40 * g[6] - 32 * g[5] - 17 * g[4]) +
        (long long)g[5] * (13 - 24 * g[8] - 38 * g[7] - 48 * g[6] - 11 * g[5]) +
        (long long)g[6] * (16 - 48 * g[8] - 36 * g[7] - 8 * g[6]) +
        (long long)g[7] * (24 - 36 * g[8] - 20 * g[7]) +
        (long long)g[8] * (16 - 8 * g[8])) +
      (long long)g[2] * (
        (long long)g[2] * (-8 * g[7] - 16 * g[6] - 4 * g[4] - 8 * g[3]) +
        (long long)g[3] * (16 - 48 * g[8] - 48 * g[7] - 44 * g[6] - 36 * g[5] - 40 * g[4] - 20 * g[3]) +
        (long long)g[4] * (12 - 28 * g[8] - 40 * g[7] - 48 * g[6] - 20 * g[5] - 16 * g[4]) +
        (long long)g[5] * (-24 * g[7] - 44 * g[6]) +
        (long long)g[6] * (16 - 48 * g[8] - 44 * g[7] - 16 * g[6]) +
        (long long)g[7] * (16 - 28 * g[8] - 20 * g[7])) +
      (long long)g[3] * (
        (long long)g[3] * (-20 * g[8] - 11 * g[7] - 20 * g[5] - 11 * g[4]) +
        (long long)g[4] * (17 - 40 * g[8] - 32 * g[7] - 20 * g[6] - 42 * g[5] - 17 * g[4]) +
        (long long)g[5] * (24 - 36 * g[8] - 38 * g[7] - 36 * g[6] - 20 * g[5]) +
        (long long)g[6] * (-28 * g[8] - 16 * g[7]) +
        (long long)g[7] * (13 - 24 * g[8] - 11 * g[7]) +
        (long long)g[8] * (16 - 8 * g[8])) +
      (long long)g[4] * (
        (long long)g[4] * (11 - 16 * g[8] - 17 * g[7] - 16 * g[6] - 17 * g[5] - 6 * g[4]) +
        (long long)g[5] * (17 - 20 * g[8] - 32 * g[7] - 40 * g[6] - 11 * g[5]) +
        (long long)g[6] * (12 - 28 * g[8] - 20 * g[7] - 4 * g[6]) +
        (long long)g[7] * (17 - 20 * g[8] - 11 * g[7]) +
        (long long)g[8] * (12 - 4 * g[8]) +
        (long long)(-6)) +
      (long long)g[5] * (
        (long long)g[5] * (-11 * g[7] - 20 * g[6]) +
        (long long)g[6] * (16 - 28 * g[8] - 24 * g[7] - 8 * g[6]) +
        (long long)g[7] * (13 - 16 * g[8] - 11 * g[7]));
}

}  // namespace geno
}  // namespace pgld
