// fxsum.cuh -- the product with exact fixed-point sums (uniform couplings).
//
// GB300 issues FP64 FMAs at about 1.9 per clock per SM (1.2 TFLOP/s), so a
// FP64 CSR product at L = 24 spends as long in the FP64 pipe (36.6 M FMAs)
// as in HBM, while the integer pipes idle.  Many of the reference's models
// (XY, XXZ/Heisenberg with fields, any uniform hopping) have one value c on
// every off-diagonal entry; then
//     (H x)_r = d_r x_r + c * sum_{k in row r, k != r} x_k,
// and the sum needs no multiplication.  This form stores the diagonal d and
// the off-diagonal columns (int32, no values), keeps beside every Lanczos
// vector a 128-bit fixed-point copy X = round_toward_zero(x * 2^F), and sums
// X over the row with integer adds: the sum is exact, rounded once to FP64.
// F is fixed per Hamiltonian from the bound |x_i| <= max(1, ||H||_inf) that
// every Lanczos vector obeys (unit start vector; n_k <= ||H||), leaving 7
// bits of headroom for up to 128 summands: F = 119 - ceil(log2(bound)), so
// elements down to 2^-66 of the bound convert exactly and the result is at
// least as accurate as a sequential FP64 sum.  A value above the bound sets
// an overflow flag and the solver reruns on the FP64 CSR product.
#pragma once

#include "common.cuh"

namespace qd {

struct FxForm {
  DBuf<int32_t> rowptr;  // dim + 1 (off-diagonal entries only)
  DBuf<int32_t> colidx;  // off-diagonal columns, ascending within each row
  DBuf<double> diag;     // d_r (0 where the CSR has no diagonal entry)
  double c = 0.0;        // the common off-diagonal value
  int F = 0;             // fixed-point scale 2^F
  int64_t nnz = 0;
};

#ifdef __CUDACC__
// x * 2^F rounded toward zero into a signed 128-bit integer; flags |x| >= 2^(126 - 7 - F).
__device__ __forceinline__ __int128 fx_from_double(double x, int F, int* ovf) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ffu);
  if (e == 0) return 0;  // zero or subnormal: below the quantum
  const unsigned long long m = (bits & 0xfffffffffffffull) | (1ull << 52);
  const int sh = e - 1075 + F;  // x * 2^F = m * 2^sh
  unsigned __int128 v;
  if (sh >= 0) {
    if (sh > 126 - 7 - 53) {
      if (ovf) *ovf = 1;
      return 0;
    }
    v = (unsigned __int128)m << sh;
  } else if (sh > -64) {
    v = (unsigned __int128)(m >> (-sh));
  } else {
    v = 0;
  }
  const __int128 s = (__int128)v;
  return (bits >> 63) ? -s : s;
}
#endif

}  // namespace qd
