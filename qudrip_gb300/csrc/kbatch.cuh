// kbatch.cuh -- batched Krylov real-time steps (one persistent launch).
#pragma once

#include "ham.cuh"

namespace qd {

struct KbArgs {
  int64_t dim;
  const int64_t* rowptr;
  const int32_t* colidx;
  int m;
  int nvec;
  double h;
  const cplx* X;   // input columns (ldx apart); null: unit vectors e_0 .. e_{nvec-1}
  int64_t ldx;
  cplx* Y64;       // output columns, complex128 (may be null)
  float2* Y32;     // output columns, complex64 (may be null)
  int64_t ldy;
  int64_t ld;      // basis leading dimension
  cplx* work;      // per-CTA Krylov bases
  unsigned* counter;
  int* act_out;
};

// Y[:, b] = exp(-i H h) X[:, b] / ||X[:, b]|| with m - 1 Arnoldi products each.
void krylov_batch(qd_ham* H, const cplx* X, int64_t ldx, int nvec, double h, int m, cplx* Y64, float2* Y32,
                  int64_t ldy, int* act_out);

}  // namespace qd
