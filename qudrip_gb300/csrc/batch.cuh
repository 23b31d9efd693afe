// batch.cuh -- work-list entries of the batched (persistent) Lanczos solver.
#pragma once

#include "ham.cuh"

namespace qd {

struct BatchInst {
  int64_t dim;
  int steps;
  int pad;
  int64_t ld;
  const int64_t* rowptr;
  const int32_t* colidx;
  const float* vals_f;   // FP32 copy of the values
  const int* uniform;    // device flag: every off-diagonal value is *coff (the product reads no values)
  const float* coff;
  const float* diag_f;   // uniform form: d_r - c where row r stores its diagonal, else 0
  const double* vals_d;  // FP64 values (refinement)
  const float* v0;       // start vector
  float* V;              // (steps + 1) x ld Krylov basis
  float* w;
  float* psi;            // Ritz vector
  double* out;           // ritz value, refined energy, psi^T psi, act_dim, breakdown
};

void batch_lanczos(Ctx* ctx, qd_ham* const* hams, const double* const* v0s, int ninst, int steps, double* out);

}  // namespace qd
