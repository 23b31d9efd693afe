// evolve.cuh -- buffers of the Krylov real-time step (cached per Hamiltonian).
#pragma once

#include "ham.cuh"

namespace qd {

struct ArnoldiBuffers {
  int64_t n = 0;
  int m = 0;
  int64_t ld = 0;
  int grid_cap = 0;
  DBuf<cplx> V;         // (m + 1) x ld basis
  DBuf<cplx> w;
  DBuf<cplx> proj;      // projections of the current pass
  DBuf<cplx> hcol;      // Hessenberg columns, 64 entries each
  DBuf<double> nrm, nrm2;
  DBuf<int> stop;
  DBuf<cplx> e;         // first column of the small exponential
  DBuf<cplx> partials;  // grid x 32 multi-dot partials
  DBuf<double> rpart;
  DBuf<unsigned> tickets;
  void ensure(int64_t n_, int m_, int grid, cudaStream_t stream);
};

void arnoldi_evolve(qd_ham* H, const cplx* psi_in, cplx* psi_out, double h, int m, int* act_out);

}  // namespace qd
