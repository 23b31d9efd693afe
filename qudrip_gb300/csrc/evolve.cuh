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
  // the m - 1 Arnoldi steps captured once and replayed (they read and write only these
  // buffers and the Hamiltonian's arrays, so the graph stays valid while neither changes)
  cudaGraphExec_t steps_exec = nullptr;
  int steps_m = 0, steps_kind = 0, steps_variant = -1;
  const void* steps_vals = nullptr;  // the matrix arrays the graph reads
  const void* steps_rowptr = nullptr;
  long long steps_seen = -1;  // key of the last uncaptured run (its lazy allocations are done)
  int64_t steps_kernels = 0;
  void ensure(int64_t n_, int m_, int grid, cudaStream_t stream);
  void drop_graph();
  ~ArnoldiBuffers() { drop_graph(); }
};

void arnoldi_evolve(qd_ham* H, const cplx* psi_in, cplx* psi_out, double h, int m, int* act_out);

// Solve state of the Arnoldi ground state (ArnoldiSolver<T, herm=0>::getGroundState), kept per
// Hamiltonian so that a later call can grow the same Krylov space.
struct ArnoldiGround {
  int64_t n = 0;
  int kdim = 0;
  int64_t ld = 0;
  int ldh = 0;          // Hessenberg column stride (kdim + 1)
  int grid_cap = 0;
  int act = 0;          // Krylov dimension reached (act_dim)
  bool open = false;    // a solve that a later call may grow
  bool broke = false;   // the last step broke down (||w|| < 1e-10)
  DBuf<cplx> V;         // (kdim + 1) x ld orthonormal basis
  DBuf<cplx> w;
  DBuf<cplx> proj;      // projections of the current pass (kdim + 1)
  DBuf<cplx> hcol;      // Hessenberg column i at i * ldh: <v_j, H v_i>, j <= i
  DBuf<double> nrm, nrm2;
  DBuf<int> stop;
  DBuf<cplx> e;         // Ritz coefficients
  DBuf<cplx> partials;  // grid x 32 multi-dot partials
  DBuf<double> rpart;
  DBuf<unsigned> tickets;
  void ensure(int64_t n_, int kdim_, int grid, cudaStream_t stream);
};

// psi = Ritz vector of the lowest eigenvalue of the symmetric tridiagonal matrix read from the
// Arnoldi matrix's lower triangle.  extend = false starts from psi (initKrylov); true grows the
// open solve.  add_dim <= 0 or beyond kry_dim: up to kry_dim.
void arnoldi_ground(qd_ham* H, cplx* psi, int kdim, int add_dim, bool extend, double* evals_out,
                    qd_lanczos_result* res);

}  // namespace qd
