// XY chain ground state through the C++ drop-in header (the README example of
// QuDrip, programs/spin.cpp, with only the include and namespace changed and
// a seeded start vector).
//
//   g++ -std=c++17 -O2 examples/spin.cpp -Iinclude -Lqudrip_gb300 -lqudrip_gb300 \
//       -Wl,-rpath,$PWD/qudrip_gb300 -o spin && ./spin 16
#include <chrono>
#include <cstdio>
#include <iostream>
#include <string>

#include "qudrip_gpu.hpp"

using namespace qudrip_gpu;

int main(int argc, char** argv) {
  const int Nsite = argc > 1 ? std::stoi(argv[1]) : 16;
  auto prechain = getQbits(Nsite);
  auto Nset = getNset(prechain);
  auto gc = getBoseGate(prechain);
  auto ga = getBoseGate(prechain);

  auto chain = Constrain(prechain, Nset = Nsite / 2);
  std::cout << "dimension of Hil space = " << chain.range() << std::endl;

  Matrix Uc = 0.5 * (pauli_x + II * pauli_y);
  Matrix Ua = 0.5 * (pauli_x - II * pauli_y);
  gc << Uc;
  ga << Ua;

  auto t0 = std::chrono::steady_clock::now();
  auto ham = getEmptyOperator();
  for (int i = 0; i < Nsite - 1; ++i) ham = ham + gc(i + 1) * ga(i) + gc(i) * ga(i + 1);
  auto ham_mat = ham >> chain;
  auto t1 = std::chrono::steady_clock::now();
  std::cout << "nnz = " << ham_mat.nonZeros() << ", lowered in "
            << std::chrono::duration<double>(t1 - t0).count() << " s" << std::endl;

  int krylov_dim = 100;
  auto psi = getState(chain, 1);
  shuffle_state(psi(0));
  auto solver = Arnoldi::getLanczosSolver(chain, krylov_dim);
  solver.getGroundState(ham_mat, psi(0), 0);

  auto E = psi.eval(0, ham_mat);
  std::printf("ritz = %.15f\nE = %.15f %.3e\n", solver.eigenvalues()[0], E.real(), E.imag());
  return 0;
}
