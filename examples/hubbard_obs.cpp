// Hubbard chain through the C++ drop-in header: ground state with
// Hermitian::LanczosSolver (as programs/hubbard_diss.cpp prepares its initial
// state), Krylov real-time steps with Arnoldi::getSolver(...).evolve, and the
// double occupancy <n_i,up n_i,dn>(t) accumulated by McManager.
//
//   g++ -std=c++17 -O2 examples/hubbard_obs.cpp -Iinclude -Lqudrip_gb300 -lqudrip_gb300 \
//       -Wl,-rpath,$PWD/qudrip_gb300 -o hubbard_obs && ./hubbard_obs
#include <cstdio>
#include <string>

#include "qudrip_gpu.hpp"

using namespace qudrip_gpu;

int main() {
  const int L = 4, nt = 6;
  const double U = 4.0, thop = -1.0, dt = 0.05;
  auto fermi = getQbits(2 * L);
  auto nup = getNup(fermi, L);
  auto ndo = getNdo(fermi, L);
  auto chain = Constrain(fermi, nup = 2, ndo = 2);
  auto gate = getHopFermiGate(fermi);
  auto ham = getEmptyOperator();
  for (int i = 0; i < L; ++i) {
    const int j = (i + 1) % L;
    ham = ham + thop * gate(j, i) + thop * gate(i, j) + thop * gate(j + L, i + L) + thop * gate(i + L, j + L);
  }
  for (int i = 0; i < L; ++i) ham = ham + U * (gate(i, i) * gate(i + L, i + L));
  auto H = ham >> chain;
  std::printf("dim = %lld\n", (long long)chain.range());

  auto psi = getState(chain, nt);
  shuffle_state(psi(0));
  Hermitian::LanczosSolver gs(chain, 60);
  gs.getGroundState(H, psi, 0);
  std::printf("E0 = %.15f\n", gs.eigenvalues()[0]);

  McManager mc(nt, &psi);
  mc.addObs("docc", L);
  for (int i = 0; i < L; ++i) {
    auto d = getEmptyOperator() + 1.0 * (gate(i, i) * gate(i + L, i + L));
    mc.updateMatrix("docc", i, d >> chain);
  }
  auto solver = Arnoldi::getSolver(chain, 20);
  for (int t = 0; t < nt; ++t) {
    if (t > 0) solver.evolve(H, psi, t - 1, dt);
    mc.incrAllObs(t);
  }
  mc.normAll();
  for (int t = 0; t < nt; ++t) std::printf("docc0(%d) = %.15f\n", t, mc.value("docc", t, 0).real());
  return 0;
}
