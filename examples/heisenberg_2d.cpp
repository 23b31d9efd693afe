// 2D Heisenberg model on a periodic square cluster through the C++ drop-in
// headers, written the way programs/two_liquid_sq.cpp drives its model: the
// parameters come from a `name = value` file (param_finder), the cluster is a
// Lattice<2> with periodicity vectors, a Model<double, 2> collects the bonds
// with their params_type, getHamiltonian emits the operator sum that `>>`
// lowers on the device (getHamiltonianMatrix sums per-bond lowered matrices
// instead), the Lanczos ground state gives E0, and McManager writes the
// local <S^z_i S^z_j> correlations with outFile.
//
//   g++ -std=c++17 -O2 examples/heisenberg_2d.cpp -Iinclude -Lqudrip_gb300 -lqudrip_gb300 \
//       -Wl,-rpath,$PWD/qudrip_gb300 -o heisenberg_2d && ./heisenberg_2d params.txt out.tsv
//
// params.txt:  Nx = 4   Ny = 4   J = 1   Jz = 1   krylov = 100   matrix_sum = 0
#include <cstdio>
#include <string>

#include "qudrip_gpu.hpp"
#include "qudrip_gpu_lattice.hpp"
#include "qudrip_gpu_params.hpp"

using namespace qudrip_gpu;

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s params.txt out.tsv\n", argv[0]);
    return 2;
  }
  int Nx = 4, Ny = 4, krylov = 100, matrix_sum = 0;
  double J = 1.0, Jz = 1.0;
  try {
    param_finder pf(argv[1]);
    pf.find_param("Nx", Nx, 1);
    pf.find_param("Ny", Ny, 1);
    pf.find_param("J", J, 1);
    pf.find_param("Jz", Jz, 1);
    pf.find_param("krylov", krylov);
    pf.find_param("matrix_sum", matrix_sum);
  } catch (std::string& missing) {
    std::printf("Missing %s\n", missing.c_str());
    return 1;
  }

  std::vector<c2> coords, pvecs{c2{Nx, 0}, c2{0, Ny}};
  for (int i = 0; i < Nx; ++i)
    for (int j = 0; j < Ny; ++j) coords.push_back(c2{i, j});
  Lattice<2> lat(coords, pvecs);
  params_type<double> param;
  param("J") = J;
  param("Jz") = Jz;
  Model<double, 2> m(lat);
  for (size_t i = 0; i < lat.N(); ++i) {
    const auto& c = lat(i);
    m.addBond((int)i, (int)lat(c + c2{1, 0}), param);
    m.addBond((int)i, (int)lat(c + c2{0, 1}), param);
  }

  const int N = (int)lat.N();
  auto spins = getQbits(N);
  auto nset = getNset(spins);
  auto sector = Constrain(spins, nset = N / 2);
  auto gc = getBoseGate(spins), ga = getBoseGate(spins), gz = getBoseGate(spins);
  gc << 0.5 * (pauli_x + II * pauli_y);
  ga << 0.5 * (pauli_x - II * pauli_y);
  gz << 0.5 * pauli_z;
  auto bond = [&](int s1, int s2, const params_type<double>& p) {
    return (0.5 * p("J")) * (gc(s1) * ga(s2)) + (0.5 * p("J")) * (gc(s2) * ga(s1)) + p("Jz") * (gz(s1) * gz(s2));
  };
  SpMatrix H;
  if (matrix_sum)
    H = m.getHamiltonianMatrix([&](int a, int b, const params_type<double>& p) { return bond(a, b, p) >> sector; },
                               getEmptyOperator() >> sector);
  else
    H = m.getHamiltonian(bond) >> sector;
  std::printf("sites = %d dim = %lld nnz = %lld bonds = %zu\n", N, (long long)sector.range(),
              (long long)H.nonZeros(), m.nbonds());

  auto psi = getState(sector, 1);
  shuffle_state(psi(0));
  auto solver = Arnoldi::getLanczosSolver(sector, krylov);
  solver.getGroundState(H, psi, 0);
  std::printf("E0 = %.15f\n", solver.eigenvalues()[0]);

  McManager mc(1, &psi);
  mc.addObs("SzSz", N, MC_REAL);
  for (int i = 0; i < N; ++i) mc.updateMatrix("SzSz", i, (getEmptyOperator() + 1.0 * (gz(0) * gz(i))) >> sector);
  mc.incrAllObs(0);
  mc.normAll();
  mc.outFile(1.0, argv[2], {"SzSz"});
  std::printf("SzSz(0,1) = %.15f\n", mc.obsValue("SzSz", 0, 1).real());
  return 0;
}
