"""Incremental Arnoldi ground state vs the oracle.

Arnoldi::getSolver(index, kry_dim).getGroundState(H, psi, 0, Niter) in the
convergence loop of programs/two_liquid_sq.cpp:464-476 -- convergeEV, repeated
calls of Niter steps each until error() falls below eps or the space is full
(sparse_algorithm.hpp:494-500, 521-546, 564-585 with expandBasis<0>
:372-393).  After every call the device's Krylov eigenvalues match the oracle's
restatement run to the same dimension within 1e-10, the Ritz vector is the
oracle's up to its sign (the eigensolver fixes no sign), and error() is the
change of the tracked eigenvalues.
"""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import chains
from qudrip_gb300.operators import getHopFermiGate

pytestmark = pytest.mark.gpu


def converge_loop(spec, ham, kry_dim, niter, nconv, iv, seed):
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    oh = O.Ham(O.Sector(spec), ham)
    v0 = q.start_vector(sec.dim, seed).astype(np.complex128)
    psi = q.getState(sec, 1)
    psi.set(0, v0)
    solver = q.Arnoldi.getSolver(sec, kry_dim)
    solver.convergeEV(nconv, iv)
    prev = np.full(nconv, iv)
    calls = 0
    while solver.act_dim() < kry_dim:
        solver.getGroundState(H, psi, 0, niter)
        calls += 1
        act = solver.act_dim()
        assert act == min(calls * niter, kry_dim) or solver.result.breakdown
        ref = oh.arnoldi_ground(v0, act)
        assert ref["act_dim"] == act
        ev = solver.eigenvalues()
        assert np.allclose(ev, ref["evals"], rtol=0, atol=1e-10 * max(1.0, np.abs(ref["evals"]).max()))
        m = min(nconv, act)
        assert abs(solver.error() - np.sqrt(np.sum((ev[:m] - prev[:m]) ** 2))) <= 1e-12 * (1 + np.abs(ev[:m]).max())
        prev[:m] = ev[:m]
        g = psi.get(0)
        ov = abs(np.vdot(ref["psi"], g))
        assert abs(ov - 1.0) <= 1e-8 and abs(np.linalg.norm(g) - 1.0) <= 1e-10
        if abs(solver.error()) < 1e-10:
            break
    return solver, sec, H, psi, calls


def test_convergence_loop_hermitian(ctx):
    """XXZ chain with random fields (L=12, dim 924), kry_dim 80, Niter 10, two tracked
    eigenvalues starting at 0: grows until the lowest two stop moving."""
    h = np.random.default_rng(3).uniform(-1.0, 1.0, 12)
    spec, ham = chains.xxz_chain(12, 1.0, 0.7, True, h)
    solver, sec, H, psi, calls = converge_loop(spec, ham, 80, 10, 2, 0.0, 17)
    assert solver.error() < 1e-10 and calls >= 3
    # the converged Ritz value is the lowest eigenvalue of H
    import scipy.sparse.linalg as sla
    oh = O.Ham(O.Sector(spec), ham)
    e0 = sla.eigsh(oh.scipy().tocsr(), k=1, which="SA", tol=1e-13)[0][0]
    assert abs(solver.eigenvalues()[0] - e0) <= 1e-10 * abs(e0)
    # the loop stopped on error() before the space was full
    assert solver.act_dim() < 80


def test_convergence_loop_non_hermitian(ctx):
    """The no-jump generator of the dissipative Hubbard chain (L=4, 2+2 fermions, dim 36,
    H - (i/2) gamma sum n): the eigensolve reads the Arnoldi matrix's lower triangle (real
    parts of the diagonal, sub-diagonal norms) as the reference's SelfAdjointEigenSolver does."""
    spec, ham = chains.hubbard_chain(4, 2, 2, 4.0, -1.0)
    gate = getHopFermiGate(spec.index)
    for s in range(8):
        ham = ham + (-0.05j * (1 + s % 3)) * gate(s, s)
    converge_loop(spec, ham, 30, 6, 3, 0.0, 5)


def test_full_space_and_breakdown(ctx):
    """kry_dim beyond the sector dimension: the space closes by breakdown (the breaking
    step counts, expandBasis<0>), later calls return at once, and the Ritz value is exact."""
    spec, ham = chains.xxz_chain(6, 1.0, 1.0, True)  # dim 20
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    oh = O.Ham(O.Sector(spec), ham)
    v0 = q.start_vector(sec.dim, 2).astype(np.complex128)
    psi = q.getState(sec, 1)
    psi.set(0, v0)
    solver = q.Arnoldi.getSolver(sec, 40)
    r = solver.getGroundState(H, psi, 0, -1)
    ref = oh.arnoldi_ground(v0, 40)
    assert r.breakdown == 1 and r.act_dim == ref["act_dim"]
    assert np.allclose(solver.eigenvalues(), ref["evals"], atol=1e-10)
    e = np.linalg.eigvalsh(oh.scipy().toarray())
    assert abs(solver.eigenvalues()[0] - e[0]) <= 1e-10
    before = psi.get(0)
    solver.getGroundState(H, psi, 0, 5)
    assert np.array_equal(psi.get(0), before)


def test_cpp_header_arnoldi_ground_state(ctx):
    """The same loop through include/qudrip_gpu.hpp, as a reference program writes it."""
    import os
    import subprocess
    import tempfile
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = r'''
#include "qudrip_gpu.hpp"
#include <cstdio>
using namespace qudrip_gpu;
int main() {
  const int L = 10;
  auto pre = getQbits(L);
  auto Nset = getNset(pre);
  auto chain = Constrain(pre, Nset = L / 2);
  auto gc = getBoseGate(pre), ga = getBoseGate(pre), gz = getBoseGate(pre);
  gc << 0.5 * (pauli_x + II * pauli_y);
  ga << 0.5 * (pauli_x - II * pauli_y);
  gz << 0.5 * pauli_z;
  auto ham = getEmptyOperator();
  for (int i = 0; i < L; ++i) {
    int j = (i + 1) % L;
    ham = ham + 0.5 * (gc(i) * ga(j)) + 0.5 * (gc(j) * ga(i)) + gz(i) * gz(j);
  }
  auto H = ham >> chain;
  auto psi = getState(chain, 1);
  shuffle_state(psi(0));
  auto solver = Arnoldi::getSolver(chain, 60);
  solver.convergeEV(2, 0.0);
  int calls = 0;
  while (solver.act_dim() < 60) {
    solver.getGroundState(H, psi(0), 0, 10);
    ++calls;
    if (std::abs(solver.error()) < 1e-10) break;
  }
  std::printf("%d %d %.15f\n", calls, solver.act_dim(), solver.eigenvalues()[0]);
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        cpp = os.path.join(d, "arnoldi_gs.cpp")
        exe = os.path.join(d, "arnoldi_gs")
        with open(cpp, "w") as f:
            f.write(src)
        lib = os.path.join(root, "qudrip_gb300")
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(root, "include"), cpp, "-o", exe,
                        "-L", lib, "-lqudrip_gb300", "-Wl,-rpath," + lib], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    calls, act, e0 = int(out[0]), int(out[1]), float(out[2])
    spec, ham = chains.xxz_chain(10, 1.0, 1.0, True)
    oh = O.Ham(O.Sector(spec), ham)
    ev = np.linalg.eigvalsh(oh.scipy().toarray())
    assert abs(e0 - ev[0]) <= 1e-10 * abs(ev[0]) and act == 10 * calls
