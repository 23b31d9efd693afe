"""Krylov real-time steps on the device vs the oracle and the dense propagator."""
import numpy as np
import pytest
import scipy.linalg as sl

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import chains
from qudrip_gb300.operators import OperatorSum, getHopFermiGate

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-8  # 2-norm, evolved states


def heff_hubbard(L, Nup, Ndo, U, gamma):
    """H - (i/2) gamma sum_s n_s: the no-jump generator of the trajectory loop."""
    spec, ham = chains.hubbard_chain(L, Nup, Ndo, U, -1.0)
    gate = getHopFermiGate(spec.index)
    for s in range(2 * L):
        ham = ham + (-0.5j * gamma) * gate(s, s)
    return spec, ham


@pytest.mark.parametrize("case", ["hubbard4_real", "hubbard4_heff", "xxz12_complex_state"])
def test_evolve_matches_oracle(ctx, case):
    if case == "hubbard4_real":
        spec, ham = chains.hubbard_chain(4, 2, 2, 4.0, -1.0, periodic=True)
    elif case == "hubbard4_heff":
        spec, ham = heff_hubbard(4, 2, 2, 4.0, 0.1)
    else:
        spec, ham = chains.xxz_chain(12, 1.0, 0.5, True, [0.2 * (i % 5) for i in range(12)])
    oh = O.Ham(O.Sector(spec), ham)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    rng = np.random.default_rng(8)
    psi0 = rng.normal(size=sec.dim) + 1j * rng.normal(size=sec.dim)
    psi0 /= np.linalg.norm(psi0)
    st = q.getState(sec, 2)
    st.set(0, psi0)
    solver = q.Arnoldi.getSolver(sec, 30)
    for h in (0.01, 0.05):
        solver.evolve(H, st(0), 0, h)
        got = st.get(1)
        ref, act = oh.arnoldi_evolve(psi0, h, 30)
        assert solver.act_dim() == act
        assert np.linalg.norm(got - ref) <= STATE_TOL
        exact = sl.expm(-1j * h * oh.scipy().toarray()) @ psi0
        assert np.linalg.norm(got - exact) <= STATE_TOL


def test_evolve_many_steps_unitary(ctx):
    spec, ham = chains.xxz_chain(14)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    psi = q.start_vector(sec.dim, 3).astype(complex)
    psi /= np.linalg.norm(psi)
    st = q.getState(sec, 1)
    st.set(0, psi)
    solver = q.Arnoldi.getSolver(sec, 20)
    e0 = st.eval(0, H)
    for _ in range(20):
        solver.evolve_inplace(H, st, 0, 0.05)
    out = st.get(0)
    assert abs(np.linalg.norm(out) - 1) < 1e-10
    assert abs(st.eval(0, H) - e0) < 1e-9  # energy conserved
    Hd = O.Ham(O.Sector(spec), ham).scipy()
    import scipy.sparse.linalg as sla
    ref = sla.expm_multiply(-1j * 1.0 * Hd, psi)
    assert np.linalg.norm(out - ref) < 1e-8


def test_evolve_breakdown_small_space(ctx):
    spec, ham = chains.hubbard_chain(2, 1, 1, 4.0, -1.0)  # dim 4
    oh = O.Ham(O.Sector(spec), ham)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    psi0 = np.array([1.0, 0.2, -0.3, 0.5], dtype=complex)
    st = q.getState(sec, 2)
    st.set(0, psi0)
    solver = q.Arnoldi.getSolver(sec, 30)
    solver.evolve(H, st(0), 0, 0.1)
    ref, act = oh.arnoldi_evolve(psi0, 0.1, 30)
    assert solver.act_dim() == act <= 4
    assert np.linalg.norm(st.get(1) - ref) <= STATE_TOL
