"""Edge cases of the device path: an empty sector, a one-state sector, argument limits, and a
sector whose Krylov space closes after one step.  The reference has no tests of its own; where its
behaviour is undefined (a 0 x 0 Lanczos matrix) the engine reports an error code instead."""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains

pytestmark = pytest.mark.gpu


def sector(spec):
    return q.Sector(spec.index, spec.constraints, spec.tight)


def test_empty_sector(ctx):
    spec, ham = chains.xxz_chain(8, 1.0, 1.0, periodic=True)
    pre = spec.index
    empty = q.SectorSpec(pre, [q.getNset(pre) == 9])  # more particles than sites: no state
    sec = sector(empty)
    assert sec.dim == 0 and len(sec.basis()) == 0
    H = sec.lower(ham)
    assert H.dim == 0 and H.nnz == 0
    with pytest.raises(A.QDError) as e:
        q.getState(sec, 1)
    assert e.value.code == A.QD_ERR_INVALID
    assert (H + H).nnz == 0


def test_one_state_sector(ctx):
    L = 6
    h = np.linspace(-1.0, 1.0, L)
    spec, ham = chains.xxz_chain(L, 1.0, 0.5, periodic=True, fields=h)
    pre = spec.index
    vac = q.SectorSpec(pre, [q.getNset(pre) == 0])  # the empty chain only
    sec = sector(vac)
    assert sec.dim == 1 and list(sec.basis()) == [0]
    H = sec.lower(ham)
    E = H.scipy().toarray()[0, 0].real
    o = O.Ham(O.Sector(vac), ham)
    assert o.scipy().toarray()[0, 0] == E  # bit for bit
    psi = q.getState(sec, 1)
    psi.set(0, np.array([1.0 + 0j]))
    assert psi.eval(0, H).real == E
    # the first Lanczos step already closes the space: the reference's act_dim would be 0
    with pytest.raises(A.QDError) as e:
        q.LanczosSolver(sec, 10).getGroundState(H, psi, 0)
    assert e.value.code == A.QD_ERR_BREAKDOWN


def test_two_state_sector_closes_after_one_step(ctx):
    """Two sites, one particle: dim 2.  With the start vector an eigenvector the space closes at the
    first step (the oracle fails the same way); otherwise it closes at the second, and expandBasis<1>
    returns step - 1 = 1, so the Ritz value is the start vector's Rayleigh quotient, as in the oracle."""
    spec, ham = chains.xy_chain(2)
    sec = sector(spec)
    assert sec.dim == 2
    H = sec.lower(ham)
    psi = q.getState(sec, 1)
    v0 = np.array([1.0, 1.0]) / np.sqrt(2.0)  # eigenvector of the hop (energy +1)
    psi.set(0, v0.astype(np.complex128))
    with pytest.raises(A.QDError) as e:
        q.LanczosSolver(sec, 5).getGroundState(H, psi, 0)
    assert e.value.code == A.QD_ERR_BREAKDOWN
    v1 = np.array([1.0, 0.3])
    psi.set(0, (v1 / np.linalg.norm(v1)).astype(np.complex128))
    r = q.LanczosSolver(sec, 5).getGroundState(H, psi, 0)
    o = O.Ham(O.Sector(spec), ham).lanczos_ground(v1 / np.linalg.norm(v1), 5)
    assert r.act_dim == o["act_dim"] == 1
    assert abs(r.ritz_value - 0.6 / 1.09) < 1e-15 and abs(o["ritz"] - r.ritz_value) < 1e-15


def test_argument_limits(ctx):
    spec, ham = chains.xy_chain(8)
    sec = sector(spec)
    H = sec.lower(ham)
    psi = q.getState(sec, 1)
    psi.set(0, q.start_vector(sec.dim, 1))
    import ctypes as C
    for kdim in (0, 4097):
        opts = A.qd_lanczos_opts(kdim, A.QD_SPMV_CSR, A.QD_RITZ_STORED_BASIS, 0)
        res = A.qd_lanczos_result()
        with pytest.raises(A.QDError) as e:
            A.call("qd_lanczos_ground", H.handle, psi.handle, 0, C.byref(opts), None, C.byref(res))
        assert e.value.code == A.QD_ERR_INVALID
    assert q.LanczosSolver(sec, 0).getGroundState(H, psi, 0) is None  # a full (empty) space returns at once
    with pytest.raises(A.QDError):
        psi.eval(1, H)  # time slot outside the state
    with pytest.raises(A.QDError):
        A.call("qd_ham_set_spmv_kernel", H.handle, 99)


def test_step_barrier_wait_runs_out_and_next_solve_is_unchanged(ctx, monkeypatch):
    """The one-launch Lanczos step's grid barrier is a bounded wait.  With the
    test control QD_STEP_WAIT_OUT the publishing block publishes no alpha and beta, so
    every block gives up after a few polls, skips its update and still joins the
    norm's reduction: the kernel returns and the solve reports QD_ERR_TIMEOUT.
    The next solve on the same operator carries the bits of one on a fresh
    operator."""
    spec, ham = chains.xxz_chain(16)  # uniform couplings: the one-launch step
    sec = sector(spec)
    v0 = q.start_vector(sec.dim, 5)

    def solve(H):
        psi = q.getState(sec, 1)
        psi.set(0, v0)
        r = q.Arnoldi.getLanczosSolver(sec, 40).getGroundState(H, psi(0), 0)
        return r, psi.get(0)

    H = sec.lower(ham)
    r0, p0 = solve(H)
    import ctypes as C
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, C.byref(info))
    assert info.step_launches == 1
    monkeypatch.setenv("QD_STEP_WAIT_OUT", "8")
    with pytest.raises(A.QDError) as e:
        solve(H)
    assert e.value.code == A.QD_ERR_TIMEOUT
    monkeypatch.delenv("QD_STEP_WAIT_OUT")
    r1, p1 = solve(H)
    r2, p2 = solve(sec.lower(ham))
    assert r1.ritz_value == r0.ritz_value == r2.ritz_value
    assert np.array_equal(p1, p0) and np.array_equal(p2, p0)


def test_step_mailbox_across_runs_and_forms(ctx, monkeypatch):
    """The one-launch step hands alpha and beta to every block through a
    mailbox whose set alternates with the launch parity.  Solves of different
    lengths and solves in the two-launch form, interleaved on one operator,
    each carry the bits of the same solve in the same form on a fresh
    operator."""
    spec, ham = chains.xxz_chain(14)
    sec = sector(spec)
    v0 = q.start_vector(sec.dim, 11)

    def solve(H, kdim, split):
        if split:
            monkeypatch.setenv("QD_LANCZOS_STEP", "split")
        else:
            monkeypatch.delenv("QD_LANCZOS_STEP", raising=False)
        psi = q.getState(sec, 1)
        psi.set(0, v0)
        r = q.Arnoldi.getLanczosSolver(sec, kdim).getGroundState(H, psi(0), 0)
        return r.ritz_value, psi.get(0)

    plan = ((17, False), (30, False), (17, True), (30, False), (17, False), (30, True), (17, False))
    fresh = {key: solve(sec.lower(ham), *key) for key in set(plan)}
    H = sec.lower(ham)
    for key in plan:
        e, p = solve(H, *key)
        assert e == fresh[key][0]
        assert np.array_equal(p, fresh[key][1])
    monkeypatch.delenv("QD_LANCZOS_STEP", raising=False)
