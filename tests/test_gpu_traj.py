"""Batched Krylov steps and quantum-jump ensembles vs the oracle."""
import ctypes as C

import numpy as np
import pytest
import scipy.linalg as sl

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains
from qudrip_gb300.operators import getHopFermiGate

pytestmark = pytest.mark.gpu


def heff_hubbard(L, Nup, Ndo, U, gamma, periodic=False):
    spec, ham = chains.hubbard_chain(L, Nup, Ndo, U, -1.0, periodic=periodic)
    gate = getHopFermiGate(spec.index)
    for s in range(2 * L):
        ham = ham + (-0.5j * gamma) * gate(s, s)
    return spec, ham


def test_krylov_batch_matches_single_and_dense(ctx):
    spec, ham = heff_hubbard(3, 2, 1, 4.0, 0.3, periodic=True)
    oh = O.Ham(O.Sector(spec), ham)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    n = sec.dim
    rng = np.random.default_rng(1)
    X = rng.normal(size=(5, n)) + 1j * rng.normal(size=(5, n))
    sx = q.getState(sec, 5)
    sy = q.getState(sec, 5)
    for b in range(5):
        sx.set(b, X[b])
    ld = (sx.device_ptr(1) - sx.device_ptr(0)) // 16
    acts = (C.c_int * 5)()
    A.call("qd_krylov_evolve_batch", H.handle, C.c_void_p(sx.device_ptr(0)), ld, 5, 0.07, 12,
           C.c_void_p(sy.device_ptr(0)), ld, acts)
    for b in range(5):
        ref, act = oh.arnoldi_evolve(X[b], 0.07, 12)
        assert acts[b] == act
        assert np.linalg.norm(sy.get(b) - ref) < 1e-10
    # unit vectors: the columns of exp(-i H h)
    su = q.getState(sec, n)
    ldu = (su.device_ptr(1) - su.device_ptr(0)) // 16
    A.call("qd_krylov_evolve_batch", H.handle, None, 0, n, 0.05, 30, C.c_void_p(su.device_ptr(0)), ldu, None)
    Uref = sl.expm(-1j * 0.05 * oh.scipy().toarray())
    for b in range(n):
        col = Uref[:, b] / np.linalg.norm(np.eye(n)[:, b])
        assert np.linalg.norm(su.get(b) - col) < 1e-10


def test_trajectories_match_oracle(ctx):
    L = 4
    gamma, dt, nsteps, ntraj, m, seed = 0.5, 0.05, 40, 64, 12, 777
    spec, heff = heff_hubbard(L, 2, 2, 4.0, gamma)
    oh = O.Ham(O.Sector(spec), heff)
    osec = O.Sector(spec)
    basis = osec.basis()
    # start from the ground state of the Hermitian part
    spec_h, ham = chains.hubbard_chain(L, 2, 2, 4.0, -1.0)
    Hd = O.Ham(O.Sector(spec_h), ham).scipy().toarray()
    psi0 = np.linalg.eigh(Hd)[1][:, 0].astype(complex)
    chan = list(range(2 * L))
    obs = [(i, i + L) for i in range(L)]
    ref, ref_jumps = O.traj_run(oh, basis, ntraj, nsteps, dt, gamma, seed, m, chan, obs, psi0)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(heff)
    mean, err, st = q.traj_run(H, psi0, ntraj, nsteps, dt, gamma, seed, m, chan, obs)
    assert st.jumps == ref_jumps
    assert np.abs(mean - ref).max() < 2e-5
    assert np.all(err >= 0)


def replay_case(L, Nup, Ndo, gamma, dt, nsteps, ntraj, m, seed, amps=None):
    """A Hubbard chain (optionally with per-bond hopping amplitudes) and its
    trajectories on the device and in the oracle, with the same Philox decisions."""
    from qudrip_gb300.operators import getEmptyOperator
    if amps is None:
        spec, heff = heff_hubbard(L, Nup, Ndo, 4.0, gamma)
        spec_h, ham = chains.hubbard_chain(L, Nup, Ndo, 4.0, -1.0)
    else:
        spec, ham0 = chains.hubbard_chain(L, Nup, Ndo, 4.0, -1.0)
        gate = getHopFermiGate(spec.index)
        ham = getEmptyOperator()
        for i in range(L - 1):
            for o in (0, L):
                ham = ham + amps[i] * gate(i + 1 + o, i + o) + amps[i] * gate(i + o, i + 1 + o)
        for i in range(L):
            ham = ham + 4.0 * (gate(i, i) * gate(i + L, i + L))
        heff = ham
        for s in range(2 * L):
            heff = heff + (-0.5j * gamma) * gate(s, s)
        spec_h = spec
    Hd = O.Ham(O.Sector(spec_h), ham).scipy()
    import scipy.sparse.linalg as sla
    if Hd.shape[0] > 400:
        psi0 = sla.eigsh(Hd.tocsr().real, k=1, which="SA", tol=1e-12)[1][:, 0].astype(complex)
    else:
        psi0 = np.linalg.eigh(Hd.toarray())[1][:, 0].astype(complex)
    osec = O.Sector(spec)
    oh = O.Ham(osec, heff)
    chan = list(range(2 * L))
    obs = [(i, i + L) for i in range(L)]
    ref, ref_jumps = O.traj_run(oh, osec.basis(), ntraj, nsteps, dt, gamma, seed, m, chan, obs, psi0)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(heff)
    mean, err, st = q.traj_run(H, psi0, ntraj, nsteps, dt, gamma, seed, m, chan, obs)
    return ref, ref_jumps, mean, err, st


def test_arnoldi_form_matches_oracle(ctx, monkeypatch):
    """QD_TRAJ_ARNOLDI=1: every step an FP64 Arnoldi exponential per trajectory (kbatch) and the
    decision kernel on complex128 states -- the same decisions and observables as the oracle."""
    monkeypatch.setenv("QD_TRAJ_ARNOLDI", "1")
    ref, ref_jumps, mean, err, st = replay_case(4, 2, 2, 0.5, 0.05, 40, 64, 12, 777)
    assert st.path == 1
    assert st.jumps == ref_jumps
    assert np.abs(mean - ref).max() < 1e-6  # observables are recorded in FP32


def test_resident_form_and_fallback_choice(ctx):
    ref, ref_jumps, mean, err, st = replay_case(4, 2, 2, 0.5, 0.05, 40, 64, 12, 777)
    assert st.path == 0  # one off-diagonal value (-t): the resident Taylor kernel
    assert st.jumps == ref_jumps
    assert np.abs(mean - ref).max() < 2e-5
    # per-bond amplitudes: off-diagonal values other than +-c take the Arnoldi form
    amps = [-1.0, -0.8, -1.2]
    ref, ref_jumps, mean, err, st = replay_case(4, 2, 2, 0.5, 0.05, 40, 64, 12, 99, amps=amps)
    assert st.path == 1
    assert st.jumps == ref_jumps
    assert np.abs(mean - ref).max() < 1e-6


def test_resident_replay_at_the_workload_size(ctx):
    """The trajectory workload's system (L=8, dim 4,900, gamma=0.1, dt=0.01, m=30): 16 trajectories
    x 100 steps replayed by the oracle, the same jumps and observables within complex64 rounding."""
    ref, ref_jumps, mean, err, st = replay_case(8, 4, 4, 0.1, 0.01, 100, 16, 30, 4242)
    assert st.path == 0
    assert st.jumps == ref_jumps
    assert np.abs(mean - ref).max() < 2e-5


def test_ensemble_matches_fp64_oracle_ensemble(ctx):
    """4,096 device trajectories to T=10 against 1,024 FP64 oracle trajectories with other seeds
    (tests/golden/traj_ensemble_L8.json, made by tests/golden/make_traj_ensemble.py):
    <n_{i,up} n_{i,dn}>(t) agrees within 4.5 combined standard errors at every recorded time
    (808 comparisons), the mean |z| stays near its N(0,1) value 0.80, and t=0 is the same state."""
    import json
    import os
    import scipy.sparse.linalg as sla
    with open(os.path.join(os.path.dirname(__file__), "golden", "traj_ensemble_L8.json")) as f:
        g = json.load(f)
    L = g["L"]
    spec, heff = heff_hubbard(L, g["Nup"], g["Ndo"], g["U"], g["gamma"])
    spec_h, ham = chains.hubbard_chain(L, g["Nup"], g["Ndo"], g["U"], g["thop"])
    sec = q.Sector(spec.index, spec.constraints)
    Hh = sec.lower(ham)
    rp, ci, vals = Hh.csr()
    import scipy.sparse as sp
    w, v = sla.eigsh(sp.csr_matrix((vals.real, ci, rp), shape=(sec.dim, sec.dim)), k=1, which="SA", tol=1e-13)
    assert abs(w[0] - g["ground_energy"]) < 1e-10
    psi0 = v[:, 0].astype(complex)
    H = sec.lower(heff)
    mean, err, st = q.traj_run(H, psi0, 4096, g["nsteps"], g["dt"], g["gamma"], 4242, g["m"], g["channels"],
                               [tuple(o) for o in g["observables"]])
    assert st.path == 0
    rows = g["steps"]
    om = np.array(g["mean"])
    oe = np.array(g["stderr"])
    gm = mean[rows]
    ge = err[rows]
    assert np.abs(gm[0] - om[0]).max() < 1e-6
    z = (gm[1:] - om[1:]) / np.sqrt(ge[1:] ** 2 + oe[1:] ** 2)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert np.abs(z).mean() < 1.25, np.abs(z).mean()


def test_resident_propagation_matches_exact_exponential(ctx):
    """gamma = 0 (no jump ever fires): the resident kernel's truncated Taylor steps against the
    exact exp(-i H t) of a dense H applied to a random start state, observables <n_up n_dn>(t)
    over 100 steps of dt = 0.01 at the workload's L = 8 Hubbard chain (dim 4,900).  The series is
    truncated where its remainder bound falls below a sixth of the complex64 state's rounding per
    step; the observables must stay within the FP32 record's accumulated rounding."""
    import scipy.sparse.linalg as sla
    L, dt, nsteps = 8, 0.01, 100
    spec, heff = heff_hubbard(L, 4, 4, 4.0, 0.0)
    osec = O.Sector(spec)
    Hs = O.Ham(osec, heff).scipy().tocsr()
    rng = np.random.default_rng(3)
    psi0 = rng.normal(size=osec.dim) + 1j * rng.normal(size=osec.dim)
    psi0 /= np.linalg.norm(psi0)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(heff)
    obs = [(i, i + L) for i in range(L)]
    mean, err, st = q.traj_run(H, psi0, 2, nsteps, dt, 0.0, 11, 30, list(range(2 * L)), obs)
    assert st.path == 0 and st.jumps == 0
    basis = osec.basis()
    nn = np.array([[((int(b) >> a) & 1) * ((int(b) >> c) & 1) for (a, c) in obs] for b in basis], dtype=float)
    psi = psi0.copy()
    worst = 0.0
    for t in range(nsteps + 1):
        ref = (np.abs(psi) ** 2) @ nn
        worst = max(worst, np.abs(mean[t] - ref).max())
        psi = sla.expm_multiply(-1j * dt * Hs, psi)
    assert worst < 1e-5, worst
