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
