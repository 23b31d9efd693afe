"""The CPU oracle against independent known answers (tests/golden/golden.json)."""
import numpy as np
import pytest

import oracle as O
from qudrip_gb300 import chains
from qudrip_gb300.operators import (SectorSpec, getFermiGate, getQbits, getNset, getEmptyOperator,
                                    pauli_x, pauli_y, II)


def dense_from_oracle(spec, ham):
    sec = O.Sector(spec)
    H = O.Ham(sec, ham)
    return sec, H, H.scipy().toarray()


def dense_from_golden(rec):
    n = rec["dim"]
    M = np.zeros((n, n), dtype=complex)
    for r, c, re, im in rec["entries"]:
        M[r, c] = complex(re, im)
    return M


def fermi_bitgate_chain(L):
    pre = getQbits(L)
    spec = SectorSpec(pre, [getNset(pre) == L // 2])
    fc = getFermiGate(pre)
    fa = getFermiGate(pre)
    fc << 0.5 * (pauli_x + II * pauli_y)
    fa << 0.5 * (pauli_x - II * pauli_y)
    t = 0.7 + 0.2j
    ham = getEmptyOperator()
    for i in range(L - 1):
        ham = ham + t * (fc(i + 1) * fa(i)) + np.conj(t) * (fc(i) * fa(i + 1))
    return spec, ham


CASES = {
    "dense_xy_L6_open": lambda: chains.xy_chain(6),
    "dense_xxz_L6_periodic_fields": lambda: chains.xxz_chain(6, 1.0, 0.7, True, [0.3, -0.5, 1.1, 0.0, -0.2, 0.9]),
    "dense_hubbard_L3_periodic_2up1dn": lambda: chains.hubbard_chain(3, 2, 1, 4.0, -1.0, periodic=True),
    "dense_hubbard_L4_open_2up2dn": lambda: chains.hubbard_chain(4, 2, 2, 4.0, -1.0, periodic=False),
    "dense_fermi_bitgates_L6": lambda: fermi_bitgate_chain(6),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matrix_matches_independent_construction(golden, name):
    rec = golden[name]
    spec, ham = CASES[name]()
    sec, H, M = dense_from_oracle(spec, ham)
    assert [int(s) for s in sec.basis()] == rec["states"]
    ref = dense_from_golden(rec)
    assert np.array_equal(M, ref), np.abs(M - ref).max()


def test_oracle_xy_closed_form(golden):
    for L, e_exact in golden["xy_open_closed_form"].items():
        L = int(L)
        spec, ham = chains.xy_chain(L)
        sec = O.Sector(spec)
        H = O.Ham(sec, ham)
        v0 = np.random.default_rng(L).uniform(-1, 1, sec.dim)
        r = H.lanczos_ground(v0, min(100, sec.dim))
        assert abs(r["ritz"] - e_exact) <= 1e-10 * abs(e_exact)


def test_oracle_xy_L16_nnz(golden):
    spec, ham = chains.xy_chain(16)
    H = O.Ham(O.Sector(spec), ham)
    assert H.nnz == golden["xy_open_nnz"]["16"]


@pytest.mark.parametrize("L", [12, 14, 16])
def test_oracle_xxz_structure(golden, L):
    spec, ham = chains.xxz_chain(L)
    sec = O.Sector(spec)
    H = O.Ham(sec, ham)
    dim, nnz = golden["xxz_periodic_dim_nnz"][str(L)]
    assert (sec.dim, H.nnz) == (dim, nnz)
    colptr, rowidx, vals = H.csc()
    # rows strictly ascending inside every column (Eigen compressed storage)
    d = np.diff(rowidx.astype(np.int64))
    starts = colptr[1:-1]
    mask = np.ones(len(d), dtype=bool)
    mask[starts[starts < len(d) + 1] - 1] = False
    assert np.all(d[mask] > 0)


@pytest.mark.parametrize("L", [12, 16, 20])
def test_oracle_heisenberg_ground_energy(golden, L):
    spec, ham = chains.xxz_chain(L)
    sec = O.Sector(spec)
    H = O.Ham(sec, ham)
    v0 = np.random.default_rng(7).uniform(-1, 1, sec.dim)
    r = H.lanczos_ground(v0, 100)
    e0 = golden["heisenberg_periodic_e0"][str(L)]["e0"]
    assert abs(r["ritz"] - e0) <= 1e-10 * abs(e0)
    psi = r["psi"]
    rq = H.eval(psi).real / np.vdot(psi, psi).real
    assert abs(rq - e0) <= 1e-10 * abs(e0)


def test_oracle_hubbard_two_site(golden):
    spec, ham = chains.hubbard_chain(2, 1, 1, 4.0, -1.0, periodic=False)
    sec = O.Sector(spec)
    H = O.Ham(sec, ham)
    e = np.linalg.eigvalsh(H.scipy().toarray())[0]
    assert abs(e - golden["hubbard_2site_closed_form_U4"]) < 1e-12
    r = H.hermitian_lanczos_ground(np.ones(sec.dim), 3)
    assert abs(r["evals"][0] - e) < 1e-10


def test_oracle_tridiag_and_expm():
    import scipy.linalg as sl
    rng = np.random.default_rng(3)
    for n in (1, 2, 7, 40):
        d = rng.normal(size=n)
        e = rng.normal(size=max(n - 1, 0))
        ev, z = O.tridiag_eig(d, e)
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        assert np.allclose(ev, np.linalg.eigvalsh(T), atol=1e-12)
        assert np.allclose(T @ z, z * ev, atol=1e-10)
    for scale in (1e-3, 0.1, 1.0, 5.0, 40.0):
        A = (rng.normal(size=(12, 12)) + 1j * rng.normal(size=(12, 12))) * scale / 4
        E = O.expm(A)
        R = sl.expm(A)
        assert np.abs(E - R).max() <= 1e-11 * max(1.0, np.abs(R).max())


def test_oracle_arnoldi_evolve_matches_dense_propagator():
    import scipy.linalg as sl
    spec, ham = chains.hubbard_chain(3, 2, 1, 4.0, -1.0, periodic=True)
    sec = O.Sector(spec)
    H = O.Ham(sec, ham)
    Hd = H.scipy().toarray()
    psi = np.random.default_rng(5).normal(size=sec.dim) + 0j
    psi /= np.linalg.norm(psi)
    out, act = O.Ham.arnoldi_evolve(H, psi, 0.05, 6)
    ref = sl.expm(-1j * 0.05 * Hd) @ psi
    assert act == 5
    assert np.linalg.norm(out - ref) < 1e-8


def test_oracle_lanczos_breakdown_small_space():
    # dim 2 space: the recurrence stops at norm < 1e-10 (sparse_algorithm.hpp:421)
    spec, ham = chains.hubbard_chain(2, 1, 0, 0.0, -1.0)
    sec = O.Sector(spec)
    H = O.Ham(sec, ham)
    r = H.lanczos_ground(np.array([1.0, 0.3]), 10)
    assert r["breakdown"] == 1 and r["act_dim"] == 1


def test_trajectory_ensemble_fixture_consistent():
    """tests/golden/traj_ensemble_L8.json (the FP64 oracle ensemble the device ensemble is
    compared with): every trajectory starts in the ground state, so at t=0 the mean is that
    state's <n_{i,up} n_{i,dn}> with zero spread; later means are probabilities with small errors."""
    import json
    import os
    import scipy.sparse.linalg as sla
    import oracle as O
    from qudrip_gb300 import chains
    with open(os.path.join(os.path.dirname(__file__), "golden", "traj_ensemble_L8.json")) as f:
        g = json.load(f)
    L = g["L"]
    spec, ham = chains.hubbard_chain(L, g["Nup"], g["Ndo"], g["U"], g["thop"])
    osec = O.Sector(spec)
    H = O.Ham(osec, ham).scipy().tocsr()
    w, v = sla.eigsh(H.real, k=1, which="SA", tol=1e-13)
    assert abs(w[0] - g["ground_energy"]) < 1e-10
    p = np.abs(v[:, 0]) ** 2
    b = osec.basis()
    docc0 = [p[(b >> i) & (b >> (i + L)) & 1 == 1].sum() for i in range(L)]
    mean = np.array(g["mean"])
    err = np.array(g["stderr"])
    assert mean.shape == (g["nsteps"] // g["record_every"] + 1, L)
    assert np.abs(mean[0] - docc0).max() < 1e-9 and np.all(err[0] < 1e-9)
    assert np.all((mean >= 0) & (mean <= 1)) and np.all(err[1:] > 0) and np.all(err < 0.01)
    assert g["jumps"] > 0.5 * g["ntraj"] * g["gamma"] * (g["Nup"] + g["Ndo"]) * g["nsteps"] * g["dt"]
