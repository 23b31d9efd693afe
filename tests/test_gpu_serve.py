"""Request loop and the short-recurrence Krylov exponential vs the oracle.

The server's results are compared with the oracle's restatement of the
reference solvers, with each other across the plain and mixed forms, and --
the continuous-batching property -- between a request served alone and the
same request served in a mix of concurrent requests.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as sla

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains

pytestmark = pytest.mark.gpu

DE_TOL = 1e-8      # relative energy tolerance of the served forms
PSI_TOL = 1e-8     # 2-norm tolerance of evolved states


def xxz(L, seed, fields=True):
    rng = np.random.default_rng(seed)
    Jz = float(rng.uniform(0.0, 2.0))
    h = rng.uniform(-1.0, 1.0, size=L) if fields else None
    return chains.xxz_chain(L, 1.0, Jz, periodic=True, fields=h)


def oracle_ground(spec, ham, psi0, k):
    oh = O.Ham(O.Sector(spec), ham)
    r = oh.lanczos_ground(psi0, k)
    psi = r["psi"]
    n2 = np.vdot(psi, psi).real
    return r["ritz"], oh.eval(psi).real / n2


def oracle_evolve(spec, ham, psi0, dt, nsteps, m):
    oh = O.Ham(O.Sector(spec), ham)
    psi = np.asarray(psi0, dtype=np.complex128)
    for _ in range(nsteps):
        psi, _ = oh.arnoldi_evolve(psi, dt, m)
    return psi


# ------------------------------------------------------------------ Hermitian Krylov exponential
@pytest.mark.parametrize("complex_h", [False, True])
def test_lanczos_evolve_matches_arnoldi_and_expm(ctx, complex_h):
    L = 10
    spec, ham = xxz(L, 3)
    if complex_h:  # a Hermitian term with imaginary matrix elements
        gx = q.getBoseGate(spec.index)
        gx << q.pauli_x
        gy = q.getBoseGate(spec.index)
        gy << q.pauli_y
        ham = ham + 0.3 * (gx(1) * gy(4))  # imaginary exchange inside the Sz sector
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    assert H.is_hermitian
    assert H.is_real != complex_h
    n = sec.dim
    rng = np.random.default_rng(5)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    psi = q.getState(sec, 2)
    psi.set(0, x)
    dt, m, nsteps = 0.05, 16, 6
    for _ in range(nsteps):
        act = q.lanczos_evolve(H, psi, 0, 0, dt, m)
        assert act == m - 1
    got = psi.get(0)
    ref = oracle_evolve(spec, ham, x, dt, nsteps, m)
    assert np.linalg.norm(got - ref) < PSI_TOL
    assert abs(np.linalg.norm(got) - 1.0) < 1e-12
    # exact propagator on the normalised input
    Hs = H.scipy()
    ex = sla.expm_multiply(-1j * dt * nsteps * Hs, x / np.linalg.norm(x))
    assert np.linalg.norm(got - ex) < 1e-9
    # all steps in one call (one graph launch per step) give the same bits
    psi.set(1, x)
    act = q.lanczos_evolve(H, psi, 1, 1, dt, m, nsteps=nsteps)
    assert act == m - 1
    assert np.array_equal(psi.get(1), got)


def test_lanczos_evolve_breakdown_keeps_the_reference_count(ctx):
    # start vector in a 2-dimensional invariant subspace: breakdown at step 2
    L = 6
    spec, ham = chains.xxz_chain(L, 1.0, 1.0, periodic=True)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    Hs = H.scipy().toarray()
    w, v = np.linalg.eigh(Hs)
    x = (v[:, 0] + 0.5j * v[:, 3]).astype(np.complex128)
    psi = q.getState(sec, 1)
    psi.set(0, x)
    act = q.lanczos_evolve(H, psi, 0, 0, 0.3, 10)
    oh = O.Ham(O.Sector(spec), ham)
    ref, oact = oh.arnoldi_evolve(x, 0.3, 10)
    assert act == oact
    assert np.linalg.norm(psi.get(0) - ref) < PSI_TOL


def test_lanczos_evolve_rejects_non_hermitian(ctx):
    spec, ham = chains.hubbard_chain(3, 1, 1, 2.0, -1.0)
    g = q.getHopFermiGate(spec.index)
    ham = ham + (-0.05j) * g(0, 0)
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    psi = q.getState(sec, 1)
    psi.set(0, np.ones(sec.dim))
    with pytest.raises(A.QDError) as e:
        q.lanczos_evolve(H, psi, 0, 0, 0.1, 8)
    assert e.value.code == A.QD_ERR_NOT_HERMITIAN


# ------------------------------------------------------------------ request loop
def make_requests():
    """Ground states and evolutions on XXZ chains of several sizes (L = 8..14)."""
    reqs = []
    for i, L in enumerate([8, 10, 12, 14, 10, 12]):
        spec, ham = xxz(L, 100 + i, fields=(i % 2 == 0))
        reqs.append(dict(kind="ground", spec=spec, ham=ham, L=L, seed=1000 + i, k=80))
    for i, L in enumerate([8, 10, 12]):
        spec, ham = xxz(L, 200 + i)
        reqs.append(dict(kind="evolve", spec=spec, ham=ham, L=L, seed=2000 + i, dt=0.05, nsteps=8, m=16))
    return reqs


def dim_of(L):
    from math import comb
    return comb(L, L // 2)


def submit(srv, r, tag):
    n = dim_of(r["L"])
    if r["kind"] == "ground":
        return srv.submit_ground(r["spec"], r["ham"], krylov_dim=r["k"], seed=r["seed"], tag=tag)
    return srv.submit_evolve(r["spec"], r["ham"], r["dt"], r["nsteps"], m=r["m"], seed=r["seed"],
                             want_state=True, dim_hint=n, tag=tag)


def serve(mode, reqs, alone, **kw):
    srv = q.Server(mode=mode, **kw)
    out = {}
    try:
        if alone:
            for t, r in enumerate(reqs):
                rid = submit(srv, r, t)
                got = srv.wait_all([rid])
                out[t] = got[rid]
        else:
            ids = [submit(srv, r, t) for t, r in enumerate(reqs)]
            got = srv.wait_all(ids)
            for res in got.values():
                out[res["tag"]] = res
        stats = srv.stats()
    finally:
        srv.close()
    return out, stats


@pytest.fixture(scope="module")
def requests():
    return make_requests()


@pytest.fixture(scope="module")
def oracle_results(requests):
    res = {}
    for t, r in enumerate(requests):
        n = dim_of(r["L"])
        psi0 = q.seeded_start(r["seed"], n).astype(np.complex128)
        if r["kind"] == "ground":
            res[t] = oracle_ground(r["spec"], r["ham"], psi0, r["k"])
        else:
            res[t] = oracle_evolve(r["spec"], r["ham"], psi0, r["dt"], r["nsteps"], r["m"])
    return res


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_served_results_match_oracle(ctx, requests, oracle_results, mode):
    # batch_min=1: the batch lanes take every waiting small ground state, so batched results are checked
    out, stats = serve(mode, requests, alone=False, batch_min=1)
    assert stats["completed"] == len(requests) and stats["failed"] == 0
    for t, r in enumerate(requests):
        res = out[t]
        assert res["status"] == A.QD_OK
        if r["kind"] == "ground":
            ritz, energy = oracle_results[t]
            assert abs(res["energy"] - energy) <= DE_TOL * abs(energy), (t, res["energy"], energy)
            if res["path"] == A.QD_PATH_GRID:
                assert abs(res["ritz"] - ritz) <= 1e-10 * abs(ritz)
        else:
            ref = oracle_results[t]
            assert np.linalg.norm(res["state"] - ref) < PSI_TOL
            assert abs(res["norm"] - 1.0) < 1e-10
    if mode == "mixed":
        assert stats["batches"] >= 1 and stats["batched"] >= 1
    else:
        assert stats["batches"] == 0


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_each_result_same_alone_and_in_the_mix(ctx, requests, mode):
    mix, st_mix = serve(mode, requests, alone=False)
    alone, st_alone = serve(mode, requests, alone=True)
    assert st_alone["max_active"] == 1
    assert st_mix["max_active"] > 1, "requests did not overlap"
    for t, r in enumerate(requests):
        a, b = alone[t], mix[t]
        assert a["path"] == b["path"] or mode == "mixed"
        if a["path"] == b["path"]:
            assert a["energy"] == b["energy"], (t, a["energy"], b["energy"])
            if r["kind"] == "evolve":
                assert np.array_equal(a["state"], b["state"])
        else:  # a lone small ground state may take a grid lane when the batch lanes are busy
            assert abs(a["energy"] - b["energy"]) <= DE_TOL * abs(a["energy"])


def test_lone_small_ground_states_skip_the_batch(ctx, requests):
    """With the default batch_min (4), small ground states that arrive one at a time are served by
    the small lanes at once (no batch launch); the energies match the batched ones within DE_TOL."""
    alone, st = serve("mixed", requests, alone=True)
    assert st["batches"] == 0
    batched, st_b = serve("mixed", requests, alone=False, batch_min=1)
    assert st_b["batches"] >= 1
    for t, r in enumerate(requests):
        if r["kind"] == "ground":
            assert abs(alone[t]["energy"] - batched[t]["energy"]) <= DE_TOL * abs(alone[t]["energy"])


def test_admission_respects_the_byte_budget(ctx, requests):
    # a budget below two requests' footprint admits one request at a time
    out, stats = serve("plain", requests[:5], alone=False, hbm_budget=1)
    assert stats["max_active"] == 1
    assert stats["completed"] == 5 and stats["failed"] == 0
    out2, stats2 = serve("plain", requests[:5], alone=False)
    for t in range(5):
        assert out[t]["energy"] == out2[t]["energy"]
    assert stats2["bytes_peak"] >= max(r["bytes"] for r in out2.values())


def test_bad_request_fails_alone(ctx, requests):
    srv = q.Server(mode="mixed")
    try:
        r = requests[0]
        bad = srv.submit_ground(r["spec"], r["ham"], krylov_dim=20, psi0=np.ones(7), tag=1)
        good = srv.submit_ground(r["spec"], r["ham"], krylov_dim=20, seed=3, tag=2)
        got = srv.wait_all([bad, good])
    finally:
        srv.close()
    assert got[bad]["status"] == A.QD_ERR_INVALID
    assert got[good]["status"] == A.QD_OK
