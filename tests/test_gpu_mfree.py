"""Matrix-free products (compiled operator tree, on-the-fly ranks) vs the CSR path and the oracle."""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains

from test_gpu_parity import SYSTEMS, gpu_objects

pytestmark = pytest.mark.gpu


def heff_hubbard(L, Nup, Ndo, U, gamma):
    spec, ham = chains.hubbard_chain(L, Nup, Ndo, U, -1.0, periodic=False)
    g = q.getHopFermiGate(spec.index)
    for s in range(2 * L):
        ham = ham + (-0.5j * gamma) * g(s, s)
    return spec, ham


CASES = dict(SYSTEMS)
CASES["heff_hubbard4"] = lambda: heff_hubbard(4, 2, 2, 4.0, 0.2)  # complex diagonal, not Hermitian
CASES["loose_xy10"] = lambda: (lambda s, h: (q.SectorSpec(s.index, s.constraints, tight=1), h))(*chains.xy_chain(10))


@pytest.mark.parametrize("name", sorted(CASES))
def test_matrix_free_product_matches_csr(ctx, name):
    spec, ham = CASES[name]()
    sec, H = gpu_objects(spec, ham)
    n = sec.dim
    Hs = H.scipy()
    rng = np.random.default_rng(11)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    xs = q.getState(sec, 1)
    ys = q.getState(sec, 1)
    xs.set(0, x)
    q.apply(H, xs, 0, ys, 0, matrix_free=True)
    y = ys.get(0)
    ref = Hs @ x
    scale = np.abs(Hs).sum(axis=1).max() * np.abs(x).max()
    assert np.max(np.abs(y - ref)) <= 1e-14 * scale * 8
    # the stored diagonal is the CSR diagonal, bit for bit
    d = Hs.diagonal()
    for i in sorted(set([0, n // 3, n // 2, n - 1])):
        e = np.zeros(n, dtype=np.complex128)
        e[i] = 1.0
        xs.set(0, e)
        q.apply(H, xs, 0, ys, 0, matrix_free=True)
        assert ys.get(0)[i] == d[i]
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, info)
    assert info.has_matrix_free == 1


def _mf_lanczos(spec, ham, kry, v0):
    sec, H = gpu_objects(spec, ham)
    psi = q.getState(sec, 1)
    psi.set(0, v0)
    solver = q.LanczosSolver(sec, kry, spmv=A.QD_SPMV_MATRIX_FREE)
    r = solver.getGroundState(H, psi, 0)
    return r, psi.get(0), H


def test_matrix_free_lanczos_xy16_matches_oracle(ctx):
    spec, ham = chains.xy_chain(16)
    n = 12870
    v0 = q.start_vector(n, 2024)
    r, psi, H = _mf_lanczos(spec, ham, 100, v0)
    oh = O.Ham(O.Sector(spec), ham)
    o = oh.lanczos_ground(v0, 100)
    assert r.act_dim == o["act_dim"]
    assert abs(r.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])
    e_gpu = np.vdot(psi, H.scipy() @ psi).real / np.vdot(psi, psi).real
    e_ref = o["energy"].real / np.vdot(o["psi"], o["psi"]).real
    assert abs(e_gpu - e_ref) <= 1e-10 * abs(e_ref)


def test_matrix_free_lanczos_xxz24_energy(ctx, golden):
    """Config-2 size: XXZ L=24 periodic, Sz=0 (dim 2,704,156), matrix-free FP64 Lanczos."""
    spec, ham = chains.xxz_chain(24, 1.0, 1.0, periodic=True)
    n = 2704156
    v0 = q.start_vector(n, 7)
    r, psi, H = _mf_lanczos(spec, ham, 100, v0)
    e0 = golden["heisenberg_periodic_e0"]["24"]["e0"]
    assert abs(r.ritz_value - e0) <= 1e-10 * abs(e0)
    # the same solve through the CSR product
    sec, Hc = gpu_objects(spec, ham)
    p2 = q.getState(sec, 1)
    p2.set(0, v0)
    rc = q.LanczosSolver(sec, 100).getGroundState(Hc, p2, 0)
    assert abs(r.ritz_value - rc.ritz_value) <= 1e-11 * abs(e0)
