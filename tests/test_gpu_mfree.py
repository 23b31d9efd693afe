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
    """Full size: XXZ L=24 periodic, Sz=0 (dim 2,704,156), matrix-free Lanczos."""
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


def _lanczos(sec, H, v0, kry, spmv=A.QD_SPMV_CSR, kernel=None):
    if kernel is not None:
        A.call("qd_ham_set_spmv_kernel", H.handle, kernel)
    psi = q.getState(sec, 1)
    psi.set(0, v0)
    r = q.LanczosSolver(sec, kry, spmv=spmv).getGroundState(H, psi, 0)
    return r, psi.get(0)


def _mf_bytes(H):
    import ctypes as C
    ms, nb = C.c_double(), C.c_double()
    A.call("qd_ham_time_spmv", H.handle, A.QD_SPMV_MATRIX_FREE, 2, C.byref(ms), C.byref(nb))
    return nb.value


@pytest.mark.parametrize("case", ["xxz16", "xy14_open", "two_species"])
def test_matrix_free_uniform_form_bit_identical_to_csr(ctx, case):
    """Uniform couplings on the matrix-free path take the fixed-point form built from the terms alone (no
    stored matrix): the block layout of the sector (its tables checked on the device against the
    transitions' target states), else the slots (offsets checked on the host against whole-field ranks);
    its recurrence is bit-identical to the stored-matrix forms (codes 120 and 121), and so is the slot
    form's (QD_MF_BLOCK=0)."""
    from test_gpu_fx import two_species_xy
    spec, ham = {"xxz16": lambda: chains.xxz_chain(16, 1.0, 0.8, periodic=True,
                                                   fields=np.linspace(-1, 1, 16)),
                 "xy14_open": lambda: chains.xy_chain(14),
                 "two_species": lambda: two_species_xy(6, True)}[case]()
    sec, H = gpu_objects(spec, ham)
    v0 = q.start_vector(sec.dim, 31)
    r_mf, p_mf = _lanczos(sec, H, v0, 80, spmv=A.QD_SPMV_MATRIX_FREE)
    # the slot form as the recurrence runs it (the whole step in one launch: v_k and its fixed-point copy
    # written, w kept on chip), not the FP64 matrix-free product
    from test_gpu_fx import one_launch_extra
    assert _mf_bytes(H) == sec.dim * (4 + 8 + 8 + 16 + 8 + 8) + sec.dim * one_launch_extra()
    r_120, p_120 = _lanczos(sec, H, v0, 80, kernel=A.QD_SPMV_FX)
    r_121, p_121 = _lanczos(sec, H, v0, 80, kernel=A.QD_SPMV_FX_SLOTS)
    assert r_mf.ritz_value == r_120.ritz_value == r_121.ritz_value
    assert np.array_equal(p_mf, p_120) and np.array_equal(p_mf, p_121)
    import os
    os.environ["QD_MF_BLOCK"] = "0"
    try:
        sec2, H2 = gpu_objects(spec, ham)
        r_sl, p_sl = _lanczos(sec2, H2, v0, 80, spmv=A.QD_SPMV_MATRIX_FREE)
    finally:
        del os.environ["QD_MF_BLOCK"]
    assert r_sl.ritz_value == r_mf.ritz_value and np.array_equal(p_sl, p_mf)
    o = O.Ham(O.Sector(spec), ham).lanczos_ground(v0, 80)
    assert abs(r_mf.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])


def test_matrix_free_nonuniform_keeps_fp64_product(ctx):
    """Bond-dependent couplings: no single off-diagonal value, so the matrix-free path stays on the FP64
    product of the compiled transitions (8-byte basis words), and agrees with the CSR path."""
    L = 12
    pre = q.getQbits(L)
    gc, ga = q.getBoseGate(pre), q.getBoseGate(pre)
    gc << 0.5 * (q.pauli_x + q.II * q.pauli_y)
    ga << 0.5 * (q.pauli_x - q.II * q.pauli_y)
    J = np.random.default_rng(5).uniform(0.5, 1.5, L)
    ham = q.getEmptyOperator()
    for i in range(L):
        j = (i + 1) % L
        ham = ham + float(J[i]) * (gc(i) * ga(j)) + float(J[i]) * (gc(j) * ga(i))
    spec = q.SectorSpec(pre, [q.getNset(pre) == L // 2])
    sec, H = gpu_objects(spec, ham)
    v0 = q.start_vector(sec.dim, 8)
    r_mf, _ = _lanczos(sec, H, v0, 60, spmv=A.QD_SPMV_MATRIX_FREE)
    assert _mf_bytes(H) == sec.dim * (8 + 8 + 8 + 8)
    r_csr, _ = _lanczos(sec, H, v0, 60)
    assert abs(r_mf.ritz_value - r_csr.ritz_value) <= 1e-12 * abs(r_csr.ritz_value)
