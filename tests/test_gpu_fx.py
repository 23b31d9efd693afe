"""Uniform-coupling product with exact fixed-point sums (kernel code 120) vs the FP64 CSR path and the oracle."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains

from test_gpu_parity import gpu_objects

pytestmark = pytest.mark.gpu


def one_launch_extra():
    """Bytes per row the one-launch Lanczos step adds to the product's count (v_k 8 and its fixed-point
    copy 16 written, w 8 not); 0 when QD_LANCZOS_STEP=split keeps the step in two launches."""
    return 0 if os.environ.get("QD_LANCZOS_STEP") == "split" else 16


def solve(sec, H, v0, kry, kernel=None):
    if kernel is not None:
        A.call("qd_ham_set_spmv_kernel", H.handle, kernel)
    psi = q.getState(sec, 1)
    psi.set(0, v0)
    r = q.LanczosSolver(sec, kry).getGroundState(H, psi, 0)
    return r, psi.get(0)


@pytest.mark.parametrize("L,fields", [(16, None), (14, "random"), (12, "random")])
def test_fixed_point_lanczos_matches_csr_and_oracle(ctx, L, fields):
    h = np.random.default_rng(L).uniform(-1, 1, L) if fields else None
    spec, ham = chains.xxz_chain(L, 1.0, 0.7, periodic=True, fields=h)
    sec, H = gpu_objects(spec, ham)
    v0 = q.start_vector(sec.dim, 99)
    r_fx, psi_fx = solve(sec, H, v0, 100)                 # default: fixed-point form
    r_csr, psi_csr = solve(sec, H, v0, 100, kernel=110)   # FP64 CSR
    o = O.Ham(O.Sector(spec), ham).lanczos_ground(v0, 100)
    assert r_fx.act_dim == r_csr.act_dim == o["act_dim"]
    assert abs(r_fx.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])
    assert abs(r_fx.ritz_value - r_csr.ritz_value) <= 1e-12 * abs(o["ritz"])
    Hs = H.scipy()
    e_fx = np.vdot(psi_fx, Hs @ psi_fx).real / np.vdot(psi_fx, psi_fx).real
    e_ref = o["energy"].real / np.vdot(o["psi"], o["psi"]).real
    assert abs(e_fx - e_ref) <= 1e-10 * abs(e_ref)


def test_fixed_point_product_timing_and_applicability(ctx):
    spec, ham = chains.xxz_chain(16, 1.0, 1.0, periodic=True)
    sec, H = gpu_objects(spec, ham)
    ms, nb = C.c_double(), C.c_double()
    A.call("qd_ham_time_spmv", H.handle, 120, 5, C.byref(ms), C.byref(nb))
    assert ms.value > 0
    # columns in 32-row slices, each slice as wide as its longest row rounded up to 4
    ptr, col, val = H.csr()
    rows = np.repeat(np.arange(sec.dim), np.diff(ptr))
    off = np.bincount(rows[(col != rows) & (val != 0)], minlength=sec.dim)
    pad = np.concatenate([off, np.zeros(-sec.dim % 32, dtype=off.dtype)]).reshape(-1, 32).max(axis=1)
    cols = int(((pad + 3) // 4 * 128).sum())
    assert nb.value == cols * 4 + ((sec.dim + 31) // 32 + 1) * 8 + sec.dim + sec.dim * 40
    # Hubbard hopping carries both signs (Jordan-Wigner): the form does not apply
    spec2, ham2 = chains.hubbard_chain(4, 2, 2, 4.0, -1.0, periodic=True)
    sec2, H2 = gpu_objects(spec2, ham2)
    with pytest.raises(A.QDError) as e:
        A.call("qd_ham_time_spmv", H2.handle, 120, 2, C.byref(ms), C.byref(nb))
    assert e.value.code == A.QD_ERR_UNSUPPORTED
    # ... and its Lanczos solve takes the CSR product without complaint
    v0 = q.start_vector(sec2.dim, 5)
    r, _ = solve(sec2, H2, v0, 60)
    o = O.Ham(O.Sector(spec2), ham2).lanczos_ground(v0, 60)
    assert abs(r.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])


def product_kernel(H):
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, info)
    return info.product_kernel


def two_species_xy(L, periodic):
    """Hard-core bosons of two species on bits 0..L-1 and L..2L-1 (two popcount fields), uniform hopping."""
    from qudrip_gb300.operators import (II, SectorSpec, getBoseGate, getEmptyOperator, getNdo, getNup, getQbits,
                                        pauli_x, pauli_y, pauli_z)
    pre = getQbits(2 * L)
    spec = SectorSpec(pre, [getNup(pre, L) == L // 2, getNdo(pre, L) == L // 2 - 1])
    gc, ga, gz = getBoseGate(pre), getBoseGate(pre), getBoseGate(pre)
    gc << 0.5 * (pauli_x + II * pauli_y)
    ga << 0.5 * (pauli_x - II * pauli_y)
    gz << 0.5 * pauli_z
    ham = getEmptyOperator()
    for sp in (0, L):
        for i in range(L if periodic else L - 1):
            a, b = sp + i, sp + (i + 1) % L
            ham = ham + 0.75 * (gc(a) * ga(b)) + 0.75 * (gc(b) * ga(a))
    for i in range(L):
        ham = ham + 1.3 * (gz(i) * gz(i + L))
    return spec, ham


CASES = {
    "xxz16_periodic": lambda: chains.xxz_chain(16, 1.0, 0.7, periodic=True),
    "xxz14_open_fields": lambda: chains.xxz_chain(14, 1.0, 1.0, periodic=False,
                                                  fields=np.random.default_rng(3).uniform(-1, 1, 14)),
    "xy12_open": lambda: chains.xy_chain(12),
    "two_species_periodic": lambda: two_species_xy(6, True),
    "two_species_open": lambda: two_species_xy(7, False),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_columns_on_the_fly_bit_identical_to_stored_columns(ctx, name):
    """Code 121 computes each row's columns from the compiled terms (a table over the set bits below a
    contiguous support, byte-table ranks for the periodic bond); the build checks them against the stored
    columns, and the recurrence launches the same grid and reduction, so the solve is bit-identical."""
    spec, ham = CASES[name]()
    sec, H = gpu_objects(spec, ham)
    assert product_kernel(H) == A.QD_SPMV_FX  # stored columns by default
    v0 = q.start_vector(sec.dim, 17)
    r121, psi121 = solve(sec, H, v0, 60, kernel=A.QD_SPMV_FX_SLOTS)
    r120, psi120 = solve(sec, H, v0, 60, kernel=A.QD_SPMV_FX)
    assert product_kernel(H) == A.QD_SPMV_FX
    assert r121.ritz_value == r120.ritz_value and r121.act_dim == r120.act_dim
    assert np.array_equal(psi121, psi120)
    o = O.Ham(O.Sector(spec), ham).lanczos_ground(v0, 60)
    assert abs(r121.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])


def test_columns_on_the_fly_timing_and_fallback(ctx):
    spec, ham = chains.xxz_chain(16, 1.0, 1.0, periodic=True)
    sec, H = gpu_objects(spec, ham)
    ms, nb = C.c_double(), C.c_double()
    A.call("qd_ham_time_spmv", H.handle, A.QD_SPMV_FX_SLOTS, 5, C.byref(ms), C.byref(nb))
    assert ms.value > 0 and nb.value == sec.dim * (4 + 8 + 8 + 16 + 8)
    A.call("qd_ham_set_spmv_kernel", H.handle, A.QD_SPMV_FX_SLOTS)
    A.call("qd_ham_time_spmv", H.handle, A.QD_SPMV_CSR, 5, C.byref(ms), C.byref(nb))  # what Lanczos launches
    # the whole Lanczos step in one launch: w stays on chip, v_k (8) and its fixed-point copy (16) are written
    assert nb.value == sec.dim * (4 + 8 + 8 + 16 + 8 + 8) + sec.dim * one_launch_extra()
    # a term on 7 sites is beyond the compiled form: the stored columns stay, 121 is refused, 120 runs
    from qudrip_gb300.operators import II, SectorSpec, getBoseGate, getEmptyOperator, getNset, getQbits
    pre = getQbits(12)
    gc, ga, gn = getBoseGate(pre), getBoseGate(pre), getBoseGate(pre)
    gc << 0.5 * (q.pauli_x + II * q.pauli_y)
    ga << 0.5 * (q.pauli_x - II * q.pauli_y)
    gn << np.array([[0, 0], [0, 1]], dtype=complex)
    ham2 = getEmptyOperator()
    for i in range(11):
        ham2 = ham2 + gc(i) * ga(i + 1) + gc(i + 1) * ga(i)
    ham2 = ham2 + gc(0) * ga(2) * gn(3) * gn(4) * gn(5) * gn(6) * gn(7)
    ham2 = ham2 + gc(2) * ga(0) * gn(3) * gn(4) * gn(5) * gn(6) * gn(7)
    sec2, H2 = gpu_objects(SectorSpec(pre, [getNset(pre) == 6]), ham2)
    assert product_kernel(H2) == A.QD_SPMV_FX
    if True:
        with pytest.raises(A.QDError) as e:
            A.call("qd_ham_set_spmv_kernel", H2.handle, A.QD_SPMV_FX_SLOTS)
        assert e.value.code == A.QD_ERR_UNSUPPORTED


@pytest.mark.parametrize("name", sorted(CASES))
def test_block_layout_step_matches_stored_columns(ctx, name, monkeypatch):
    """Code 122: the block layout of the sector (rows grouped by the high part of their state; tables of
    the low and high parts' targets, checked against the stored columns at build).  Its one-launch step
    runs on code 120's grid, row order and reduction tree, so the solve is bit-identical; the staged
    variant (QD_FX_BLOCK_STAGED=1: each group of whole blocks copied into shared memory by one bulk
    copy) adds the inner products in another order and agrees to rounding."""
    spec, ham = CASES[name]()
    v0 = q.start_vector(q.Sector(spec.index, spec.constraints).dim, 17)
    sec, H = gpu_objects(spec, ham)
    r120, psi120 = solve(sec, H, v0, 60, kernel=A.QD_SPMV_FX)
    r122, psi122 = solve(sec, H, v0, 60, kernel=A.QD_SPMV_FX_BLOCK)
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, C.byref(info))
    assert info.product_kernel == A.QD_SPMV_FX_BLOCK and info.step_launches == 1
    assert r122.ritz_value == r120.ritz_value and np.array_equal(psi122, psi120)
    monkeypatch.setenv("QD_FX_BLOCK_STAGED", "1")
    sec2, H2 = gpu_objects(spec, ham)
    r_st, psi_st = solve(sec2, H2, v0, 60, kernel=A.QD_SPMV_FX_BLOCK)
    A.call("qd_ham_get_info", H2.handle, C.byref(info))
    assert info.step_launches == 1
    assert r_st.act_dim == r120.act_dim and r_st.matvecs == r120.matvecs
    assert abs(r_st.ritz_value - r120.ritz_value) <= 1e-12 * abs(r120.ritz_value)
    ov = abs(np.vdot(psi_st, psi120)) / (np.linalg.norm(psi_st) * np.linalg.norm(psi120))
    assert ov >= 1 - 1e-10
    o = O.Ham(O.Sector(spec), ham).lanczos_ground(v0, 60)
    assert abs(r_st.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])


def test_block_layout_two_launch_step_bit_identical(ctx, monkeypatch):
    monkeypatch.setenv("QD_LANCZOS_STEP", "split")
    spec, ham = chains.xxz_chain(16, 1.0, 0.7, periodic=True)
    sec, H = gpu_objects(spec, ham)
    v0 = q.start_vector(sec.dim, 3)
    r120, psi120 = solve(sec, H, v0, 60, kernel=A.QD_SPMV_FX)
    r122, psi122 = solve(sec, H, v0, 60, kernel=A.QD_SPMV_FX_BLOCK)
    assert r122.ritz_value == r120.ritz_value and np.array_equal(psi122, psi120)


@pytest.mark.parametrize("L,fields,kernel", [(16, None, None), (14, "random", None), (14, None, 121)])
def test_one_launch_step_matches_two_launch_step(ctx, monkeypatch, L, fields, kernel):
    """The default Lanczos step of the uniform-coupling form is one cooperative launch (product, dots,
    update, norm); QD_LANCZOS_STEP=split runs the product with its dots and the update as two launches.
    alpha, beta and v_k carry the same bits; only the norm's reduction order differs."""
    h = np.random.default_rng(L).uniform(-1, 1, L) if fields else None
    spec, ham = chains.xxz_chain(L, 1.0, 0.7, periodic=True, fields=h)
    v0 = q.start_vector(q.Sector(spec.index, spec.constraints).dim, 5)
    sec, H = gpu_objects(spec, ham)
    r1, psi1 = solve(sec, H, v0, 80, kernel=kernel)
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, C.byref(info))
    assert info.step_launches == 1
    monkeypatch.setenv("QD_LANCZOS_STEP", "split")
    sec2, H2 = gpu_objects(spec, ham)
    r2, psi2 = solve(sec2, H2, v0, 80, kernel=kernel)
    A.call("qd_ham_get_info", H2.handle, C.byref(info))
    assert info.step_launches == 2
    assert r1.act_dim == r2.act_dim and r1.matvecs == r2.matvecs
    assert abs(r1.ritz_value - r2.ritz_value) <= 1e-13 * abs(r2.ritz_value)
    ov = abs(np.vdot(psi1, psi2)) / (np.linalg.norm(psi1) * np.linalg.norm(psi2))
    assert ov >= 1 - 1e-10
    o = O.Ham(O.Sector(spec), ham).lanczos_ground(v0, 80)
    assert abs(r1.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])


def test_large_sector_takes_the_two_launch_step(ctx):
    """XXZ L=26 (dim 10,400,600): the one-launch step would keep 45 rows of w per thread in shared
    memory (90 KB per block), room for two of its 912 blocks per SM, so it cannot be resident at once
    and the recurrence runs the product and the update as two launches; the result agrees with the
    FP64 CSR product."""
    spec, ham = chains.xxz_chain(26, 1.0, 1.0, periodic=True)
    sec, H = gpu_objects(spec, ham)
    assert sec.dim == 10400600
    v0 = q.start_vector(sec.dim, 3)
    r_fx, psi_fx = solve(sec, H, v0, 30)
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, C.byref(info))
    assert info.product_kernel == A.QD_SPMV_FX and info.step_launches == 2
    r_blk, psi_blk = solve(sec, H, v0, 30, kernel=A.QD_SPMV_FX_BLOCK)  # the block form's two-launch step
    assert r_blk.ritz_value == r_fx.ritz_value and np.array_equal(psi_blk, psi_fx)
    r_csr, psi_csr = solve(sec, H, v0, 30, kernel=110)
    assert r_fx.act_dim == r_csr.act_dim == 30
    assert abs(r_fx.ritz_value - r_csr.ritz_value) <= 1e-12 * abs(r_csr.ritz_value)
    ov = abs(np.vdot(psi_fx, psi_csr)) / (np.linalg.norm(psi_fx) * np.linalg.norm(psi_csr))
    assert ov >= 1 - 1e-10


@pytest.mark.parametrize("L,fields", [(16, None), (14, "random")])
def test_real_state_expectation_on_the_uniform_form(ctx, L, fields):
    """psi.eval of a real state on an operator whose uniform-coupling form a solve has built reads the
    sliced columns (fx_eval_real_kernel): within 1e-13 of the complex CSR product and of a host FP64 sum.
    A state with an imaginary part takes the complex CSR product, whose bits the forced CSR path gives."""
    h = np.random.default_rng(L).uniform(-1, 1, L) if fields else None
    spec, ham = chains.xxz_chain(L, 1.0, 0.7, periodic=True, fields=h)
    sec, H = gpu_objects(spec, ham)
    v0 = q.start_vector(sec.dim, 21)
    r, psi = solve(sec, H, v0, 60)  # builds the uniform-coupling form
    rng = np.random.default_rng(L + 1)
    real = rng.uniform(-1, 1, sec.dim).astype(np.complex128)
    cplx = real + 1j * rng.uniform(-1, 1, sec.dim)
    one = real.copy()
    one[sec.dim // 3] += 0.25j  # a single entry with an imaginary part still takes the complex product
    Hs = H.scipy()
    st = q.getState(sec, 2)
    got = {}
    for name, x in (("ground", psi), ("real", real), ("cplx", cplx), ("one", one)):
        st.set(0, x)
        got[name] = st.eval(0, H)
        ref = np.vdot(x, Hs @ x)
        scale = np.abs(np.conj(x) * (Hs @ x)).sum()
        assert abs(got[name] - ref) <= 1e-13 * scale, (name, got[name], ref)
        if name in ("ground", "real"):
            assert got[name].imag == 0.0
    A.call("qd_ham_set_spmv_kernel", H.handle, 110)  # the FP64 CSR path for every product, eval included
    for name, x in (("ground", psi), ("real", real), ("cplx", cplx), ("one", one)):
        st.set(0, x)
        e_csr = st.eval(0, H)
        scale = np.abs(np.conj(x) * (Hs @ x)).sum()
        assert abs(got[name] - e_csr) <= 1e-13 * scale, (name, got[name], e_csr)
        if name in ("cplx", "one"):
            assert got[name] == e_csr  # a state with an imaginary part took the CSR product in both
