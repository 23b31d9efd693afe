"""Uniform-coupling product with exact fixed-point sums (kernel code 120) vs the FP64 CSR path and the oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains

from test_gpu_parity import gpu_objects

pytestmark = pytest.mark.gpu


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
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, info)
    nnz_off = info.nnz - sec.dim  # every row of the periodic XXZ chain has a diagonal entry
    assert nb.value == nnz_off * 4 + (sec.dim + 1) * 4 + sec.dim * 40
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
