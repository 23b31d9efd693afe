"""The allocation-free expectation value, checked against a host FP64 sum and psi.eval.

qd_csr_expect_noalloc exists for callers that may not allocate device memory
(an application that owns the device memory pool, or an allocation-free
request path).  The test plays such a caller: it owns every device buffer
(allocated here through torch) and passes their addresses in; the entry point
itself allocates nothing and keeps its reduction scratch in a fixed array of
the library's device image.  Each case makes two calls in a row with different
states; both must agree with psi^dagger (H psi) summed on the host in FP64 from
the same CSR arrays, and with the allocating path (psi.eval), showing that the
shared scratch carries nothing over.  The second case has thousands of blocks
(the periodic XXZ chain at L=24, 2,704,156 rows, 1,321 partial sums), so the
fixed partial-sum array is exercised far beyond one block.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ROWS = 4194304  # 2,048 blocks of 2,048 rows: the fixed scratch's limit


def complex_fermion_chain(L):
    from qudrip_gb300.operators import (II, SectorSpec, getEmptyOperator, getFermiGate, getNset, getQbits,
                                        pauli_x, pauli_y)
    pre = getQbits(L)
    spec = SectorSpec(pre, [getNset(pre) == L // 2])
    fc, fa = getFermiGate(pre), getFermiGate(pre)
    fc << 0.5 * (pauli_x + II * pauli_y)
    fa << 0.5 * (pauli_x - II * pauli_y)
    ham = getEmptyOperator()
    for i in range(L - 1):
        t = 0.8 + 0.3j * (i % 3 - 1)
        ham = ham + t * (fc(i + 1) * fa(i)) + np.conj(t) * (fc(i) * fa(i + 1))
    return spec, ham


def run_case(spec, ham, seed, check_eval):
    torch = pytest.importorskip("torch")
    import scipy.sparse as sp
    import qudrip_gb300 as q
    from qudrip_gb300 import _capi as A
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    n = sec.dim
    rowptr, colidx, vals = H.csr()
    M = sp.csr_matrix((vals, colidx, rowptr), shape=(n, n))
    dev = torch.device("cuda", 0)
    d_rowptr = torch.from_numpy(rowptr).to(dev)
    d_colidx = torch.from_numpy(colidx).to(dev)
    d_vals = torch.from_numpy(np.ascontiguousarray(vals).view(np.float64)).to(dev)
    d_out = torch.zeros(2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = q.getState(sec, 1) if check_eval else None
    rng = np.random.default_rng(seed)
    for call in range(2):
        psi = rng.normal(size=n) + 1j * rng.normal(size=n)
        terms = np.conj(psi) * (M @ psi)
        ref = terms.sum()  # host FP64 sum of psi^dagger H psi from the same arrays
        scale = np.abs(terms).sum()
        d_psi = torch.from_numpy(psi.view(np.float64)).to(dev)
        d_out.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        A.call("qd_csr_expect_noalloc", C.c_void_p(d_rowptr.data_ptr()), C.c_void_p(d_colidx.data_ptr()),
               C.c_void_p(d_vals.data_ptr()), n, C.c_void_p(d_psi.data_ptr()),
               C.c_void_p(d_out.data_ptr()), C.c_void_p(stream))
        torch.cuda.synchronize(dev)
        got = complex(*d_out.cpu().numpy())
        assert abs(got - ref) <= 1e-12 * scale, (call, got, ref)
        if check_eval:
            st.set(0, psi)
            e = st.eval(0, H)
            assert abs(got - e) <= 1e-12 * scale, (call, got, e)
    return d_rowptr, d_colidx, d_vals, d_psi, d_out, stream


def test_noalloc_expectation_complex_chain():
    spec, ham = complex_fermion_chain(14)
    from qudrip_gb300 import _capi as A
    d_rowptr, d_colidx, d_vals, d_psi, d_out, stream = run_case(spec, ham, 21, True)
    # sizes beyond the fixed scratch are refused before any device work
    with pytest.raises(A.QDError) as e:
        A.call("qd_csr_expect_noalloc", C.c_void_p(d_rowptr.data_ptr()), C.c_void_p(d_colidx.data_ptr()),
               C.c_void_p(d_vals.data_ptr()), MAX_ROWS + 1, C.c_void_p(d_psi.data_ptr()),
               C.c_void_p(d_out.data_ptr()), C.c_void_p(stream))
    assert e.value.code == A.QD_ERR_INVALID


def test_noalloc_expectation_many_blocks():
    from qudrip_gb300 import chains
    spec, ham = chains.xxz_chain(24, 1.0, 1.0, True)
    run_case(spec, ham, 5, False)
