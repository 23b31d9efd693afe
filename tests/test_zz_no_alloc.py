"""The allocation-free expectation value, checked against psi.eval.

qd_csr_expect_noalloc exists for callers that may not allocate device memory
(an application that owns the device memory pool, or an allocation-free
request path).  The test plays such a caller: it owns every device buffer
(allocated here through torch) and passes their addresses in; the entry point
itself allocates nothing and keeps its reduction scratch in a fixed array of
the library's device image.  Two calls in a row must both agree with the
allocating path, showing that the shared scratch carries nothing over.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_expectation_matches_state_eval():
    torch = pytest.importorskip("torch")
    import qudrip_gb300 as q
    from qudrip_gb300 import _capi as A
    from qudrip_gb300.operators import (II, SectorSpec, getEmptyOperator, getFermiGate, getNset, getQbits,
                                        pauli_x, pauli_y)

    # a complex Hermitian operator (fermionic hopping with a complex amplitude)
    L = 14
    pre = getQbits(L)
    spec = SectorSpec(pre, [getNset(pre) == L // 2])
    fc, fa = getFermiGate(pre), getFermiGate(pre)
    fc << 0.5 * (pauli_x + II * pauli_y)
    fa << 0.5 * (pauli_x - II * pauli_y)
    ham = getEmptyOperator()
    for i in range(L - 1):
        t = 0.8 + 0.3j * (i % 3 - 1)
        ham = ham + t * (fc(i + 1) * fa(i)) + np.conj(t) * (fc(i) * fa(i + 1))
    sec = q.Sector(spec.index, spec.constraints)
    H = sec.lower(ham)
    rowptr, colidx, vals = H.csr()
    dev = torch.device("cuda", 0)
    d_rowptr = torch.from_numpy(rowptr).to(dev)
    d_colidx = torch.from_numpy(colidx).to(dev)
    d_vals = torch.from_numpy(np.ascontiguousarray(vals).view(np.float64)).to(dev)
    d_out = torch.zeros(2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = q.getState(sec, 1)
    rng = np.random.default_rng(21)
    for call in range(2):
        psi = rng.normal(size=sec.dim) + 1j * rng.normal(size=sec.dim)
        st.set(0, psi)
        ref = st.eval(0, H)
        d_psi = torch.from_numpy(psi.view(np.float64)).to(dev)
        d_out.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        A.call("qd_csr_expect_noalloc", C.c_void_p(d_rowptr.data_ptr()), C.c_void_p(d_colidx.data_ptr()),
               C.c_void_p(d_vals.data_ptr()), sec.dim, C.c_void_p(d_psi.data_ptr()),
               C.c_void_p(d_out.data_ptr()), C.c_void_p(stream))
        torch.cuda.synchronize(dev)
        got = complex(*d_out.cpu().numpy())
        assert abs(got - ref) <= 1e-12 * abs(ref), (call, got, ref)
    # sizes beyond the fixed scratch are refused before any device work
    with pytest.raises(A.QDError) as e:
        A.call("qd_csr_expect_noalloc", C.c_void_p(d_rowptr.data_ptr()), C.c_void_p(d_colidx.data_ptr()),
               C.c_void_p(d_vals.data_ptr()), 4194305, C.c_void_p(d_psi.data_ptr()),
               C.c_void_p(d_out.data_ptr()), C.c_void_p(stream))
    assert e.value.code == A.QD_ERR_INVALID
