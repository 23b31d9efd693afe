"""Bit-exact basis and lowered matrix at the full sizes of the workloads.

The sector basis (ascending integer order, conservation.hpp:212-225 with
SubIndex's ranks, index.hpp:234-240) and the CSC matrix of `ham >> chain`
(operator.hpp:235-267: pattern, explicit zeros and complex128 values) are
compared with == against the oracle's restatement at:

* the periodic XXZ chain at L=24, Sz=0 (dim 2,704,156, nnz 36,564,892), the
  Lanczos headline workload;
* a random-field XXZ chain at L=20 (h_i ~ U[-2,2], Jz=1, periodic, Sz=0,
  dim 184,756), the largest instance of the batched disorder sweep;
* an XXZ chain at L=22 with Jz ~ U[0,2] and fields h_i ~ U[-1,1] (Sz=0,
  dim 705,432), the largest request of the serving mix.

Each case also checks sampled ranks, including states outside the sector
(rank = dim), and the CSR the device keeps (the transpose of the CSC).
"""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import chains

pytestmark = pytest.mark.gpu


def disorder_instance(L=20, seed=2024):
    rng = np.random.Generator(np.random.PCG64(seed))
    h = rng.uniform(-2.0, 2.0, L)
    return chains.xxz_chain(L, 1.0, 1.0, True, h)


def serving_instance(L=22, seed=77):
    rng = np.random.Generator(np.random.PCG64(seed))
    Jz = float(rng.uniform(0.0, 2.0))
    h = rng.uniform(-1.0, 1.0, size=L)
    return chains.xxz_chain(L, 1.0, Jz, True, h)


CASES = {
    "xxz_L24_periodic": lambda: chains.xxz_chain(24, 1.0, 1.0, True),
    "xxz_L20_random_field": disorder_instance,
    "xxz_L22_fields_random_Jz": serving_instance,
}


@pytest.mark.parametrize("name", list(CASES))
def test_full_size_basis_and_matrix_bit_exact(ctx, golden, name):
    spec, ham = CASES[name]()
    L = spec.nbits
    osec = O.Sector(spec)
    gsec = q.Sector(spec.index, spec.constraints)
    dim, nnz = golden["xxz_periodic_dim_nnz"][str(L)]
    assert gsec.dim == osec.dim == dim
    ob = osec.basis()
    assert np.array_equal(gsec.basis(), ob)
    rng = np.random.default_rng(L)
    states = np.concatenate([ob[rng.integers(0, dim, 4000)],
                             rng.integers(0, 1 << L, 4000, dtype=np.uint64)])
    ref = np.array([osec.rank(int(s)) for s in states])
    assert np.array_equal(gsec.rank(states), ref)
    assert np.count_nonzero(ref == dim) > 0  # some sampled states lie outside the sector
    del ob

    oh = O.Ham(osec, ham)
    gh = gsec.lower(ham)
    assert (gh.dim, gh.nnz) == (oh.dim, oh.nnz) == (dim, nnz)
    ocp, ori, ocv = oh.csc()
    cp, ri, cv = gh.csc()
    assert np.array_equal(cp, ocp)
    assert np.array_equal(ri, ori)
    assert np.array_equal(cv.view(np.float64), ocv.view(np.float64))  # same bits, zeros included
    del cp, ri, cv
    # the device's row-major copy is the exact transpose of the oracle's matrix
    import scipy.sparse as sp
    M = sp.csc_matrix((ocv, ori, ocp), shape=(dim, dim)).tocsr()
    M.sort_indices()
    rp, ci, rv = gh.csr()
    assert np.array_equal(rp, M.indptr)
    assert np.array_equal(ci, M.indices)
    assert np.array_equal(rv.view(np.float64), M.data.view(np.float64))
