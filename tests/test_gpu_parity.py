"""GPU engine vs the CPU oracle, through the C ABI.

Integer work (basis, ranks, CSC/CSR pattern) must be bit-exact; lowered values
are compared with == (the device reproduces the reference's rounding); FP64
solver results use the stated tolerances.
"""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import chains
from qudrip_gb300.operators import (SectorSpec, getFermiGate, getNd, getNdo, getNset, getNup, getQbits,
                                    getEmptyOperator, pauli_x, pauli_y, II)

pytestmark = pytest.mark.gpu

E_TOL = 1e-10  # relative, FP64 ground-state energies


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


def hubbard_nd_sector(L, Nup, Ndo, docc):
    """Hubbard chain in a sector fixed by Nup, Ndo and the doublon count (no product structure)."""
    spec, ham = chains.hubbard_chain(L, Nup, Ndo, 4.0, -1.0, periodic=True)
    spec.constraints.append(getNd(spec.index, L) == docc)
    return spec, ham


SYSTEMS = {
    "xy16": lambda: chains.xy_chain(16),
    "xxz14_fields": lambda: chains.xxz_chain(14, 1.0, 0.6, True, list(np.linspace(-1.5, 1.2, 14))),
    "hubbard4_periodic": lambda: chains.hubbard_chain(4, 2, 2, 4.0, -1.0, periodic=True),
    "hubbard5_open": lambda: chains.hubbard_chain(5, 3, 2, 2.5, -1.0, periodic=False),
    "fermi_complex10": lambda: fermi_bitgate_chain(10),
    "hubbard4_nd": lambda: hubbard_nd_sector(4, 2, 2, 1),
}


def gpu_objects(spec, ham):
    sec = q.Sector(spec.index, spec.constraints, spec.tight)
    return sec, sec.lower(ham)


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_basis_and_ranks_bit_exact(ctx, name):
    spec, _ = SYSTEMS[name]()
    osec = O.Sector(spec)
    gsec = q.Sector(spec.index, spec.constraints, spec.tight)
    assert gsec.dim == osec.dim
    assert np.array_equal(gsec.basis(), osec.basis())
    rng = np.random.default_rng(0)
    states = np.concatenate([osec.basis()[rng.integers(0, osec.dim, 200)],
                             rng.integers(0, 1 << spec.nbits, 200, dtype=np.uint64),
                             np.array([(1 << spec.nbits), 2**63], dtype=np.uint64)])
    ref = np.array([osec.rank(int(s)) for s in states])
    assert np.array_equal(gsec.rank(states), ref)


def test_sector_kinds(ctx):
    spec, _ = chains.xy_chain(12)
    assert q.Sector(spec.index, spec.constraints).rank_kind() == 1
    spec, _ = hubbard_nd_sector(4, 2, 2, 1)
    assert q.Sector(spec.index, spec.constraints).rank_kind() == 0
    pre = getQbits(10)
    loose = q.LooseConstrain(pre, 1, getNset(pre) == 5)
    osec = O.Sector(SectorSpec(pre, [getNset(pre) == 5], tight=1))
    assert np.array_equal(loose.basis(), osec.basis())
    # combination nup + ndo = 3 with an overlapping Nset
    fermi = getQbits(8)
    combo = [getNup(fermi, 4) + getNdo(fermi, 4) == 3]
    assert np.array_equal(q.Sector(fermi, combo).basis(), O.Sector(SectorSpec(fermi, combo)).basis())
    empty = q.Sector(getQbits(6), [getNset(getQbits(6)) == 9])
    assert empty.dim == 0


@pytest.mark.parametrize("path", ["rows", "tree"])
@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_lowering_bit_exact(ctx, name, path, monkeypatch):
    if path == "tree":  # the per-column tree walk instead of the compiled row-wise pull
        monkeypatch.setenv("QD_LOWER_TREE", "1")
    spec, ham = SYSTEMS[name]()
    osec = O.Sector(spec)
    oh = O.Ham(osec, ham)
    gsec, gh = gpu_objects(spec, ham)
    assert (gh.dim, gh.nnz) == (oh.dim, oh.nnz)
    cp, ri, cv = gh.csc()
    ocp, ori, ocv = oh.csc()
    assert np.array_equal(cp, ocp)
    assert np.array_equal(ri, ori)
    assert np.array_equal(cv, ocv)  # IEEE equality: the reference's own rounding
    # CSR is the exact transpose
    rp, ci, rv = gh.csr()
    M = oh.scipy().tocsr()
    M.sort_indices()
    assert np.array_equal(rp, M.indptr) and np.array_equal(ci, M.indices) and np.array_equal(rv, M.data)
    real = not np.any(ocv.imag != 0)
    assert gh.is_real == real
    assert gh.is_hermitian


def test_explicit_zeros_kept(ctx, golden):
    spec, ham = chains.xxz_chain(16)
    gsec, gh = gpu_objects(spec, ham)
    dim, nnz = golden["xxz_periodic_dim_nnz"]["16"]
    assert (gh.dim, gh.nnz) == (dim, nnz)
    rp, ci, rv = gh.csr()
    assert np.count_nonzero(rv == 0) > 0  # diagonal entries where the bond sum cancels


@pytest.mark.parametrize("name", ["xy16", "xxz14_fields", "fermi_complex10", "hubbard4_nd"])
def test_apply_and_eval(ctx, name):
    spec, ham = SYSTEMS[name]()
    oh = O.Ham(O.Sector(spec), ham)
    gsec, gh = gpu_objects(spec, ham)
    rng = np.random.default_rng(11)
    x = rng.normal(size=gh.dim) + 1j * rng.normal(size=gh.dim)
    st = q.getState(gsec, 2)
    st.set(0, x)
    q.apply(gh, st, 0, st, 1)
    y = st.get(1)
    yo = oh.apply(x)
    assert np.abs(y - yo).max() <= 1e-13 * np.abs(yo).max()
    e = st.eval(0, gh)
    eo = oh.eval(x)
    assert abs(e - eo) <= 1e-12 * abs(eo)


def lanczos_pair(spec, ham, kry, seed, ritz=q._capi.QD_RITZ_STORED_BASIS, v0=None):
    osec = O.Sector(spec)
    oh = O.Ham(osec, ham)
    gsec, gh = gpu_objects(spec, ham)
    if v0 is None:
        v0 = q.start_vector(gsec.dim, seed)
    ores = oh.lanczos_ground(v0, kry)
    psi = q.getState(gsec, 1)
    psi.set(0, v0)
    solver = q.Arnoldi.getLanczosSolver(gsec, kry, ritz=ritz)
    res = solver.getGroundState(gh, psi(0), 0)
    gpsi = psi.get(0)
    E = psi.eval(0, gh)
    return oh, ores, gh, solver, res, gpsi, E


def check_energies(oh, ores, solver, res, gpsi, E):
    lam_o = ores["ritz"]
    lam = res.ritz_value
    assert abs(lam - lam_o) <= E_TOL * abs(lam_o)
    nrm = np.vdot(gpsi, gpsi).real
    rq = E.real / nrm
    orq = ores["energy"].real / np.vdot(ores["psi"], ores["psi"]).real
    assert abs(rq - orq) <= E_TOL * abs(orq)
    # the raw psi.eval value carries the norm defect of the unorthogonalised
    # Ritz vector; it agrees with the oracle's within that conditioning
    defect = abs(nrm - 1) + abs(np.vdot(ores["psi"], ores["psi"]).real - 1)
    assert abs(E.real - ores["energy"].real) <= abs(lam_o) * defect + E_TOL * abs(lam_o)
    assert res.act_dim == ores["act_dim"] and res.breakdown == ores["breakdown"]


def test_lanczos_xy16_open_chain(ctx, golden):
    spec, ham = chains.xy_chain(16)
    oh, ores, gh, solver, res, gpsi, E = lanczos_pair(spec, ham, 100, 12345)
    check_energies(oh, ores, solver, res, gpsi, E)
    exact = golden["xy_open_closed_form"]["16"]
    assert abs(res.ritz_value - exact) <= 1e-12 * abs(exact)
    # without reorthogonalisation copies ("ghosts") of the converged ground
    # level appear at rounding-dependent positions; the first genuinely
    # excited level is converged and must agree
    ev = solver.eigenvalues()
    lam0 = ev[0]
    first = ev[ev > lam0 + 1e-3][0]
    ofirst = ores["evals"][ores["evals"] > lam0 + 1e-3][0]
    assert abs(first - ofirst) <= 1e-9


def test_lanczos_complex_hamiltonian(ctx):
    spec, ham = fermi_bitgate_chain(12)
    oh, ores, gh, solver, res, gpsi, E = lanczos_pair(spec, ham, 80, 3)
    assert not gh.is_real
    check_energies(oh, ores, solver, res, gpsi, E)


def test_lanczos_complex_start_vector(ctx):
    spec, ham = chains.xxz_chain(12, 1.0, 0.8, True, [0.1 * i for i in range(12)])
    rng = np.random.default_rng(4)
    v0 = rng.uniform(-1, 1, 924) + 1j * rng.uniform(-1, 1, 924)
    oh, ores, gh, solver, res, gpsi, E = lanczos_pair(spec, ham, 60, 0, v0=v0)
    check_energies(oh, ores, solver, res, gpsi, E)


def test_lanczos_breakdown_matches_oracle(ctx):
    spec, ham = chains.hubbard_chain(2, 1, 0, 0.0, -1.0)
    oh, ores, gh, solver, res, gpsi, E = lanczos_pair(spec, ham, 10, 0, v0=np.array([1.0, 0.3]))
    assert res.breakdown == 1 and res.act_dim == ores["act_dim"] == 1


def test_second_pass_equals_stored_basis(ctx):
    spec, ham = chains.xxz_chain(14)
    gsec, gh = gpu_objects(spec, ham)
    v0 = q.start_vector(gsec.dim, 9)
    out = []
    for ritz in (q._capi.QD_RITZ_STORED_BASIS, q._capi.QD_RITZ_SECOND_PASS):
        psi = q.getState(gsec, 1)
        psi.set(0, v0)
        s = q.Arnoldi.getLanczosSolver(gsec, 50, ritz=ritz)
        r = s.getGroundState(gh, psi(0), 0)
        out.append((psi.get(0), r.matvecs))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[1][1] == out[0][1] + 50


def test_xxz_L24_periodic_full_size(ctx, golden):
    spec, ham = chains.xxz_chain(24, 1.0, 1.0, True)
    gsec, gh = gpu_objects(spec, ham)
    dim, nnz = golden["xxz_periodic_dim_nnz"]["24"]
    assert (gsec.dim, gh.nnz) == (dim, nnz)
    assert gh.max_row_nnz == 25
    b = gsec.basis()
    assert np.all(np.diff(b.astype(np.int64)) > 0)
    psi = q.getState(gsec, 1)
    psi.set(0, q.start_vector(gsec.dim, 12345))
    res = q.Arnoldi.getLanczosSolver(gsec, 100).getGroundState(gh, psi(0), 0)
    e0 = golden["heisenberg_periodic_e0"]["24"]["e0"]
    assert abs(res.ritz_value - e0) <= E_TOL * abs(e0)
    g = psi.get(0)
    rq = psi.eval(0, gh).real / np.vdot(g, g).real
    assert abs(rq - e0) <= E_TOL * abs(e0)


def all_to_all_hopping(L):
    """Long rows (every pair hops): exercises the long-row fallbacks of the tile kernels."""
    pre = getQbits(L)
    spec = SectorSpec(pre, [getNset(pre) == L // 2])
    gc = q.getBoseGate(pre)
    ga = q.getBoseGate(pre)
    gc << 0.5 * (pauli_x + II * pauli_y)
    ga << 0.5 * (pauli_x - II * pauli_y)
    ham = getEmptyOperator()
    for i in range(L):
        for j in range(L):
            if i != j:
                ham = ham + (0.1 * (i + 1) + 0.01 * j) * (gc(i) * ga(j))
    return spec, ham


@pytest.mark.parametrize("name", ["xxz14_fields", "fermi_complex10", "all_to_all12"])
def test_every_product_kernel(ctx, name):
    import ctypes as C
    from qudrip_gb300 import _capi as A
    spec, ham = all_to_all_hopping(12) if name == "all_to_all12" else SYSTEMS[name]()
    oh = O.Ham(O.Sector(spec), ham)
    gsec, gh = gpu_objects(spec, ham)
    rng = np.random.default_rng(2)
    x = rng.normal(size=gh.dim) + 1j * rng.normal(size=gh.dim)
    yo = oh.apply(x)
    st = q.getState(gsec, 2)
    st.set(0, x)
    for kern in sorted(A.SPMV_KERNELS):
        A.call("qd_ham_set_spmv_kernel", gh.handle, kern)
        q.apply(gh, st, 0, st, 1)
        y = st.get(1)
        assert np.abs(y - yo).max() <= 1e-13 * np.abs(yo).max(), A.SPMV_KERNELS[kern]
        e = st.eval(0, gh)
        assert abs(e - oh.eval(x)) <= 1e-12 * abs(e)
    chosen = C.c_int(0)
    ms = C.c_double(0)
    A.call("qd_ham_autotune", gh.handle, 3, C.byref(chosen), C.byref(ms))
    # 120 (the uniform-coupling fixed-point form) competes where it applies
    assert (chosen.value in A.SPMV_KERNELS or chosen.value in (A.QD_SPMV_FX, A.QD_SPMV_FX_SLOTS)) and ms.value > 0


def test_incremental_add_dim_grows_the_same_krylov_space(ctx):
    """getGroundState(..., add_dim) three times = one solve of the full dimension
    (updateKrylovRepr, sparse_algorithm.hpp:521-546), with error() the change of
    the tracked eigenvalues between calls."""
    spec, ham = chains.xxz_chain(14, 1.0, 0.8, True, list(np.linspace(-0.5, 0.7, 14)))
    gsec, gh = gpu_objects(spec, ham)
    v0 = q.start_vector(gsec.dim, 21)
    one = q.Arnoldi.getLanczosSolver(gsec, 60)
    p1 = q.getState(gsec, 1)
    p1.set(0, v0)
    one.getGroundState(gh, p1(0), 0)
    inc = q.Arnoldi.getLanczosSolver(gsec, 60)
    inc.convergeEV(2)
    p2 = q.getState(gsec, 1)
    p2.set(0, v0)
    oh = O.Ham(O.Sector(spec), ham)
    prev = np.zeros(2)
    for step, k in enumerate((20, 40, 60)):
        inc.getGroundState(gh, p2(0), 0, add_dim=20)
        assert inc.act_dim() == k
        ev = inc.eigenvalues()
        assert abs(inc.error() - np.sqrt(np.sum((ev[:2] - prev) ** 2))) <= 1e-12 * (1 + abs(ev[0]))
        prev = ev[:2].copy()
        o = oh.lanczos_ground(v0, k)
        assert abs(ev[0] - o["ritz"]) <= 1e-10 * abs(o["ritz"])
    assert np.array_equal(inc.eigenvalues(), one.eigenvalues())
    assert np.array_equal(p2.get(0), p1.get(0))
    inc.getGroundState(gh, p2(0), 0, add_dim=20)  # the space is full: nothing changes
    assert inc.act_dim() == 60
