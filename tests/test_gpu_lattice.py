"""Lattice models through the device path: Model.getHamiltonian feeds the lowering like any operator
(lattice.hpp:370-383), Model.getHamiltonianMatrix sums lowered matrices on the device
(lattice.hpp:355-368, qd_ham_add), and McManager's incrMatrix / normMatrix (mc_manager.hpp:72-83)."""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A

pytestmark = pytest.mark.gpu


def square(nx, ny):
    return q.Lattice([(i, j) for i in range(nx) for j in range(ny)], [(nx, 0), (0, ny)])


def heisenberg_model(nx, ny, J=1.0, Jz=1.0):
    L = square(nx, ny)
    m = q.Model(L)
    p = q.params_type()
    p["J"] = J
    p["Jz"] = Jz
    for i in range(L.N()):
        for a in ((1, 0), (0, 1)):
            m.addBond(i, L(L(i) + np.array(a)), p)
    pre = q.getQbits(L.N())
    gc, ga, gz = q.getBoseGate(pre), q.getBoseGate(pre), q.getBoseGate(pre)
    gc << 0.5 * (q.pauli_x + q.II * q.pauli_y)
    ga << 0.5 * (q.pauli_x - q.II * q.pauli_y)
    gz << 0.5 * q.pauli_z

    def bond(s1, s2, p):
        return (0.5 * p("J")) * (gc(s1) * ga(s2)) + (0.5 * p("J")) * (gc(s2) * ga(s1)) + p("Jz") * (gz(s1) * gz(s2))

    spec = q.SectorSpec(pre, [q.getNset(pre) == L.N() // 2])
    return L, m, bond, spec


def sector_of(spec):
    return q.Sector(spec.index, spec.constraints, spec.tight)


def test_model_hamiltonian_ground_state_4x4(ctx):
    L, m, bond, spec = heisenberg_model(4, 4)
    ham = m.getHamiltonian(bond)
    sec = sector_of(spec)
    H = sec.lower(ham)
    assert sec.dim == 12870
    v0 = q.start_vector(sec.dim, 4)
    psi = q.getState(sec, 1)
    psi.set(0, v0)
    r = q.LanczosSolver(sec, 100).getGroundState(H, psi, 0)
    o = O.Ham(O.Sector(spec), ham).lanczos_ground(v0, 100)
    assert r.act_dim == o["act_dim"]
    assert abs(r.ritz_value - o["ritz"]) <= 1e-10 * abs(o["ritz"])
    import scipy.sparse.linalg as sla
    e0 = sla.eigsh(H.scipy().real, k=1, which="SA", tol=1e-12)[0][0]
    assert abs(r.ritz_value - e0) <= 1e-8 * abs(e0)
    assert abs(e0 - (-11.228483208428854)) < 1e-8  # 4x4 periodic Heisenberg, -0.70178 per site


def test_matrix_sum_equals_lowering_of_the_sum(ctx):
    L, m, bond, spec = heisenberg_model(3, 4, J=0.8, Jz=1.3)
    sec = sector_of(spec)
    Hs = m.getHamiltonianMatrix(lambda a, b, p: sec.lower(bond(a, b, p)), sec)
    Ho = sec.lower(m.getHamiltonian(bond))
    p1, c1, v1 = Hs.csr()
    p2, c2, v2 = Ho.csr()
    assert Hs.nnz == Ho.nnz and np.array_equal(p1, p2) and np.array_equal(c1, c2)
    assert np.array_equal(v1, v2)  # per-entry sums in the same term order (signed zeros aside)
    assert Hs.is_real and Hs.is_hermitian
    # a sum has no operator terms: no matrix-free form, but every solver takes it
    with pytest.raises(A.QDError) as e:
        A.call("qd_ham_build_matrix_free", Hs.handle)
    assert e.value.code == A.QD_ERR_UNSUPPORTED
    v0 = q.start_vector(sec.dim, 9)
    out = []
    for H in (Hs, Ho):
        psi = q.getState(sec, 1)
        psi.set(0, v0)
        out.append(q.LanczosSolver(sec, 60).getGroundState(H, psi, 0).ritz_value)
    assert abs(out[0] - out[1]) <= 1e-12 * abs(out[1])


def test_add_scale_copy(ctx):
    from qudrip_gb300 import chains
    spec, ham = chains.xxz_chain(10, 1.0, 0.6, periodic=False, fields=np.linspace(-1, 1, 10))
    spec2, ham2 = chains.xy_chain(10, periodic=True)
    sec = sector_of(spec)
    a, b = sec.lower(ham), sec.lower(ham2)
    s = a + b
    da, db, ds = a.scipy().toarray(), b.scipy().toarray(), s.scipy().toarray()
    assert np.array_equal(ds, da + db)
    pa, ca, _ = a.csr()
    pb, cb, _ = b.csr()
    union = sum(len(set(ca[pa[r]:pa[r + 1]]) | set(cb[pb[r]:pb[r + 1]])) for r in range(sec.dim))
    assert s.nnz == union  # explicit zeros kept
    z = complex(0.3, -1.7)
    c = z * a  # a scaled copy; a itself unchanged
    assert np.array_equal(a.scipy().toarray(), da)
    _, _, va = a.csr()
    _, _, vc = c.csr()
    np.testing.assert_allclose(vc, va * z, rtol=4e-16, atol=0)
    assert not c.is_real and not c.is_hermitian
    c.scale(1 / z)
    np.testing.assert_allclose(c.scipy().toarray(), da, rtol=1e-15, atol=1e-15)
    with pytest.raises(A.QDError):
        _ = a + sector_of(spec2).lower(ham2)  # different sectors


def test_mcmanager_incr_and_norm_matrix(ctx):
    from qudrip_gb300 import chains
    Lc = 8
    spec, ham = chains.xxz_chain(Lc, 1.0, 0.4, periodic=True, fields=np.linspace(-0.5, 0.5, Lc))
    sec = sector_of(spec)
    H = sec.lower(ham)
    psi = q.getState(sec, 1)
    psi.set(0, q.start_vector(sec.dim, 3))
    q.LanczosSolver(sec, 40).getGroundState(H, psi, 0)
    pre = spec.index
    gn = q.getBoseGate(pre)
    gn << np.array([[0, 0], [0, 1]], dtype=complex)
    mc = q.McManager(1, psi)
    mc.addObs("nbar", 1, q.MC_REAL)
    mc.addObs("n", Lc)
    for i in range(Lc):
        ni = sec.lower(q.OperatorSum([(gn(i), 1.0 + 0j)]))
        mc.updateMatrix("n", i, ni)
        mc.incrMatrix("nbar", 0, ni)
    mc.normMatrix("nbar", 0, 1.0 / Lc)
    mc.incrAllObs(0)
    mc.normAll()
    dens = mc.data["n"][0]
    assert abs(mc.obsValue("nbar", 0, 0) - dens.mean()) < 1e-13
    assert abs(dens.sum().real - Lc // 2) < 1e-10  # Sz = 0 sector: half filling
