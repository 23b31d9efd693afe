"""Batched mixed-precision Lanczos vs the FP64 oracle, instance by instance."""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import chains

pytestmark = pytest.mark.gpu

DE_TOL = 1e-8  # relative, refined energy vs the FP64 oracle


def disorder_instances(n, Ls, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        L = int(rng.choice(Ls))
        h = rng.uniform(-2.0, 2.0, L)
        out.append((L, h))
    return out


def test_batch_matches_fp64_oracle(ctx):
    inst = disorder_instances(12, [10, 12, 14], 3)
    hams, v0s, oracles = [], [], []
    for L, h in inst:
        spec, ham = chains.xxz_chain(L, 1.0, 1.0, True, h)
        sec = q.Sector(spec.index, spec.constraints)
        hams.append(sec.lower(ham))
        v0 = q.start_vector(sec.dim, 100 + L)
        v0s.append(v0)
        oh = O.Ham(O.Sector(spec), ham)
        oracles.append(oh.lanczos_ground(v0, 80))
        hams[-1]._keep = sec
    out = q.batch_lanczos(hams, v0s, 80)
    for i, o in enumerate(oracles):
        ref = o["ritz"]
        assert abs(out[i, 1] - ref) <= DE_TOL * abs(ref), (i, out[i], ref)
        assert abs(out[i, 0] - ref) <= 1e-5 * abs(ref)  # FP32 Krylov eigenvalue before refinement
        assert out[i, 3] == 80 and out[i, 4] == 0


def test_batch_small_spaces_break_down(ctx):
    # dims below the step count: the recurrence stops, the result is still exact
    hams, v0s, exact = [], [], []
    for L in (4, 6, 8):  # dims 6 and 20 are exhausted within 40 steps, 70 is not
        spec, ham = chains.xxz_chain(L, 1.0, 0.5, True, np.linspace(-1, 1, L))
        sec = q.Sector(spec.index, spec.constraints)
        H = sec.lower(ham)
        H._keep = sec
        hams.append(H)
        v0s.append(q.start_vector(sec.dim, L))
        exact.append(np.linalg.eigvalsh(H.scipy().toarray())[0])
    out = q.batch_lanczos(hams, v0s, 40)
    for i, e in enumerate(exact):
        assert out[i, 4] == (1 if i < 2 else 0)
        assert abs(out[i, 1] - e) <= 1e-9 * abs(e)


def test_batch_cluster_instances_match_fp64(ctx):
    """Instances of dim >= 32768 run on thread-block clusters (row slices, inner products combined
    through distributed shared memory; 8-CTA clusters for a call with this few of them); mixed in one
    call with single-CTA instances, every refined energy stays within 1e-8 of the FP64 Lanczos of the
    same start vector."""
    inst = [(18, np.random.default_rng(1).uniform(-2, 2, 18)), (12, np.random.default_rng(2).uniform(-2, 2, 12)),
            (18, np.random.default_rng(3).uniform(-2, 2, 18)), (14, np.random.default_rng(4).uniform(-2, 2, 14))]
    hams, v0s, ref = [], [], []
    for L, h in inst:
        spec, ham = chains.xxz_chain(L, 1.0, 1.0, True, h)
        sec = q.Sector(spec.index, spec.constraints)
        H = sec.lower(ham)
        H._keep = sec
        hams.append(H)
        v0 = q.start_vector(sec.dim, 7 + L)
        v0s.append(v0)
        psi = q.getState(sec, 1)
        psi.set(0, v0)
        ref.append(q.LanczosSolver(sec, 80).getGroundState(H, psi, 0).ritz_value)
    assert hams[0].dim == 48620  # a cluster instance
    out = q.batch_lanczos(hams, v0s, 80)
    for i, e in enumerate(ref):
        assert abs(out[i, 1] - e) <= DE_TOL * abs(e), (i, out[i], e)
        assert out[i, 3] == 80 and out[i, 4] == 0
    # the same instances alone give the same bits as in the mix
    alone = q.batch_lanczos(hams[:1], v0s[:1], 80)
    assert np.array_equal(alone[0, :5], out[0, :5])


def test_batch_many_large_instances_take_small_clusters(ctx):
    """A call with more large instances than 4-CTA clusters can hold at once runs them on 2-CTA
    clusters (more instances side by side); a sample of the energies stays within 1e-8 of the FP64
    Lanczos, and the call's instances agree with the same instances in a call of two (8-CTA
    clusters) to the same tolerance."""
    n = 160
    rng = np.random.default_rng(11)
    hams, v0s = [], []
    for i in range(n):
        spec, ham = chains.xxz_chain(18, 1.0, 1.0, True, rng.uniform(-2, 2, 18))
        sec = q.Sector(spec.index, spec.constraints)
        H = sec.lower(ham)
        H._keep = sec
        hams.append(H)
        v0s.append(q.start_vector(sec.dim, 500 + i))
    out = q.batch_lanczos(hams, v0s, 80)
    few = q.batch_lanczos(hams[:2], v0s[:2], 80)
    for i in (0, 1, 77, 159):
        psi = q.getState(hams[i]._keep, 1)
        psi.set(0, v0s[i])
        e = q.LanczosSolver(hams[i]._keep, 80).getGroundState(hams[i], psi, 0).ritz_value
        assert abs(out[i, 1] - e) <= DE_TOL * abs(e), (i, out[i], e)
        assert out[i, 3] == 80 and out[i, 4] == 0
    for i in (0, 1):
        assert abs(out[i, 1] - few[i, 1]) <= DE_TOL * abs(few[i, 1])


def bond_disorder_xxz(L, seed):
    """XXZ ring with bond-dependent hopping: no common off-diagonal value."""
    from qudrip_gb300.operators import (II, SectorSpec, getBoseGate, getEmptyOperator, getNset, getQbits,
                                        pauli_x, pauli_y, pauli_z)
    rng = np.random.default_rng(seed)
    pre = getQbits(L)
    gc, ga, gz = getBoseGate(pre), getBoseGate(pre), getBoseGate(pre)
    gc << 0.5 * (pauli_x + II * pauli_y)
    ga << 0.5 * (pauli_x - II * pauli_y)
    gz << 0.5 * pauli_z
    ham = getEmptyOperator()
    for i in range(L):
        j = (i + 1) % L
        t = float(rng.uniform(0.5, 1.5))
        ham = ham + (0.5 * t) * (gc(i) * ga(j)) + (0.5 * t) * (gc(j) * ga(i)) + gz(i) * gz(j)
    return SectorSpec(pre, [getNset(pre) == L // 2]), ham


def test_batch_uniform_and_valued_products_in_one_call(ctx):
    """One call mixing the two FP32 products: uniform hopping with a diagonal (random-field
    XXZ), uniform hopping without stored diagonal entries (open XY chain: the column sum must
    not count x_r), bond disorder (the valued product) and a diagonal matrix (no off-diagonal
    value: the valued product).  Each refined energy is within
    DE_TOL of the FP64 oracle; out[:, 5:8] hold each instance's device start and end (ns) and
    the CTAs that computed it."""
    cases = [chains.xxz_chain(14, 1.0, 1.0, True, np.random.default_rng(7).uniform(-2, 2, 14)),
             chains.xy_chain(14),
             bond_disorder_xxz(14, 8),
             bond_disorder_xxz(18, 9),  # a cluster instance (dim 48,620) on the valued product
             chains.xxz_chain(12, 0.0, 1.0, True, np.linspace(-1, 1, 12))]  # no off-diagonal entry at all
    hams, v0s, refs = [], [], []
    for spec, ham in cases:
        sec = q.Sector(spec.index, spec.constraints)
        H = sec.lower(ham)
        H._keep = sec
        hams.append(H)
        v0 = q.start_vector(sec.dim, 40 + len(hams))
        v0s.append(v0)
        refs.append(O.Ham(O.Sector(spec), ham).lanczos_ground(v0, 60)["ritz"])
    out = q.batch_lanczos(hams, v0s, 60)
    for i, ref in enumerate(refs):
        assert abs(out[i, 1] - ref) <= DE_TOL * abs(ref), (i, out[i, 1], ref)
    assert np.all(out[:, 6] > out[:, 5]) and np.all(out[:, 5] > 0)
    assert out[3, 7] >= 2 and out[0, 7] == 1
    # the same energies when every instance takes the valued product
    import os
    os.environ["QD_BATCH_UNIFORM"] = "0"
    try:
        out2 = q.batch_lanczos(hams, v0s, 60)
    finally:
        del os.environ["QD_BATCH_UNIFORM"]
    assert np.allclose(out2[:, 1], out[:, 1], rtol=DE_TOL, atol=0)


def test_batch_one_state_and_empty_instances(ctx):
    """A one-state sector (no particle) batched beside a normal instance gives its diagonal
    value exactly; a sector without states is refused before any device work."""
    from qudrip_gb300 import _capi as A
    spec1, ham1 = chains.xxz_chain(6, 1.0, 1.0, True, np.linspace(-1, 1, 6))
    vac = q.SectorSpec(spec1.index, [q.getNset(spec1.index) == 0])
    sec0 = q.Sector(vac.index, vac.constraints)
    H0 = sec0.lower(ham1)
    H0._keep = sec0
    assert sec0.dim == 1
    spec2, ham2 = chains.xxz_chain(10, 1.0, 1.0, True, np.linspace(-1, 1, 10))
    sec2 = q.Sector(spec2.index, spec2.constraints)
    H2 = sec2.lower(ham2)
    H2._keep = sec2
    out = q.batch_lanczos([H0, H2], [np.ones(1), q.start_vector(sec2.dim, 3)], 40)
    d = H0.scipy().toarray()[0, 0].real
    assert abs(out[0, 1] - d) <= 1e-12 * max(1.0, abs(d)) and out[0, 3] == 1
    ref = O.Ham(O.Sector(spec2), ham2).lanczos_ground(q.start_vector(sec2.dim, 3), 40)["ritz"]
    assert abs(out[1, 1] - ref) <= DE_TOL * abs(ref)
    empty = q.SectorSpec(spec1.index, [q.getNset(spec1.index) == 7])
    sec_e = q.Sector(empty.index, empty.constraints)
    He = sec_e.lower(ham1)
    He._keep = sec_e
    with pytest.raises(A.QDError) as e:
        q.batch_lanczos([He], [np.ones(0)], 10)
    assert e.value.code == A.QD_ERR_INVALID


def test_full_disorder_sweep_within_tolerance_of_fp64(ctx):
    """The batched workload at its full size: 512 random-field XXZ chains (L drawn from
    {14, 16, 18, 20}, h_i ~ U[-2, 2], periodic, Sz = 0), 80 steps each, in one call; every refined
    energy within 1e-8 relative of the plain FP64 Lanczos solve of the same instance and start
    vector, and the device clock columns consistent (every instance starts and ends inside the
    call, on the CTAs its size asks for)."""
    rng = np.random.Generator(np.random.PCG64(2024))
    hams, v0s, dims = [], [], []
    for i in range(512):
        L = int(rng.choice([14, 16, 18, 20]))
        h = rng.uniform(-2.0, 2.0, L)
        spec, ham = chains.xxz_chain(L, 1.0, 1.0, True, h)
        sec = q.Sector(spec.index, spec.constraints)
        H = sec.lower(ham)
        H._keep = sec
        hams.append(H)
        v0s.append(q.start_vector(sec.dim, 2024 + i))
        dims.append(sec.dim)
    out = q.batch_lanczos(hams, v0s, 80)
    worst = 0.0
    states = {}
    for i, H in enumerate(hams):
        st = states.get(dims[i])
        if st is None:
            st = states[dims[i]] = q.getState(H._keep, 1)
        st.set(0, v0s[i])
        e = q.Arnoldi.getLanczosSolver(H._keep, 80).getGroundState(H, st(0), 0).ritz_value
        worst = max(worst, abs(out[i, 1] - e) / abs(e))
    assert worst <= DE_TOL, worst
    big = np.array(dims) >= 32768
    assert np.all(out[big, 7] >= 2) and np.all(out[~big, 7] == 1)
    assert np.all(out[:, 6] > out[:, 5])
    assert out[:, 6].max() - out[:, 5].min() < 5e9  # the whole call inside five seconds of device time
