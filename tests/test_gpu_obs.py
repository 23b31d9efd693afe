"""Observable lists (McManager::incrAllObs / normAll) against the oracle's psi.eval."""
import numpy as np
import pytest

import oracle as O
import qudrip_gb300 as q
from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains

pytestmark = pytest.mark.gpu


def observables(spec, L):
    g = q.getHopFermiGate(spec.index)
    ops = {}
    for i in range(L):
        ops[f"docc{i}"] = chains.docc_operator(L, i, spec.index)
        ops[f"nup{i}"] = 1.0 * g(i, i)
    ops["hop01"] = 1.0 * g(1, 0) + 1.0 * g(0, 1)
    ops["current01"] = 1j * g(1, 0) + (-1j) * g(0, 1)
    return ops


def test_obs_eval_and_mc_manager_match_the_oracle(ctx):
    L = 4
    spec, ham = chains.hubbard_chain(L, 2, 2, 4.0, -1.0, periodic=True)
    sec = q.Sector(spec.index, spec.constraints)
    osec = O.Sector(spec)
    ops = observables(spec, L)
    psi = q.getState(sec, 3)
    mc = q.McManager(3, psi)
    mc.addObs("docc", L)
    mc.addObs("hop", 2)
    mc.addAux("docc_abs2", "docc", lambda v: abs(v) ** 2, L)
    for i in range(L):
        mc.updateMatrix("docc", i, sec.lower(ops[f"docc{i}"]))
    mc.updateMatrix("hop", 0, sec.lower(ops["hop01"]))
    mc.updateMatrix("hop", 1, sec.lower(ops["current01"]))
    rng = np.random.default_rng(4)
    want = np.zeros((3, L), dtype=np.complex128)
    want_hop = np.zeros((3, 2), dtype=np.complex128)
    want_aux = np.zeros((3, L))
    for sample in range(3):
        for t in range(3):
            v = rng.normal(size=sec.dim) + 1j * rng.normal(size=sec.dim)
            psi.set(t, v)
            for i in range(L):
                e = O.Ham(osec, ops[f"docc{i}"]).eval(v)
                want[t, i] += e
                want_aux[t, i] += abs(e) ** 2
            want_hop[t, 0] += O.Ham(osec, ops["hop01"]).eval(v)
            want_hop[t, 1] += O.Ham(osec, ops["current01"]).eval(v)
            got = q.obs_eval(psi, t, [sec.lower(ops["nup0"]), sec.lower(ops["hop01"])])
            assert abs(got[0] - O.Ham(osec, ops["nup0"]).eval(v)) <= 1e-12 * abs(got[0])
            mc.incrAllObs(t)
    mc.normAll()
    assert np.allclose(mc.data["docc"], want / 3, rtol=1e-12, atol=1e-12)
    assert np.allclose(mc.data["hop"], want_hop / 3, rtol=1e-12, atol=1e-12)
    assert np.allclose(mc.data["docc_abs2"].real, want_aux / 3, rtol=1e-10)
    assert list(mc.Nmc) == [3, 3, 3]
    with pytest.raises(KeyError):
        mc.addAux("x", "nothing", abs, 1)


def test_obs_eval_rejects_a_foreign_sector(ctx):
    spec, ham = chains.hubbard_chain(4, 2, 2, 4.0, -1.0)
    spec2, ham2 = chains.hubbard_chain(4, 2, 1, 4.0, -1.0)
    sec, sec2 = q.Sector(spec.index, spec.constraints), q.Sector(spec2.index, spec2.constraints)
    psi = q.getState(sec, 1)
    psi.set(0, np.ones(sec.dim))
    with pytest.raises(A.QDError):
        q.obs_eval(psi, 0, [sec2.lower(ham2)])
