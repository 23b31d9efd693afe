"""Generate tests/golden/traj_ensemble_L8.json: an FP64 jump-trajectory ensemble of the oracle.

The dissipative Hubbard chain of the trajectory workload: L = 8 sites,
spinful fermions (up = bits 0..7, down = bits 8..15), N_up = N_dn = 4
(dim 4,900), hopping t = 1 (thop = -1), U = 4, open boundary; jump operators
sqrt(gamma) n_{i,s} on all 16 site-spins with gamma = 0.1; steps dt = 0.01 to
T = 10 (1,000 steps) with the reference's Arnoldi exponential of m = 30
vectors (programs/hubbard_diss.cpp:439-482, sparse_algorithm.hpp:548-562, as
restated by oracle/qd_oracle.cpp); the initial state is the ground state of
the Hermitian part (scipy eigsh, tol 1e-13), as the reference program starts
from the ground state (programs/hubbard_diss.cpp:382-384).

NTRAJ independent trajectories, trajectory k drawing its decisions from
Philox4x32-10 with seed SEED0 + k, run in parallel over the host cores.  The
file holds, every RECORD steps, the mean and the standard error over the
trajectories of <n_{i,up} n_{i,dn}> for i = 0..7, plus the settings.

Run:  python tests/golden/make_traj_ensemble.py   (a few minutes on 8 cores)
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

L, NUP, NDO, U, THOP = 8, 4, 4, 4.0, -1.0
GAMMA, DT, NSTEPS, M = 0.1, 0.01, 1000, 30
NTRAJ, SEED0, RECORD = 1024, 1_000_000, 10


def system():
    from qudrip_gb300 import chains
    from qudrip_gb300.operators import getHopFermiGate
    spec, ham = chains.hubbard_chain(L, NUP, NDO, U, THOP)
    gate = getHopFermiGate(spec.index)
    heff = ham
    for s in range(2 * L):
        heff = heff + (-0.5j * GAMMA) * gate(s, s)
    chan = list(range(2 * L))
    obs = [(i, i + L) for i in range(L)]
    return spec, ham, heff, chan, obs


def ground_state(spec, ham):
    import scipy.sparse.linalg as sla
    import oracle as O
    H = O.Ham(O.Sector(spec), ham).scipy().tocsr()
    assert np.all(H.data.imag == 0)
    w, v = sla.eigsh(H.real, k=1, which="SA", tol=1e-13)
    psi0 = v[:, 0].astype(np.complex128)
    return psi0 / np.linalg.norm(psi0), float(w[0])


def main():
    import oracle as O
    spec, ham, heff, chan, obs = system()
    psi0, e0 = ground_state(spec, ham)
    osec = O.Sector(spec)
    oh = O.Ham(osec, heff)
    basis = osec.basis()

    def one(k):
        out, jumps = O.traj_run(oh, basis, 1, NSTEPS, DT, GAMMA, SEED0 + k, M, chan, obs, psi0)
        return out, jumps

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        res = list(ex.map(one, range(NTRAJ)))
    vals = np.stack([r[0] for r in res])  # NTRAJ x (NSTEPS + 1) x 8
    jumps = int(sum(r[1] for r in res))
    rows = list(range(0, NSTEPS + 1, RECORD))
    sel = vals[:, rows, :]
    mean = sel.mean(axis=0)
    stderr = sel.std(axis=0, ddof=1) / np.sqrt(NTRAJ)
    out = {
        "source": "tests/golden/make_traj_ensemble.py (oracle/qd_oracle.cpp FP64 jump loop)",
        "L": L, "Nup": NUP, "Ndo": NDO, "U": U, "thop": THOP, "gamma": GAMMA, "dt": DT,
        "nsteps": NSTEPS, "m": M, "ntraj": NTRAJ, "seed0": SEED0, "record_every": RECORD,
        "channels": chan, "observables": obs, "ground_energy": e0, "jumps": jumps,
        "steps": rows, "mean": mean.tolist(), "stderr": stderr.tolist(),
    }
    path = os.path.join(HERE, "traj_ensemble_L8.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(f"wrote {path}: {NTRAJ} trajectories, {jumps} jumps, <n_up n_dn>(T) = {mean[-1].mean():.5f}")


if __name__ == "__main__":
    main()
