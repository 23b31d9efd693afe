"""Generate tests/golden/golden.json: known answers that pin the CPU oracle.

QuDrip ships no tests or golden vectors and cannot be compiled here (it needs
Eigen3), so the oracle is pinned by answers computed independently of it:

* closed forms: the open XY chain H = sum (S+_{i+1} S-_i + h.c.) is a
  free-fermion chain with single-particle energies 2 cos(pi k / (L + 1));
  the half-filled ground energy is the sum of the negative ones;
* dense matrices of small systems built from Kronecker products of 2x2
  matrices with explicit Jordan-Wigner strings (no tree expansion, no
  sector ranking code shared with the oracle), restricted to the sector;
* ground energies of periodic Heisenberg chains from scipy eigsh on a sparse
  matrix assembled by direct bit manipulation;
* structural counts (dim, nnz with explicit zeros) from combinatorics.

Run:  python tests/golden/make_golden.py   (takes a few minutes for L = 24)
"""
from __future__ import annotations

import json
import math
import os
import sys
from functools import reduce

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

I2 = np.eye(2, dtype=complex)
Z2 = np.diag([1.0, -1.0]).astype(complex)
# bit value b: basis |0>, |1>; raising |1><0|, lowering |0><1|
RAISE = np.array([[0, 0], [1, 0]], dtype=complex)
LOWER = np.array([[0, 1], [0, 0]], dtype=complex)
NUM = np.array([[0, 0], [0, 1]], dtype=complex)
SZ = 0.5 * np.diag([1.0, -1.0]).astype(complex)  # the gate sz/2 applied as its transpose (diagonal)


def site_op(n, site, m, jw_above=False):
    """Operator m on `site` of an n-bit register, bit 0 least significant;
    optional Jordan-Wigner string Z on every site above."""
    mats = []
    for j in range(n - 1, -1, -1):
        if j == site:
            mats.append(m)
        elif jw_above and j > site:
            mats.append(Z2)
        else:
            mats.append(I2)
    return reduce(np.kron, mats)


def sector_states(n, pred):
    return [s for s in range(1 << n) if pred(s)]


def restrict(M, states):
    idx = np.array(states)
    return M[np.ix_(idx, idx)]


def popcount(x):
    return bin(x).count("1")


def xy_dense(L, periodic=False):
    n = L
    H = np.zeros((1 << n, 1 << n), dtype=complex)
    nb = L if periodic else L - 1
    for i in range(nb):
        j = (i + 1) % L
        H += site_op(n, j, RAISE) @ site_op(n, i, LOWER)
        H += site_op(n, i, RAISE) @ site_op(n, j, LOWER)
    st = sector_states(n, lambda s: popcount(s) == L // 2)
    return restrict(H, st), st


def xxz_dense(L, Jxy, Jz, fields, periodic=True):
    n = L
    H = np.zeros((1 << n, 1 << n), dtype=complex)
    nb = L if periodic else L - 1
    for i in range(nb):
        j = (i + 1) % L
        H += 0.5 * Jxy * (site_op(n, i, RAISE) @ site_op(n, j, LOWER))
        H += 0.5 * Jxy * (site_op(n, j, RAISE) @ site_op(n, i, LOWER))
        H += Jz * (site_op(n, i, SZ) @ site_op(n, j, SZ))
    for i, h in enumerate(fields or []):
        H += h * site_op(n, i, SZ)
    st = sector_states(n, lambda s: popcount(s) == L // 2)
    return restrict(H, st), st


def fermion_c(n, j):
    """c_j with the string on the sites above j (hopBitOp / bitOp convention)."""
    return site_op(n, j, LOWER, jw_above=True)


def hubbard_dense(L, Nup, Ndo, U, thop=-1.0, periodic=False):
    n = 2 * L
    c = [fermion_c(n, j) for j in range(n)]
    cd = [m.conj().T for m in c]
    H = np.zeros((1 << n, 1 << n), dtype=complex)
    for site in range(L):
        if periodic or site != L - 1:
            for off in (0, L):
                a, b = site + off, (site + 1) % L + off
                H += thop * (cd[b] @ c[a]) + thop * (cd[a] @ c[b])
    for site in range(L):
        H += U * (cd[site] @ c[site] @ cd[site + L] @ c[site + L])
    lo = (1 << L) - 1
    st = sector_states(n, lambda s: popcount(s & lo) == Nup and popcount(s >> L) == Ndo)
    return restrict(H, st), st


def fermi_bitgate_dense(L):
    """Products of getFermiGate bit gates: sum_i (c+_{i+1} c_i + h.c.) built
    from sigma+/- bit gates with the JW string, plus a complex phase term."""
    n = L
    H = np.zeros((1 << n, 1 << n), dtype=complex)
    for i in range(L - 1):
        j = i + 1
        t = 0.7 + 0.2j
        H += t * (site_op(n, j, RAISE, True) @ site_op(n, i, LOWER, True))
        H += np.conj(t) * (site_op(n, i, RAISE, True) @ site_op(n, j, LOWER, True))
    st = sector_states(n, lambda s: popcount(s) == L // 2)
    return restrict(H, st), st


def heisenberg_e0(L):
    """Ground energy of the periodic S=1/2 Heisenberg chain in Sz = 0 via eigsh."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    from itertools import combinations
    states = np.array(sorted(sum(1 << b for b in c) for c in combinations(range(L), L // 2)),
                      dtype=np.int64)
    dim = len(states)
    rows, cols, vals = [], [], []
    diag = np.zeros(dim)
    for i in range(L):
        j = (i + 1) % L
        bi = (states >> i) & 1
        bj = (states >> j) & 1
        diag += 0.25 * np.where(bi == bj, 1.0, -1.0)
        differ = np.nonzero(bi != bj)[0]
        tgt = states[differ] ^ ((1 << i) | (1 << j))
        rows.append(np.searchsorted(states, tgt))
        cols.append(differ)
        vals.append(np.full(len(differ), 0.5))
    rows.append(np.arange(dim))
    cols.append(np.arange(dim))
    vals.append(diag)
    H = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(dim, dim))
    e = sla.eigsh(H, k=1, which="SA", tol=1e-13, maxiter=20000)[0][0]
    return float(e), dim


def xxz_nnz(L):
    """dim and stored entries of the periodic XXZ Sz=0 matrix built bond by bond:
    every row keeps its diagonal (explicit zero when the bond sum cancels)."""
    dim = math.comb(L, L // 2)
    offdiag = L * 2 * math.comb(L - 2, L // 2 - 1)
    return dim, offdiag + dim


def dense_record(M, states):
    nz = np.nonzero(np.abs(M) > 0)
    return {
        "dim": len(states),
        "states": [int(s) for s in states],
        "entries": [[int(r), int(c), float(M[r, c].real), float(M[r, c].imag)] for r, c in zip(*nz)],
        "e0": float(np.linalg.eigvalsh(M)[0]),
    }


def main(skip_large: bool = False):
    out = {"source": "tests/golden/make_golden.py (independent of the oracle)"}
    out["xy_open_closed_form"] = {
        str(L): sum(2 * math.cos(math.pi * k / (L + 1)) for k in range(1, L + 1)
                    if 2 * math.cos(math.pi * k / (L + 1)) < 0) for L in (6, 8, 10, 12, 14, 16)}
    M, st = xy_dense(6)
    out["dense_xy_L6_open"] = dense_record(M, st)
    M, st = xxz_dense(6, 1.0, 0.7, [0.3, -0.5, 1.1, 0.0, -0.2, 0.9])
    out["dense_xxz_L6_periodic_fields"] = dense_record(M, st)
    M, st = hubbard_dense(3, 2, 1, 4.0, thop=-1.0, periodic=True)
    out["dense_hubbard_L3_periodic_2up1dn"] = dense_record(M, st)
    M, st = hubbard_dense(4, 2, 2, 4.0, thop=-1.0, periodic=False)
    out["dense_hubbard_L4_open_2up2dn"] = dense_record(M, st)
    M, st = fermi_bitgate_dense(6)
    out["dense_fermi_bitgates_L6"] = dense_record(M, st)
    # two-site Hubbard at half filling: E0 = (U - sqrt(U^2 + 16 t^2)) / 2
    out["hubbard_2site_closed_form_U4"] = (4.0 - math.sqrt(16.0 + 16.0)) / 2.0
    heis = {}
    for L in (12, 16, 20) + (() if skip_large else (24,)):
        e, dim = heisenberg_e0(L)
        heis[str(L)] = {"e0": e, "dim": dim}
        print("heisenberg", L, e, file=sys.stderr)
    out["heisenberg_periodic_e0"] = heis
    out["xxz_periodic_dim_nnz"] = {str(L): list(xxz_nnz(L)) for L in (12, 14, 16, 18, 20, 22, 24)}
    out["xy_open_nnz"] = {"16": 102960}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(skip_large="--skip-large" in sys.argv)
