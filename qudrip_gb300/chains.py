"""Operator trees of the chains QuDrip's programs build, written with its own API.

* `xy_chain` -- programs/spin.cpp:11-36 (README example): H = sum_i
  (S+_{i+1} S-_i + S+_i S-_{i+1}) with gc << (sx + i sy)/2, ga << (sx - i sy)/2,
  in the Nset = L/2 sector.
* `xxz_chain` -- the same ladder gates plus S^z_i S^z_j built from two bit
  gates gz << sz/2 per bond (every diagonal entry is stored, explicit zeros
  included) and optional fields h_i S^z_i, in the Nset = L/2 sector.
* `hubbard_chain` -- programs/hubbard_diss.cpp:97-159: spinful fermions on 2L
  bits (up = bits 0..L-1, down = bits L..2L-1), hopping thop * c^dagger c via
  getHopFermiGate, U * n_up n_dn, sector Nup = N_up, Ndo = N_dn.

Each builder returns (SectorSpec, OperatorSum); nothing touches the device.
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple

from .operators import (II, OperatorSum, SectorSpec, getBoseGate, getEmptyOperator, getHopFermiGate,
                        getNdo, getNset, getNup, getQbits, pauli_x, pauli_y, pauli_z)


def xy_chain(L: int, periodic: bool = False) -> Tuple[SectorSpec, OperatorSum]:
    prechain = getQbits(L)
    Nset = getNset(prechain)
    gc = getBoseGate(prechain)
    ga = getBoseGate(prechain)
    spec = SectorSpec(prechain, [Nset == L // 2])
    gc << 0.5 * (pauli_x + II * pauli_y)
    ga << 0.5 * (pauli_x - II * pauli_y)
    ham = getEmptyOperator()
    nb = L if periodic else L - 1
    for i in range(nb):
        j = (i + 1) % L
        ham = ham + gc(j) * ga(i) + gc(i) * ga(j)
    return spec, ham


def xxz_chain(L: int, Jxy: float = 1.0, Jz: float = 1.0, periodic: bool = True,
              fields: Optional[Sequence[float]] = None) -> Tuple[SectorSpec, OperatorSum]:
    prechain = getQbits(L)
    Nset = getNset(prechain)
    gc = getBoseGate(prechain)
    ga = getBoseGate(prechain)
    gz = getBoseGate(prechain)
    spec = SectorSpec(prechain, [Nset == L // 2])
    gc << 0.5 * (pauli_x + II * pauli_y)
    ga << 0.5 * (pauli_x - II * pauli_y)
    gz << 0.5 * pauli_z
    ham = getEmptyOperator()
    nb = L if periodic else L - 1
    for i in range(nb):
        j = (i + 1) % L
        ham = ham + (0.5 * Jxy) * (gc(i) * ga(j)) + (0.5 * Jxy) * (gc(j) * ga(i)) + Jz * (gz(i) * gz(j))
    if fields is not None:
        for i, h in enumerate(fields):
            ham = ham + float(h) * gz(i)
    return spec, ham


def hubbard_chain(L: int, Nup: int, Ndo: int, U: float, thop: float = -1.0,
                  periodic: bool = False) -> Tuple[SectorSpec, OperatorSum]:
    fermi = getQbits(2 * L)
    nup = getNup(fermi, L)
    ndo = getNdo(fermi, L)
    spec = SectorSpec(fermi, [nup == Nup, ndo == Ndo])
    gate = getHopFermiGate(fermi)
    ham = getEmptyOperator()
    for site in range(L):
        s1u, s2u = site, (site + 1) % L
        s1d, s2d = site + L, (site + 1) % L + L
        if periodic or site != L - 1:
            ham = ham + thop * gate(s2u, s1u) + thop * gate(s1u, s2u)
            ham = ham + thop * gate(s2d, s1d) + thop * gate(s1d, s2d)
    for site in range(L):
        ham = ham + U * (gate(site, site) * gate(site + L, site + L))
    return spec, ham


def docc_operator(L: int, site: int, fermi=None) -> OperatorSum:
    """n_{site,up} n_{site,dn} (programs/hubbard_diss.cpp:412-415)."""
    fermi = fermi or getQbits(2 * L)
    gate = getHopFermiGate(fermi)
    return OperatorSum([(gate(site, site) * gate(site + L, site + L), 1.0 + 0j)])
