"""Lattices, lattice functions and bond models: the reference's lattice.hpp.

`Lattice(coords, pvecs)` holds integer site coordinates and periodicity vectors,
reduces any coordinate into the cell and finds its site index; `LatticeFunction`
is a table over sites (or tuples of sites) with the reference's Fourier sum;
`Model` keeps bonds with named parameters and emits the Hamiltonian of a bond
functor -- as an OperatorSum (`getHamiltonian`, then lowered by `>>` on the
device like any operator) or as a sum of lowered matrices
(`getHamiltonianMatrix`, device-side sums).  Everything here is host-side
bookkeeping; none of it runs on the GPU.

Behaviour follows lattice.hpp line by line where it is defined:
* `params_type` (lattice.hpp:14-52): calling it with a name returns the value,
  creating 0 first; `get` on a missing name raises "undefined params";
  `stringize` is "name=value,...;" with C++'s std::to_string formatting.  The
  reference iterates an unordered_map; here the order is insertion order.
* reciprocal vectors and cell volume (lattice.hpp:62-110): 1D rp = p,
  vol = p.p; 2D rp0 = (-p1y, p1x), rp1 = (p0y, -p0x), vol = rp0.p0; 3D cross
  products, vol = p0.(p1 x p2).
* `reduce` (lattice.hpp:163-179): for each periodicity vector in turn,
  ir = (r.rp_i) / vol with C++ integer division (toward zero), then one less
  when the product is nonzero and its sign differs from vol's, and
  r -= ir * p_i.  A product that is an exact negative multiple of vol is
  therefore shifted one period too far (to the upper edge of the cell), as in
  the reference; such a coordinate is then not found (index N).
* `DFT(k)` (lattice.hpp:269-283): (1/N) sum_i f_i exp(i theta_i) with
  theta_i = sum_j <x_i, k_j rp_j> / vol -- no factor 2 pi, as in the reference.

Where the reference's behaviour is undefined this module defines it:
* `Lattice(coords)` without periodicity vectors: the reference reads
  pvec[0..N-1] of an empty vector; here vol = 0, the reciprocal vectors are
  zero and `reduce` returns the coordinate unchanged (its own rule for no
  periodicity vectors).
* the multi-argument `DFT(ks)` (lattice.hpp:285-306) indexes ks by the table
  index and leaves the argument tuple empty; here it sums over every tuple of
  sites with the phase sum_ix sum_j <x_{a_ix}, ks_ix,j rp_j> / vol.
* `params_type.stringize()` of no parameters (the reference writes index -1):
  here "".
"""
from __future__ import annotations

import math
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np


def _cpp_to_string(v) -> str:
    """std::to_string: integers as %d, floating point as %f."""
    if isinstance(v, (bool, np.bool_)):
        return str(int(v))
    if isinstance(v, (int, np.integer)):
        return "%d" % v
    if isinstance(v, complex):
        raise TypeError("std::to_string has no complex overload")
    return "%f" % v


class params_type:
    """Named bond parameters (lattice.hpp:14-52)."""

    def __init__(self, init: Optional[Dict[str, float]] = None, default=0.0):
        self._p: Dict[str, float] = dict(init or {})
        self._default = default

    def __call__(self, name: str):
        if name not in self._p:
            self._p[name] = self._default
        return self._p[name]

    def __getitem__(self, name: str):
        return self(name)

    def __setitem__(self, name: str, value) -> None:
        self._p[name] = value

    def get(self, name: str):
        """The const accessor: a missing name is an error."""
        if name not in self._p:
            raise KeyError("undefined params")
        return self._p[name]

    def copy(self) -> "params_type":
        return params_type(self._p, self._default)

    def names(self) -> List[str]:
        return list(self._p)

    def stringize(self) -> str:
        if not self._p:
            return ""
        return ",".join(f"{k}={_cpp_to_string(v)}" for k, v in self._p.items()) + ";"

    def __str__(self) -> str:
        return self.stringize()


def _ivec(c) -> np.ndarray:
    a = np.asarray(c, dtype=np.int64).reshape(-1)
    return a


def _cdiv(a: int, b: int) -> int:
    """C++ integer division (truncation toward zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def get_reci(pvec: Sequence[Sequence[int]]) -> Tuple[List[np.ndarray], int]:
    """Reciprocal vectors (unnormalised) and the signed cell volume (lattice.hpp:62-110)."""
    p = [_ivec(v) for v in pvec]
    n = len(p)
    if n == 1:
        return [p[0].copy()], int(p[0] @ p[0])
    if n == 2:
        r0 = np.array([-p[1][1], p[1][0]], dtype=np.int64)
        r1 = np.array([p[0][1], -p[0][0]], dtype=np.int64)
        return [r0, r1], int(r0 @ p[0])
    if n == 3:
        r0, r1, r2 = np.cross(p[1], p[2]), np.cross(p[2], p[0]), np.cross(p[0], p[1])
        return [r0.astype(np.int64), r1.astype(np.int64), r2.astype(np.int64)], int(p[0] @ np.cross(p[1], p[2]))
    raise ValueError("lattices of 1, 2 or 3 dimensions")


class Lattice:
    """Sites with integer coordinates and optional periodicity (lattice.hpp:114-198)."""

    def __init__(self, coords: Sequence[Sequence[int]], pvecs: Optional[Sequence[Sequence[int]]] = None):
        self.coords = [_ivec(c) for c in coords]
        if not self.coords:
            raise ValueError("a lattice needs at least one site")
        self.ndim = len(self.coords[0])
        self.pvecs = [_ivec(v) for v in (pvecs or [])]
        if self.pvecs:
            if len(self.pvecs) != self.ndim:
                raise ValueError("one periodicity vector per dimension")
            self.rpvecs, self._vol = get_reci(self.pvecs)
        else:
            self.rpvecs, self._vol = [np.zeros(self.ndim, dtype=np.int64) for _ in range(self.ndim)], 0
        if any((c < 0).any() for c in self.coords):
            print("Warning: non-positive coordinates are invalid for periodicity reduction.")
        self._index = {tuple(int(x) for x in c): i for i, c in reversed(list(enumerate(self.coords)))}

    def N(self) -> int:
        return len(self.coords)

    def vol(self) -> int:
        return self._vol

    def reduce(self, c) -> np.ndarray:
        r = _ivec(c).copy()
        if not self.pvecs:
            return r
        for i in range(self.ndim):
            prod = int(r @ self.rpvecs[i])
            ir = _cdiv(prod, self._vol)
            if prod != 0 and ((prod < 0) != (self._vol < 0)):
                ir -= 1
            r = r - ir * self.pvecs[i]
        return r

    def index(self, c) -> int:
        return self._index.get(tuple(int(x) for x in _ivec(c)), self.N())

    def __call__(self, arg):
        """lat(i) -> coordinate of site i; lat(coord) -> site index of the reduced coordinate (N if none)."""
        if isinstance(arg, (int, np.integer)):
            if not 0 <= arg < self.N():
                raise IndexError("site index out of range")
            return self.coords[int(arg)]
        return self.index(self.reduce(arg))

    def pvec(self, i: int) -> np.ndarray:
        return self.pvecs[i]

    def rpvec(self, i: int) -> np.ndarray:
        return self.rpvecs[i]


class LatticeFunction:
    """A table over sites or tuples of sites (lattice.hpp:202-308)."""

    def __init__(self, latt: Lattice, argn: int = 1, dtype=np.complex128):
        self.latt = latt
        self.argn = argn
        self.data = np.zeros(latt.N() ** argn, dtype=dtype)

    def _idx(self, arg) -> int:
        if isinstance(arg, (int, np.integer)):
            if self.argn != 1:
                raise ValueError("a single index needs a one-argument function")
            return int(arg)
        idx = 0
        for a in arg:
            idx = idx * self.latt.N() + int(a)
        return idx

    def __getitem__(self, arg):
        return self.data[self._idx(arg)]

    def __setitem__(self, arg, value) -> None:
        self.data[self._idx(arg)] = value

    def _phase(self, x: np.ndarray, k) -> float:
        L = self.latt
        arg = 0.0
        for j in range(L.ndim):
            arg += float(int(x @ (int(k[j]) * L.rpvecs[j]))) / float(L.vol())
        return arg

    def DFT(self, k) -> complex:
        """(1/N) sum_i f_i exp(i theta_i), theta_i = sum_j <x_i, k_j rp_j> / vol (one argument)."""
        if self.argn != 1:
            raise ValueError("DFT(k) is for one-argument functions")
        L = self.latt
        res = 0j
        for i in range(L.N()):
            th = self._phase(L.coords[i], _ivec(k))
            res += complex(self.data[i]) * complex(math.cos(th), math.sin(th))
        return res / L.N()

    def DFT_multi(self, ks: Sequence[Sequence[int]]) -> complex:
        """Fourier sum over every tuple of sites, one momentum per argument."""
        if len(ks) != self.argn:
            raise ValueError("one momentum per argument")
        L = self.latt
        n = L.N()
        res = 0j
        for idx in range(self.data.size):
            args, rem = [], idx
            for _ in range(self.argn):
                args.append(rem % n)
                rem //= n
            args.reverse()
            th = sum(self._phase(L.coords[a], _ivec(ks[ix])) for ix, a in enumerate(args))
            res += complex(self.data[idx]) * complex(math.cos(th), math.sin(th))
        return res / self.data.size


class Model:
    """Bonds of a lattice with their parameters (lattice.hpp:310-385)."""

    def __init__(self, latt: Lattice):
        self.latt = latt
        self.bonds: List[Tuple[int, int]] = []
        self.params: List[params_type] = []

    def addBond(self, s1: int, s2: int, param: params_type) -> None:
        if not (0 <= s1 < self.latt.N() and 0 <= s2 < self.latt.N()):
            raise IndexError("bond site outside the lattice")
        self.bonds.append((int(s1), int(s2)))
        self.params.append(param.copy())

    def describe(self) -> str:
        """The text print() writes (for 3D the reference repeats the second coordinate; so does this)."""
        lines = ["Bonds: "]
        for (a, b), p in zip(self.bonds, self.params):
            c1, c2 = self.latt(a), self.latt(b)
            t1 = "(" + str(int(c1[0])) + "".join("," + str(int(c1[1])) for _ in range(1, len(c1)))
            t2 = "(" + str(int(c2[0])) + "".join("," + str(int(c2[1])) for _ in range(1, len(c1)))
            lines.append(t1 + ") and " + t2 + "): " + p.stringize())
        return "\n".join(lines) + "\n"

    def print(self) -> None:
        print(self.describe(), end="")

    def getHamiltonian(self, f: Callable):
        """Sum over bonds of f(s1, s2, param), starting from getEmptyOperator()."""
        from .operators import getEmptyOperator
        ham = getEmptyOperator()
        for (a, b), p in zip(self.bonds, self.params):
            ham = ham + f(a, b, p)
        return ham

    def getHamiltonianMatrix(self, f: Callable, sector):
        """Sum over bonds of the lowered matrices f(s1, s2, param), starting from the
        empty matrix of `sector` (the reference's SpMatrix(ndim, ndim))."""
        from .engine import Hamiltonian
        ham = Hamiltonian.zero(sector)
        for (a, b), p in zip(self.bonds, self.params):
            ham = ham + f(a, b, p)
        return ham
