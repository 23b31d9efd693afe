"""Host-side operator algebra with QuDrip's semantics.

Mirrors the reference's lazily built operator trees:
  * gates -- bitOp (operators/bit.hpp:7-45) and hopBitOp (operators/hopbit.hpp:7-40);
    `gate << U` stores U as given and a call `gate(i)` snapshots it into a
    new gate instance (make_shared copy, operators/bit.hpp:17-21);
  * Operator -- an ordered product of gate instances (operator.hpp:68-132);
  * OperatorSum -- a list of (Operator, complex coefficient) with QuDrip's
    append rule: a product whose gate instances are the very same objects as
    an existing term's only adds to that coefficient (operator_abel.hpp:115-127);
    `sum + sum` and `sum - sum` concatenate without merging.
  * conserved quantities -- Nset masks and Nd doublon/holon counts
    (conservation.hpp:89-157, 233-256).

Nothing here touches the GPU; `pack()` produces the qd_term / qd_gate arrays
the C ABI lowers (`ham >> chain`).  Coefficient products are evaluated as
separate rounded float operations, the same sequence std::complex<double>
uses, so the packed coefficients are identical on every host.
"""
from __future__ import annotations

import ctypes as C
import itertools
from typing import List, Sequence, Tuple

import numpy as np

from . import _capi as A

II = 1j
pauli_x = np.array([[0, 1], [1, 0]], dtype=complex)
pauli_y = np.array([[0, -1j], [1j, 0]], dtype=complex)
pauli_z = np.array([[1, 0], [0, -1]], dtype=complex)
id = np.array([[1, 0], [0, 1]], dtype=complex)  # noqa: A001  (reference name)

BIT_LIMIT = 64


def cmul(a: complex, b: complex) -> complex:
    """(a.r*b.r - a.i*b.i, a.r*b.i + a.i*b.r), one rounding per operation."""
    a = complex(a)
    b = complex(b)
    rr = a.real * b.real
    rr = rr - a.imag * b.imag
    ri = a.real * b.imag
    ri = ri + a.imag * b.real
    return complex(rr, ri)


def cadd(a: complex, b: complex) -> complex:
    a = complex(a)
    b = complex(b)
    return complex(a.real + b.real, a.imag + b.imag)


# ----------------------------------------------------------------- indices
class QbitsIndex:
    """getQbits(N): the full space of N bits, range 2^N (index.hpp:80-94)."""

    def __init__(self, nbits: int):
        if not (1 <= nbits <= 62):
            raise ValueError("nbits must be in 1..62")
        self.nbits = int(nbits)

    def range(self) -> int:
        return 1 << self.nbits


def getQbits(N: int) -> QbitsIndex:
    return QbitsIndex(N)


# ----------------------------------------------------------------- conserved quantities
class Quantity:
    """A conserved quantity or an integer combination of them (CQContainer)."""

    def __init__(self, index: QbitsIndex, terms: List[Tuple[int, dict]]):
        self.index = index
        self.terms = terms  # list of (coef, spec dict)

    def __add__(self, other: "Quantity") -> "Quantity":
        return Quantity(self.index, self.terms + other.terms)

    def __sub__(self, other: "Quantity") -> "Quantity":
        return Quantity(self.index, self.terms + [(-c, s) for c, s in other.terms])

    def __eq__(self, value):  # `cq = v` inside Constrain(...)
        return Constraint(self, int(value))

    def assign(self, value: int) -> "Constraint":
        return Constraint(self, int(value))

    __hash__ = object.__hash__

    def evaluate(self, state: int) -> int:
        q = 0
        for coef, s in self.terms:
            if s["kind"] == A.QD_CQ_NSET:
                q += coef * bin(state & s["mask"]).count("1")
            else:
                ns = s["nsite"]
                m = ((1 << ns) - 1) if s["hole"] else 0
                q += coef * bin(((state >> ns) ^ m) & (state ^ m)).count("1")
        return q


class Constraint:
    def __init__(self, quantity: Quantity, target: int):
        if len(quantity.terms) > 4:
            raise ValueError("a constraint combines at most 4 quantities")
        self.quantity = quantity
        self.target = target

    def to_struct(self) -> A.qd_constraint:
        c = A.qd_constraint()
        c.nterms = len(self.quantity.terms)
        c.target = self.target
        for k, (coef, s) in enumerate(self.quantity.terms):
            t = c.term[k]
            t.kind = s["kind"]
            t.coef = coef
            t.mask = s.get("mask", 0)
            t.nsite = s.get("nsite", 0)
            t.hole = s.get("hole", 0)
        return c


def _mask(lo: int, hi_inclusive: int) -> int:
    m = 0
    for i in range(lo, hi_inclusive + 1):
        if i < BIT_LIMIT:
            m |= 1 << i
    return m


def getNset(index: QbitsIndex) -> Quantity:
    # Nset(index, -1, -1): bits 0 .. popcount(range-1) inclusive (conservation.hpp:417-422)
    end = bin(index.range() - 1).count("1")
    return Quantity(index, [(1, {"kind": A.QD_CQ_NSET, "mask": _mask(0, end)})])


def getNup(index: QbitsIndex, Nsite: int) -> Quantity:
    return Quantity(index, [(1, {"kind": A.QD_CQ_NSET, "mask": _mask(0, Nsite - 1)})])


def getNdo(index: QbitsIndex, Nsite: int) -> Quantity:
    return Quantity(index, [(1, {"kind": A.QD_CQ_NSET, "mask": _mask(Nsite, 2 * Nsite - 1)})])


def getNd(index: QbitsIndex, Nsite: int) -> Quantity:
    return Quantity(index, [(1, {"kind": A.QD_CQ_ND, "nsite": Nsite, "hole": 0})])


def getNh(index: QbitsIndex, Nsite: int) -> Quantity:
    return Quantity(index, [(1, {"kind": A.QD_CQ_ND, "nsite": Nsite, "hole": 1})])


class SectorSpec:
    """What Constrain(index, cq = v, ...) describes, before it is built on a device."""

    def __init__(self, index: QbitsIndex, constraints: Sequence[Constraint], tight: int = 0):
        self.index = index
        self.nbits = index.nbits
        self.constraints = list(constraints)
        self.tight = int(tight)

    def constraint_array(self):
        n = len(self.constraints)
        arr = (A.qd_constraint * max(n, 1))()
        for i, c in enumerate(self.constraints):
            arr[i] = c.to_struct()
        return arr, n

    def accepts(self, state: int) -> bool:
        return all(abs(c.quantity.evaluate(state) - c.target) <= self.tight
                   for c in self.constraints)


# ----------------------------------------------------------------- gates
_uid = itertools.count(1)


class GateInstance:
    __slots__ = ("uid", "kind", "site", "site_b", "string", "U")

    def __init__(self, kind, site, site_b, string, U):
        self.uid = next(_uid)
        self.kind = kind
        self.site = site
        self.site_b = site_b
        self.string = string
        self.U = U

    def to_struct(self) -> A.qd_gate:
        g = A.qd_gate()
        g.kind = self.kind
        g.site = self.site
        g.site_b = self.site_b
        g.string = self.string
        if self.kind == A.QD_GATE_BIT:
            for i in range(2):
                for j in range(2):
                    g.u[2 * (2 * i + j)] = float(self.U[i, j].real)
                    g.u[2 * (2 * i + j) + 1] = float(self.U[i, j].imag)
        return g


class BitGate:
    """bitOp: a single-site 2x2 gate; string -1 adds the Jordan-Wigner sign."""

    def __init__(self, index: QbitsIndex, string: int):
        self.index = index
        self.string = int(string)
        self.U = np.zeros((2, 2), dtype=complex)

    def __lshift__(self, U):
        U = np.asarray(U, dtype=complex)
        if U.shape != (2, 2):
            raise ValueError("bit gates take a 2x2 matrix")
        self.U = U.copy()
        return self

    def __call__(self, site: int) -> "Operator":
        if not (0 <= site < self.index.nbits):
            raise ValueError("site out of range")
        return Operator([GateInstance(A.QD_GATE_BIT, int(site), 0, self.string, self.U.copy())])


class HopGate:
    """hopBitOp: gate(a, b) = c^dagger_a c_b (with JW signs), gate(a, a) = n_a."""

    def __init__(self, index: QbitsIndex, string: int):
        self.index = index
        self.string = int(string)

    def __call__(self, a: int, b: int) -> "Operator":
        n = self.index.nbits
        if not (0 <= a < n and 0 <= b < n):
            raise ValueError("site out of range")
        return Operator([GateInstance(A.QD_GATE_HOP, int(a), int(b), self.string, None)])


def getBoseGate(index: QbitsIndex) -> BitGate:
    return BitGate(index, 1)


def getFermiGate(index: QbitsIndex) -> BitGate:
    return BitGate(index, -1)


def getHopFermiGate(index: QbitsIndex) -> HopGate:
    return HopGate(index, -1)


def getHopBoseGate(index: QbitsIndex) -> HopGate:
    return HopGate(index, 1)


# ----------------------------------------------------------------- operators
def _is_scalar(x) -> bool:
    return isinstance(x, (int, float, complex, np.number))


class Operator:
    def __init__(self, gates: List[GateInstance]):
        self.gates = list(gates)

    def same(self, other: "Operator") -> bool:  # Operator::operator== (pointer identity)
        return len(self.gates) == len(other.gates) and all(
            a is b for a, b in zip(self.gates, other.gates))

    def __mul__(self, other):
        if isinstance(other, Operator):
            return Operator(self.gates + other.gates)
        if isinstance(other, OperatorSum):
            return OperatorSum([(self, 1.0 + 0j)]) * other
        if _is_scalar(other):
            return OperatorSum([(self, complex(other))])
        return NotImplemented

    def __rmul__(self, other):
        if _is_scalar(other):
            return OperatorSum([(self, complex(other))])
        return NotImplemented

    def __add__(self, other):
        if isinstance(other, Operator):
            return OperatorSum([(self, 1.0 + 0j)]).append(other, 1.0 + 0j)
        if isinstance(other, OperatorSum):
            return OperatorSum([(self, 1.0 + 0j)]) + other
        return NotImplemented

    def __sub__(self, other):
        if isinstance(other, Operator):
            return OperatorSum([(self, 1.0 + 0j)]).append(other, -1.0 + 0j)
        if isinstance(other, OperatorSum):
            return OperatorSum([(self, 1.0 + 0j)]) - other
        return NotImplemented

    def __neg__(self):
        return OperatorSum([(self, -1.0 + 0j)])

    def __rshift__(self, sector):
        return OperatorSum([(self, 1.0 + 0j)]) >> sector


class OperatorSum:
    def __init__(self, terms=None):
        self.terms: List[Tuple[Operator, complex]] = list(terms or [])

    def size(self) -> int:
        return len(self.terms)

    def copy(self) -> "OperatorSum":
        return OperatorSum(list(self.terms))

    def append(self, op: Operator, coeff) -> "OperatorSum":
        for i, (o, c) in enumerate(self.terms):
            if o.same(op):
                self.terms[i] = (o, cadd(c, coeff))
                return self
        self.terms.append((op, complex(coeff)))
        return self

    def __add__(self, other):
        if isinstance(other, Operator):
            return self.copy().append(other, 1.0 + 0j)
        if isinstance(other, OperatorSum):
            return OperatorSum(self.terms + other.terms)
        return NotImplemented

    def __sub__(self, other):
        if isinstance(other, Operator):
            return self.copy().append(other, -1.0 + 0j)
        if isinstance(other, OperatorSum):
            return OperatorSum(self.terms + [(o, complex(-c.real, -c.imag)) for o, c in other.terms])
        return NotImplemented

    def __neg__(self):
        return OperatorSum([(o, complex(-c.real, -c.imag)) for o, c in self.terms])

    def __mul__(self, other):
        if isinstance(other, Operator):
            return OperatorSum([(o * other, c) for o, c in self.terms])
        if isinstance(other, OperatorSum):
            out = OperatorSum()
            for o1, c1 in self.terms:
                for o2, c2 in other.terms:
                    out.append(o1 * o2, cmul(c1, c2))
            return out
        if _is_scalar(other):
            return OperatorSum([(o, cmul(c, other)) for o, c in self.terms])
        return NotImplemented

    def __rmul__(self, other):
        if _is_scalar(other):
            return OperatorSum([(o, cmul(c, other)) for o, c in self.terms])
        return NotImplemented

    def __truediv__(self, other):
        if _is_scalar(other):
            other = complex(other)
            return OperatorSum([(o, c / other) for o, c in self.terms])
        return NotImplemented

    def pack(self):
        """(terms array, nterms, gates array, ngates) for qd_ham_lower."""
        nt = len(self.terms)
        ng = sum(len(o.gates) for o, _ in self.terms)
        terms = (A.qd_term * max(nt, 1))()
        gates = (A.qd_gate * max(ng, 1))()
        off = 0
        for i, (o, c) in enumerate(self.terms):
            terms[i].coeff_re = c.real
            terms[i].coeff_im = c.imag
            terms[i].gate_offset = off
            terms[i].ngates = len(o.gates)
            for g in o.gates:
                gates[off] = g.to_struct()
                off += 1
        return terms, nt, gates, ng

    def __rshift__(self, sector):
        return sector.lower(self)


def getEmptyOperator() -> OperatorSum:
    return OperatorSum()
