"""Host logic: operator algebra semantics, packing, and the C-ABI library exports."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from qudrip_gb300 import _capi as A
from qudrip_gb300 import chains
from qudrip_gb300.operators import (OperatorSum, cmul, getBoseGate, getEmptyOperator, getHopFermiGate,
                                    getNd, getNset, getNup, getNdo, getQbits, pauli_x, pauli_z)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_append_merges_identical_gate_instances():
    q = getQbits(4)
    g = getBoseGate(q)
    g << pauli_x
    op = g(1) * g(2)
    s = op + op  # operator+(Operator, Operator) appends: same instances -> one term, coeff 2
    assert s.size() == 1 and s.terms[0][1] == 2
    s2 = g(1) * g(2) + g(1) * g(2)  # new instances each call -> two terms
    assert s2.size() == 2
    s3 = (s + s)  # sum + sum concatenates without merging
    assert s3.size() == 2


def test_sum_products_and_scalars():
    q = getQbits(4)
    g = getHopFermiGate(q)
    a = g(0, 1) + g(1, 0)
    b = g(2, 2) - g(3, 3)
    p = a * b
    assert p.size() == 4
    assert [c for _, c in p.terms] == [1, -1, 1, -1]
    p2 = (0.5 + 0.25j) * p
    assert p2.terms[1][1] == cmul(-1, 0.5 + 0.25j)
    e = getEmptyOperator() + g(0, 0)
    assert e.size() == 1


def test_gate_snapshots_matrix_at_call_time():
    q = getQbits(3)
    g = getBoseGate(q)
    g << pauli_x
    op1 = g(0)
    g << pauli_z
    op2 = g(0)
    assert np.array_equal(op1.gates[0].U, pauli_x) and np.array_equal(op2.gates[0].U, pauli_z)


def test_masks_follow_reference():
    q = getQbits(8)
    # Nset(index, -1, -1) covers bits 0..popcount(range-1) inclusive: 9 bits for N=8
    assert getNset(q).terms[0][1]["mask"] == (1 << 9) - 1
    assert getNup(q, 4).terms[0][1]["mask"] == 0x0F
    assert getNdo(q, 4).terms[0][1]["mask"] == 0xF0
    nd = getNd(q, 4)
    assert nd.evaluate(0b0011_0001) == 1  # site 0 doubly occupied (bits 0 and 4)


def test_pack_layout():
    spec, ham = chains.xy_chain(4)
    terms, nt, gates, ng = ham.pack()
    assert nt == 6 and ng == 12
    assert terms[1].gate_offset == 2 and terms[1].ngates == 2
    g0 = gates[0]
    # gc << (sx + i sy)/2 = [[0,1],[0,0]]: U(0,1) = 1 -> u[2*(0*2+1)] = 1
    assert g0.kind == A.QD_GATE_BIT and g0.u[2] == 1.0 and g0.u[0] == 0.0
    arr, n = spec.constraint_array()
    assert n == 1 and arr[0].target == 2 and arr[0].term[0].mask == (1 << 5) - 1


def _declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(qd_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declarations_are_bound():
    declared = _declared_functions()
    assert len(declared) > 20
    assert set(declared) == set(A.declared_symbols())


def test_library_exports_every_declared_symbol():
    if not os.path.exists(A.LIB_PATH):
        from qudrip_gb300 import build
        build.build()
    lib = C.CDLL(A.LIB_PATH)  # loading needs no GPU
    missing = [n for n in _declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.qd_api_version() == 1


def _philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon et al., SC11), restated for the check below."""
    M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
    c = list(ctr)
    k0, k1 = key
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> 32, p0 & 0xFFFFFFFF
        hi1, lo1 = p1 >> 32, p1 & 0xFFFFFFFF
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c


def test_seeded_start_follows_the_documented_generator():
    # host-only entry point: needs the library, not a GPU
    if not os.path.exists(A.LIB_PATH):
        from qudrip_gb300 import build
        build.build()
    import qudrip_gb300 as q
    seed = 0x1234_5678_9ABC
    got = q.seeded_start(seed, 9)
    for i in range(9):
        c = _philox4x32_10([i // 2, 0x53544152, 0, 0], [seed & 0xFFFFFFFF, seed >> 32])
        words = (c[0], c[1]) if i % 2 == 0 else (c[2], c[3])
        u = ((words[0] >> 5) * 67108864.0 + (words[1] >> 6)) / 9007199254740992.0
        assert got[i] == 2.0 * u - 1.0
    assert np.all(np.abs(got) <= 1.0)
    assert not np.array_equal(q.seeded_start(seed + 1, 9), got)
