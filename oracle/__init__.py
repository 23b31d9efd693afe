"""CPU oracle for QuDrip's exact-diagonalization path -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker: the qudrip_gb300 product never imports it.

`qd_oracle.cpp` restates the reference algorithms (see its header for the
file:line map and for the parity status: the reference needs Eigen3, which is
absent, and has no tests or golden vectors, so parity is unpinned against the
reference itself; the oracle is checked against independent known answers in
tests/golden/).
`build()` compiles it with g++ (-ffp-contract=off, so x86-64 and aarch64 hosts
produce the same bits) into oracle/_build/libqdoracle.so.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

from qudrip_gb300 import _capi as A

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "qd_oracle.cpp")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libqdoracle.so")

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
               "-o", tmp, SRC]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_I64P = C.POINTER(C.c_int64)
_IP = C.POINTER(C.c_int)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB)
            sig = {
                "qdo_sector_create": (_P, [C.c_int, C.POINTER(A.qd_constraint), C.c_int, C.c_int]),
                "qdo_sector_dim": (C.c_int64, [_P]),
                "qdo_sector_basis": (None, [_P, C.POINTER(C.c_uint64)]),
                "qdo_sector_rank": (C.c_int64, [_P, C.c_uint64]),
                "qdo_sector_free": (None, [_P]),
                "qdo_ham_lower": (_P, [_P, C.POINTER(A.qd_term), C.c_int, C.POINTER(A.qd_gate),
                                       C.c_int, _IP]),
                "qdo_ham_dim": (C.c_int64, [_P]),
                "qdo_ham_nnz": (C.c_int64, [_P]),
                "qdo_ham_csc": (None, [_P, _I64P, C.POINTER(C.c_int32), _DP]),
                "qdo_ham_free": (None, [_P]),
                "qdo_spmv": (None, [_P, _DP, _DP]),
                "qdo_eval": (None, [_P, _DP, _DP]),
                "qdo_tridiag_eig": (C.c_int, [C.c_int, _DP, _DP, _DP, _DP]),
                "qdo_expm": (C.c_int, [C.c_int, _DP, _DP]),
                "qdo_lanczos_ground": (C.c_int, [_P, _DP, C.c_int, _DP, _DP, _IP, _DP, _DP, _IP,
                                                 _I64P, _DP]),
                "qdo_arnoldi_evolve": (C.c_int, [_P, _DP, C.c_double, C.c_int, _DP, _IP, _I64P]),
                "qdo_hermitian_lanczos_ground": (C.c_int, [_P, _DP, C.c_int, _DP, _DP, _IP, _DP,
                                                           _I64P]),
                "qdo_arnoldi_ground": (C.c_int, [_P, _DP, C.c_int, _DP, _DP, _IP, _I64P, _DP]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def as_complex(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128))


class Sector:
    def __init__(self, spec):
        arr, n = spec.constraint_array()
        self.ptr = lib().qdo_sector_create(spec.nbits, arr, n, spec.tight)
        if not self.ptr:
            raise ValueError("oracle sector: invalid arguments")
        self.dim = int(lib().qdo_sector_dim(self.ptr))

    def basis(self) -> np.ndarray:
        out = np.empty(self.dim, dtype=np.uint64)
        lib().qdo_sector_basis(self.ptr, out.ctypes.data_as(C.POINTER(C.c_uint64)))
        return out

    def rank(self, state: int) -> int:
        return int(lib().qdo_sector_rank(self.ptr, C.c_uint64(int(state))))

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().qdo_sector_free(self.ptr)
            self.ptr = None


class Ham:
    def __init__(self, sector: Sector, opsum):
        terms, nt, gates, ng = opsum.pack()
        st = C.c_int(0)
        self.ptr = lib().qdo_ham_lower(sector.ptr, terms, nt, gates, ng, C.byref(st))
        if not self.ptr:
            raise ValueError(f"oracle lowering failed: status {st.value}")
        self.dim = int(lib().qdo_ham_dim(self.ptr))
        self.nnz = int(lib().qdo_ham_nnz(self.ptr))

    def csc(self):
        colptr = np.empty(self.dim + 1, dtype=np.int64)
        rowidx = np.empty(self.nnz, dtype=np.int32)
        vals = np.empty(self.nnz, dtype=np.complex128)
        lib().qdo_ham_csc(self.ptr, colptr.ctypes.data_as(_I64P),
                          rowidx.ctypes.data_as(C.POINTER(C.c_int32)), _dp(vals))
        return colptr, rowidx, vals

    def scipy(self):
        import scipy.sparse as sp
        colptr, rowidx, vals = self.csc()
        return sp.csc_matrix((vals, rowidx, colptr), shape=(self.dim, self.dim))

    def apply(self, x) -> np.ndarray:
        x = as_complex(x)
        y = np.empty_like(x)
        lib().qdo_spmv(self.ptr, _dp(x), _dp(y))
        return y

    def eval(self, psi) -> complex:
        psi = as_complex(psi)
        out = np.zeros(2)
        lib().qdo_eval(self.ptr, _dp(psi), _dp(out))
        return complex(out[0], out[1])

    def lanczos_ground(self, psi0, kry_dim: int):
        psi0 = as_complex(psi0)
        psi = np.empty_like(psi0)
        evals = np.empty(max(kry_dim, 1))
        act = C.c_int(0)
        ritz = C.c_double(0)
        err = C.c_double(0)
        bd = C.c_int(0)
        mv = C.c_int64(0)
        energy = np.zeros(2)
        rc = lib().qdo_lanczos_ground(self.ptr, _dp(psi0), kry_dim, _dp(psi), _dp(evals),
                                      C.byref(act), C.byref(ritz), C.byref(err), C.byref(bd),
                                      C.byref(mv), _dp(energy))
        if rc != 0:
            raise RuntimeError(f"oracle lanczos failed: {rc}")
        return dict(psi=psi, evals=evals[:act.value].copy(), act_dim=act.value,
                    ritz=ritz.value, err=err.value, breakdown=bd.value, matvecs=mv.value,
                    energy=complex(energy[0], energy[1]))

    def arnoldi_evolve(self, psi, h: float, m: int):
        psi = as_complex(psi)
        out = np.empty_like(psi)
        act = C.c_int(0)
        mv = C.c_int64(0)
        rc = lib().qdo_arnoldi_evolve(self.ptr, _dp(psi), h, m, _dp(out), C.byref(act),
                                      C.byref(mv))
        if rc != 0:
            raise RuntimeError(f"oracle evolve failed: {rc}")
        return out, act.value

    def arnoldi_ground(self, psi0, steps: int):
        """Arnoldi::getSolver(...).getGroundState after `steps` Krylov steps in all."""
        psi0 = as_complex(psi0)
        psi = np.empty_like(psi0)
        evals = np.empty(steps)
        act = C.c_int(0)
        mv = C.c_int64(0)
        energy = np.zeros(2)
        rc = lib().qdo_arnoldi_ground(self.ptr, _dp(psi0), steps, _dp(psi), _dp(evals), C.byref(act),
                                      C.byref(mv), _dp(energy))
        if rc != 0:
            raise RuntimeError(f"oracle arnoldi ground state failed: {rc}")
        return dict(psi=psi, evals=evals[:act.value].copy(), act_dim=act.value, matvecs=mv.value,
                    energy=complex(energy[0], energy[1]))

    def hermitian_lanczos_ground(self, psi0, kry_dim: int):
        psi0 = as_complex(psi0)
        psi = np.empty_like(psi0)
        evals = np.empty(kry_dim + 2)
        nev = C.c_int(0)
        err = C.c_double(0)
        mv = C.c_int64(0)
        rc = lib().qdo_hermitian_lanczos_ground(self.ptr, _dp(psi0), kry_dim, _dp(psi),
                                                _dp(evals), C.byref(nev), C.byref(err),
                                                C.byref(mv))
        if rc != 0:
            raise RuntimeError(f"oracle hermitian lanczos failed: {rc}")
        return dict(psi=psi, evals=evals[:nev.value].copy(), err=err.value, matvecs=mv.value)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().qdo_ham_free(self.ptr)
            self.ptr = None


def tridiag_eig(d, e):
    d = np.ascontiguousarray(d, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    n = len(d)
    ev = np.empty(n)
    z = np.empty((n, n))  # column-major in C == row j holds eigenvector j here
    rc = lib().qdo_tridiag_eig(n, _dp(d), _dp(e if len(e) else np.zeros(1)), _dp(ev), _dp(z))
    if rc != 0:
        raise RuntimeError("tridiagonal QL did not converge")
    return ev, z.T.copy()


def expm(Amat):
    Amat = np.asfortranarray(np.asarray(Amat, dtype=np.complex128))
    n = Amat.shape[0]
    out = np.empty((n, n), dtype=np.complex128, order="F")
    rc = lib().qdo_expm(n, Amat.ctypes.data_as(_DP), out.ctypes.data_as(_DP))
    if rc != 0:
        raise RuntimeError("expm failed")
    return out


def traj_run(H: "Ham", basis, ntraj, nsteps, dt, gamma, seed, m, chan_bits, obs_pairs, psi0):
    """Trajectory ensemble restated from the reference jump loop (mean observables)."""
    L = lib()
    if not hasattr(L.qdo_traj_run, "_typed"):
        L.qdo_traj_run.restype = C.c_int
        L.qdo_traj_run.argtypes = [_P, C.POINTER(C.c_uint64), C.c_int, C.c_int, C.c_double, C.c_double,
                                   C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int,
                                   C.POINTER(C.c_int), C.POINTER(C.c_int), _DP, _DP, _I64P]
        L.qdo_traj_run._typed = True
    basis = np.ascontiguousarray(basis, dtype=np.uint64)
    cb = np.ascontiguousarray(chan_bits, dtype=np.int32)
    oa = np.ascontiguousarray([a for a, _ in obs_pairs], dtype=np.int32)
    ob = np.ascontiguousarray([b for _, b in obs_pairs], dtype=np.int32)
    psi0 = as_complex(psi0)
    out = np.zeros((nsteps + 1, len(obs_pairs)))
    jumps = C.c_int64(0)
    rc = L.qdo_traj_run(H.ptr, basis.ctypes.data_as(C.POINTER(C.c_uint64)), ntraj, nsteps, dt, gamma, seed, m,
                        len(cb), cb.ctypes.data_as(C.POINTER(C.c_int)), len(oa),
                        oa.ctypes.data_as(C.POINTER(C.c_int)), ob.ctypes.data_as(C.POINTER(C.c_int)),
                        _dp(psi0), _dp(out), C.byref(jumps))
    if rc != 0:
        raise RuntimeError("oracle trajectories failed")
    return out, jumps.value
