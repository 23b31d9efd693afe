"""Device objects behind QuDrip's API: sectors, lowered Hamiltonians, states, solvers.

Every call goes through the C ABI (include/qudrip_gb300.h) into the CUDA
library; nothing here computes on the CPU.  Names follow the reference:
`Constrain` (conservation.hpp:234-239), `ham >> chain` (operator_abel.hpp:25-34),
`getState` / `psi(t)` / `psi.eval` (state.hpp:67-102, 33-45),
`Arnoldi.getLanczosSolver(...).getGroundState` (sparse_algorithm.hpp:564-604).
"""
from __future__ import annotations

import ctypes as C
import atexit
import threading
from typing import Optional

import numpy as np

from . import _capi as A
from .operators import OperatorSum, Operator, QbitsIndex, SectorSpec, Constraint


class Context:
    """One CUDA stream on one device (qd_ctx)."""

    def __init__(self, device: int = 0):
        self.handle = C.c_void_p()
        A.call("qd_ctx_create", device, C.byref(self.handle))
        self.device = device

    def sync(self):
        A.call("qd_ctx_sync", self.handle)

    def launches(self) -> int:
        n = C.c_int64(0)
        A.call("qd_ctx_launch_count", self.handle, C.byref(n))
        return n.value

    def stream(self) -> int:
        s = C.c_void_p()
        A.call("qd_ctx_stream", self.handle, C.byref(s))
        return s.value or 0

    def close(self):
        if self.handle and not _SHUTDOWN[0]:
            A.lib().qd_ctx_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None
# At interpreter exit the handles are left to the process teardown: Python may
# finalise a context before the objects made from it.
_SHUTDOWN = [False]
atexit.register(lambda: _SHUTDOWN.__setitem__(0, True))
_default_lock = threading.Lock()


def default_context() -> Context:
    global _default
    with _default_lock:
        if _default is None:
            _default = Context(0)
    return _default


class Sector(SectorSpec):
    """Constrained sector (SubIndex) built on the device."""

    def __init__(self, index: QbitsIndex, constraints, tight: int = 0, ctx: Optional[Context] = None):
        super().__init__(index, constraints, tight)
        self.ctx = ctx or default_context()
        arr, n = self.constraint_array()
        self.handle = C.c_void_p()
        A.call("qd_sector_create", self.ctx.handle, self.nbits, arr, n, self.tight, C.byref(self.handle))
        d = C.c_int64(0)
        A.call("qd_sector_dim", self.handle, C.byref(d))
        self.dim = d.value

    def range(self) -> int:
        return self.dim

    def rank_kind(self) -> int:
        k = C.c_int(0)
        A.call("qd_sector_rank_kind", self.handle, C.byref(k))
        return k.value

    def basis(self) -> np.ndarray:
        out = np.empty(self.dim, dtype=np.uint64)
        A.call("qd_sector_basis", self.handle, out.ctypes.data_as(C.POINTER(C.c_uint64)))
        return out

    def rank(self, states) -> np.ndarray:
        s = np.ascontiguousarray(states, dtype=np.uint64)
        r = np.empty(len(s), dtype=np.int64)
        A.call("qd_sector_rank", self.handle, s.ctypes.data_as(C.POINTER(C.c_uint64)), len(s),
               r.ctypes.data_as(C.POINTER(C.c_int64)))
        return r

    def lower(self, opsum) -> "Hamiltonian":
        if isinstance(opsum, Operator):
            opsum = OperatorSum([(opsum, 1.0 + 0j)])
        return Hamiltonian(self, opsum)

    def close(self):
        if getattr(self, "handle", None) and not _SHUTDOWN[0]:
            A.lib().qd_sector_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def Constrain(index: QbitsIndex, *constraints: Constraint, ctx: Optional[Context] = None) -> Sector:
    return Sector(index, constraints, 0, ctx)


def LooseConstrain(index: QbitsIndex, tight: int, *constraints: Constraint,
                   ctx: Optional[Context] = None) -> Sector:
    return Sector(index, constraints, tight, ctx)


class Hamiltonian:
    """A lowered OperatorSum (qd_ham): CSR on the device, reference CSC on demand.

    `a + b` is the reference's SpMatrix sum (union pattern, values added, explicit
    zeros kept: qd_ham_add), `s * a` a scaled copy and `a.scale(s)` scales in place
    (qd_ham_scale); Hamiltonian.zero(sector) is the empty matrix SpMatrix(n, n)."""

    def __init__(self, sector: Sector, opsum: Optional[OperatorSum] = None, handle=None):
        self.sector = sector
        self.ctx = sector.ctx
        self.handle = C.c_void_p()
        if handle is not None:
            self.handle = handle
        else:
            terms, nt, gates, ng = (opsum or OperatorSum([])).pack()
            A.call("qd_ham_lower", sector.handle, terms, nt, gates, ng, C.byref(self.handle))
        self._refresh()

    def _refresh(self):
        info = A.qd_ham_info()
        A.call("qd_ham_get_info", self.handle, C.byref(info))
        self.dim = info.dim
        self.nnz = info.nnz
        self.flags = info.flags
        self.max_row_nnz = info.max_row_nnz

    @staticmethod
    def zero(sector: Sector) -> "Hamiltonian":
        return Hamiltonian(sector, OperatorSum([]))

    def __add__(self, other: "Hamiltonian") -> "Hamiltonian":
        if not isinstance(other, Hamiltonian):
            return NotImplemented
        h = C.c_void_p()
        A.call("qd_ham_add", self.handle, other.handle, C.byref(h))
        return Hamiltonian(self.sector, handle=h)

    def copy(self) -> "Hamiltonian":
        h = C.c_void_p()
        A.call("qd_ham_copy", self.handle, C.byref(h))
        return Hamiltonian(self.sector, handle=h)

    def scale(self, s) -> "Hamiltonian":
        s = complex(s)
        A.call("qd_ham_scale", self.handle, s.real, s.imag)
        self._refresh()
        return self

    def __mul__(self, s) -> "Hamiltonian":
        if isinstance(s, Hamiltonian):
            return NotImplemented
        return self.copy().scale(s)

    __rmul__ = __mul__

    @property
    def is_real(self) -> bool:
        return bool(self.flags & A.QD_HAM_REAL)

    @property
    def is_hermitian(self) -> bool:
        return bool(self.flags & A.QD_HAM_HERMITIAN)

    def rows(self) -> int:
        return self.dim

    def cols(self) -> int:
        return self.dim

    def _download(self, name):
        ptr = np.empty(self.dim + 1, dtype=np.int64)
        idx = np.empty(max(self.nnz, 1), dtype=np.int32)
        vals = np.empty(max(self.nnz, 1), dtype=np.complex128)
        A.call(name, self.handle, ptr.ctypes.data_as(C.POINTER(C.c_int64)),
               idx.ctypes.data_as(C.POINTER(C.c_int32)), vals.ctypes.data_as(C.POINTER(C.c_double)))
        return ptr, idx[:self.nnz], vals[:self.nnz]

    def csr(self):
        return self._download("qd_ham_download_csr")

    def csc(self):
        return self._download("qd_ham_download_csc")

    def scipy(self):
        import scipy.sparse as sp
        ptr, idx, vals = self.csr()
        return sp.csr_matrix((vals, idx, ptr), shape=(self.dim, self.dim))

    def close(self):
        if getattr(self, "handle", None) and not _SHUTDOWN[0]:
            A.lib().qd_ham_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class State:
    """getState(index, nt): nt complex128 columns on the device (state.hpp:9-104)."""

    def __init__(self, sector: Sector, nt: int):
        self.sector = sector
        self.ctx = sector.ctx
        self.dim = sector.dim
        self._nt = nt
        self.t = 0
        self.handle = C.c_void_p()
        A.call("qd_state_create", self.ctx.handle, self.dim, nt, C.byref(self.handle))

    def nt(self) -> int:
        return self._nt

    def ndim(self) -> int:
        return self.dim

    def __call__(self, t: int) -> "State":  # psi(t) selects the column, returns the state
        if not 0 <= t < self._nt:
            raise IndexError("time slot out of range")
        self.t = t
        return self

    def set(self, t: int, values) -> None:
        v = np.ascontiguousarray(np.asarray(values, dtype=np.complex128))
        if v.shape != (self.dim,):
            raise ValueError("state column has the wrong length")
        A.call("qd_state_upload", self.handle, t, v.ctypes.data_as(C.POINTER(C.c_double)))

    def get(self, t: Optional[int] = None) -> np.ndarray:
        t = self.t if t is None else t
        out = np.empty(self.dim, dtype=np.complex128)
        A.call("qd_state_download", self.handle, t, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def mat(self) -> np.ndarray:
        return self.get(self.t)

    def device_ptr(self, t: int) -> int:
        p = C.c_void_p()
        A.call("qd_state_device_ptr", self.handle, t, C.byref(p))
        return p.value

    def eval(self, t: int, ham: Hamiltonian) -> complex:
        out = (C.c_double * 2)()
        A.call("qd_state_eval", self.handle, t, ham.handle, out)
        return complex(out[0], out[1])

    def close(self):
        if getattr(self, "handle", None) and not _SHUTDOWN[0]:
            A.lib().qd_state_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def getState(index: Sector, nt: int) -> State:
    return State(index, nt)


def apply(ham: Hamiltonian, x: State, t_in: int, y: State, t_out: int, matrix_free: bool = False) -> None:
    """y(t_out) = H x(t_in) through the CSR form, or the matrix-free form."""
    name = "qd_ham_apply_matrix_free" if matrix_free else "qd_ham_apply"
    A.call(name, ham.handle, x.handle, t_in, y.handle, t_out)


def start_vector(dim: int, seed: int) -> np.ndarray:
    """Seeded i.i.d. uniform[-1, 1] real start vector (the harness's shuffle_state)."""
    return np.random.Generator(np.random.PCG64(seed)).uniform(-1.0, 1.0, dim)


def shuffle_state(psi: State, seed: int = 12345) -> None:
    v = start_vector(psi.dim, seed)
    v = v / np.sqrt(np.dot(v, v))
    psi.set(psi.t, v.astype(np.complex128))


class LanczosSolver:
    """Arnoldi::getLanczosSolver(index, kry_dim) -- ArnoldiSolver<T, herm=1>.

    As the reference solver, it keeps its Krylov space between calls: the
    first getGroundState(H, psi, tstp, add_dim) starts from psi(tstp) and runs
    add_dim steps (all kry_dim steps for add_dim = -1); later calls continue
    the same space by add_dim more steps (qd_lanczos_extend) until kry_dim, and
    once it is full they return at once.  error() is the change of the lowest
    N eigenvalues since the previous call, N and the initial values set by
    convergeEV(N, iv) (sparse_algorithm.hpp:494-500, 564-585)."""

    def __init__(self, index: Sector, kry_dim: int, spmv: int = A.QD_SPMV_CSR,
                 ritz: int = A.QD_RITZ_STORED_BASIS):
        self.index = index
        self.kry_dim = kry_dim
        self.spmv = spmv
        self.ritz = ritz
        self._evals = np.empty(0)
        self._act = 0
        self._err = 0.0
        self._evs = np.zeros(1)
        self.result = None

    def convergeEV(self, N: int, iv: float = 0.0) -> None:
        if not N < self.kry_dim:
            raise ValueError("convergeEV: N must be below kry_dim")
        self._evs = np.full(N, float(iv))

    def getGroundState(self, H: Hamiltonian, psi: State, tstp: int, add_dim: int = -1):
        if self._act >= self.kry_dim:
            return self.result
        opts = A.qd_lanczos_opts(self.kry_dim, self.spmv, self.ritz, add_dim if add_dim > 0 else 0)
        evals = np.empty(self.kry_dim, dtype=np.float64)
        res = A.qd_lanczos_result()
        name = "qd_lanczos_ground" if self._act == 0 else "qd_lanczos_extend"
        A.call(name, H.handle, psi.handle, tstp, C.byref(opts), evals.ctypes.data_as(C.POINTER(C.c_double)),
               C.byref(res))
        self._act = res.act_dim
        self._evals = evals[:res.act_dim].copy()
        m = min(len(self._evs), res.act_dim)
        self._err = float(np.sqrt(np.sum((self._evals[:m] - self._evs[:m]) ** 2)))
        self._evs[:m] = self._evals[:m]
        self.result = res
        return res

    def act_dim(self) -> int:
        return self._act

    def error(self) -> float:
        return self._err

    def eigenvalues(self) -> np.ndarray:
        return self._evals

    def storeE(self, fname: str) -> None:
        with open(fname, "w") as f:
            for e in self._evals:
                f.write(f"{e:.6g}\n")


class ArnoldiSolver:
    """Arnoldi::getSolver(index, kry_dim) -- ArnoldiSolver<T, herm=0>: Krylov real-time
    steps (evolve) and the incremental Arnoldi ground state (getGroundState).

    getGroundState(H, psi, tstp, add_dim) keeps its Krylov space between calls
    as the reference solver does: the first call starts from psi(tstp) and
    runs add_dim steps of full orthogonalisation (all kry_dim for -1), later
    calls grow the same space (qd_arnoldi_extend) until kry_dim or a
    breakdown; psi(tstp) receives the Ritz vector each time.  error() is the
    change of the lowest N eigenvalues since the previous call, N and the
    initial values set by convergeEV(N, iv) (sparse_algorithm.hpp:494-500,
    564-585), the loop of programs/two_liquid_sq.cpp:464-476."""

    def __init__(self, index: Sector, kry_dim: int):
        self.index = index
        self.kry_dim = kry_dim
        self._act = 0
        self._gs_act = 0
        self._gs_full = False
        self._evals = np.empty(0)
        self._err = 0.0
        self._evs = np.zeros(1)
        self.result = None

    def convergeEV(self, N: int, iv: float = 0.0) -> None:
        if not N < self.kry_dim:
            raise ValueError("convergeEV: N must be below kry_dim")
        self._evs = np.full(N, float(iv))

    def getGroundState(self, H: Hamiltonian, psi: State, tstp: int, add_dim: int = -1):
        if self._gs_act >= self.kry_dim or self._gs_full:
            return self.result
        opts = A.qd_lanczos_opts(self.kry_dim, A.QD_SPMV_CSR, A.QD_RITZ_STORED_BASIS, add_dim if add_dim > 0 else 0)
        evals = np.empty(self.kry_dim, dtype=np.float64)
        res = A.qd_lanczos_result()
        name = "qd_arnoldi_ground" if self._gs_act == 0 else "qd_arnoldi_extend"
        A.call(name, H.handle, psi.handle, tstp, C.byref(opts), evals.ctypes.data_as(C.POINTER(C.c_double)),
               C.byref(res))
        self._gs_act = self._act = res.act_dim
        self._gs_full = bool(res.breakdown)
        self._evals = evals[:res.act_dim].copy()
        m = min(len(self._evs), res.act_dim)
        self._err = float(np.sqrt(np.sum((self._evals[:m] - self._evs[:m]) ** 2)))
        self._evs[:m] = self._evals[:m]
        self.result = res
        return res

    def error(self) -> float:
        return self._err

    def eigenvalues(self) -> np.ndarray:
        return self._evals

    def storeE(self, fname: str) -> None:
        with open(fname, "w") as f:
            for e in self._evals:
                f.write(f"{e:.6g}\n")

    def evolve(self, H: Hamiltonian, psi: State, tstp: int, h: float, kry_dim_rt: int = 0) -> None:
        """psi(tstp + 1) = exp(-i H h) psi(tstp) / ||psi(tstp)|| (sparse_algorithm.hpp:548-562)."""
        if tstp + 1 >= psi.nt():
            raise IndexError("evolve writes psi(tstp + 1)")
        m = kry_dim_rt or self.kry_dim
        act = C.c_int(0)
        A.call("qd_arnoldi_evolve", H.handle, psi.handle, tstp, tstp + 1, float(h), m, C.byref(act))
        self._act = act.value

    def evolve_inplace(self, H: Hamiltonian, psi: State, t: int, h: float, m: int = 0) -> None:
        act = C.c_int(0)
        A.call("qd_arnoldi_evolve", H.handle, psi.handle, t, t, float(h), m or self.kry_dim, C.byref(act))
        self._act = act.value

    def act_dim(self) -> int:
        return self._act


class HermitianLanczosSolver:
    """Hermitian::LanczosSolver(index, kry_dim): two-vector Lanczos ground state."""

    def __init__(self, index: Sector, kry_dim: int):
        self.index = index
        self.kry_dim = kry_dim
        self._evals = np.empty(0)
        self.result = None

    def getGroundState(self, H: Hamiltonian, psi: State, tstp: int):
        evals = np.empty(self.kry_dim + 1, dtype=np.float64)
        res = A.qd_lanczos_result()
        A.call("qd_hermitian_lanczos_ground", H.handle, psi.handle, tstp, self.kry_dim,
               evals.ctypes.data_as(C.POINTER(C.c_double)), C.byref(res))
        self._evals = evals[:res.act_dim].copy()
        self.result = res
        return res

    def eigenvalues(self) -> np.ndarray:
        return self._evals


class Hermitian:
    LanczosSolver = HermitianLanczosSolver


class Arnoldi:
    @staticmethod
    def getLanczosSolver(index: Sector, kry_dim: int, **kw) -> LanczosSolver:
        return LanczosSolver(index, kry_dim, **kw)

    @staticmethod
    def getSolver(index: Sector, kry_dim: int) -> ArnoldiSolver:
        return ArnoldiSolver(index, kry_dim)


def batch_lanczos(hams, v0s, steps: int, ctx: Optional[Context] = None) -> np.ndarray:
    """Many ground states in one persistent launch (mixed precision, FP64 refinement).

    Returns an (ninst, 8) array: lowest Krylov eigenvalue, refined FP64 energy,
    psi^T psi, act_dim, breakdown flag, start and end of the instance on the device
    clock (ns), CTAs that computed it.
    """
    n = len(hams)
    ctx = ctx or hams[0].ctx
    hp = (C.c_void_p * n)(*[h.handle.value for h in hams])
    keep = [np.ascontiguousarray(v, dtype=np.float64) for v in v0s]
    vp = (A._DP * n)(*[k.ctypes.data_as(A._DP) for k in keep])
    out = np.zeros((n, 8))
    A.call("qd_batch_lanczos", ctx.handle, n, hp, vp, steps, out.ctypes.data_as(A._DP))
    return out


def traj_run(heff: Hamiltonian, psi0, ntraj: int, nsteps: int, dt: float, gamma: float, seed: int, m: int,
             chan_bits, obs_pairs):
    """Quantum-jump trajectories (diagonal jumps sqrt(gamma) n_bit) on the device.

    Returns (mean, stderr, stats): (nsteps+1) x len(obs_pairs) arrays of
    <n_a n_b> averaged over the trajectories, and the qd_traj_stats record.
    """
    cb = np.ascontiguousarray(chan_bits, dtype=np.int32)
    oa = np.ascontiguousarray([a for a, _ in obs_pairs], dtype=np.int32)
    ob = np.ascontiguousarray([b for _, b in obs_pairs], dtype=np.int32)
    d = A.qd_traj_desc()
    d.ntraj = ntraj
    d.nsteps = nsteps
    d.dt = dt
    d.gamma = gamma
    d.seed = seed
    d.m = m
    d.nchan = len(cb)
    d.chan_bits = cb.ctypes.data_as(C.POINTER(C.c_int32))
    d.nobs = len(oa)
    d.obs_a = oa.ctypes.data_as(C.POINTER(C.c_int32))
    d.obs_b = ob.ctypes.data_as(C.POINTER(C.c_int32))
    psi0 = np.ascontiguousarray(np.asarray(psi0, dtype=np.complex128))
    mean = np.zeros((nsteps + 1, len(oa)))
    err = np.zeros((nsteps + 1, len(oa)))
    st = A.qd_traj_stats()
    A.call("qd_traj_run", heff.handle, C.byref(d), psi0.ctypes.data_as(A._DP), mean.ctypes.data_as(A._DP),
           err.ctypes.data_as(A._DP), C.byref(st))
    return mean, err, st


def lanczos_evolve(H: Hamiltonian, psi: State, t_in: int, t_out: int, h: float, m: int, nsteps: int = 1) -> int:
    """psi(t_out) = exp(-i H h)^nsteps psi(t_in) by the short-recurrence Krylov
    exponential (Hermitian H); returns the last step's Krylov dimension."""
    act = C.c_int(0)
    A.call("qd_lanczos_evolve", H.handle, psi.handle, t_in, t_out, h, m, nsteps, C.byref(act))
    return act.value


def obs_eval(psi: State, t: int, observables) -> np.ndarray:
    """<psi(t)|O_i|psi(t)> for a list of lowered operators, one device pass each, one copy back."""
    n = len(observables)
    hp = (C.c_void_p * n)(*[o.handle.value for o in observables])
    out = np.zeros(2 * n)
    A.call("qd_obs_eval", psi.handle, t, n, hp, out.ctypes.data_as(A._DP))
    return out[0::2] + 1j * out[1::2]


MC_REAL = 0
MC_COMPLEX = 1


def _to_string(v) -> str:
    """std::to_string: %d for integers, %f for floating point."""
    return "%d" % v if isinstance(v, (int, np.integer)) else "%f" % v


class McManager:
    """McManager (mc_manager.hpp:14-214): observables are named groups of `dim`
    operators, data[name] is an (nt, dim) complex table.

    addObs(name, dim, type=MC_COMPLEX), updateMatrix(name, idx, H) / incrMatrix
    (matrix sum) / normMatrix (in-place multiple) / matrix(name, idx);
    addAux(name, name2, func, dim, aux_type) derives a table from name2's values;
    incrAllObs(tstp, psi_tstp=-1) adds psi.eval(psi_tstp, O) of every operator into
    row tstp (all evaluations in one device pass list, qd_obs_eval) and counts the
    sample; normAll() divides row t by its sample count; clearAll([tstp]);
    collectAll() averages the tables over the ranks of torch.distributed (the
    reference's MPI_Reduce, then / Nproc), a no-op in one process; outFile(h,
    fname, names) writes the reference's TSV table (rank 0 only)."""

    def __init__(self, nt: int, psi: State):
        self.nt = nt
        self.psi = psi
        self.data = {}
        self.obs = {}
        self.aux = {}
        self.func = {}
        self.type = {}
        self.Nmc = np.zeros(nt, dtype=np.int64)

    def report(self) -> int:
        import torch.distributed as dist
        return dist.get_rank() if dist.is_available() and dist.is_initialized() else 0

    def addObs(self, name: str, dim: int, type: int = MC_COMPLEX) -> None:
        self.data[name] = np.zeros((self.nt, dim), dtype=np.complex128)
        self.obs[name] = [None] * dim
        self.aux[name] = []
        self.type[name] = type

    def addAux(self, name: str, name2: str, func, dim: int, aux_type: int = MC_COMPLEX) -> None:
        if name2 not in self.obs:
            raise KeyError("addAux: wrong dependent variable!")
        self.data[name] = np.zeros((self.nt, dim), dtype=np.complex128)
        self.func[name] = func
        self.type[name] = aux_type
        self.aux[name2].append(name)

    def updateMatrix(self, name: str, idx: int, mat: Hamiltonian) -> None:
        self.obs[name][idx] = mat

    def incrMatrix(self, name: str, idx: int, mat: Hamiltonian) -> None:
        cur = self.obs[name][idx]
        self.obs[name][idx] = mat.copy() if cur is None else cur + mat

    def normMatrix(self, name: str, idx: int, s) -> None:
        self.obs[name][idx].scale(s)

    def matrix(self, name: str, idx: int) -> Hamiltonian:
        return self.obs[name][idx]

    def incrAllObs(self, tstp: int, psi_tstp: int = -1) -> None:
        if psi_tstp == -1:
            psi_tstp = tstp
        keys = [(n, d) for n, mats in self.obs.items() for d in range(len(mats))]
        if keys:
            vals = obs_eval(self.psi, psi_tstp, [self.obs[n][d] for n, d in keys])
            for (n, d), v in zip(keys, vals):
                self.data[n][tstp, d] += v
                for a in self.aux[n]:
                    self.data[a][tstp, d] += self.func[a](v)
        self.Nmc[tstp] += 1

    def clearAll(self, tstp: Optional[int] = None) -> None:
        for t in self.data.values():
            if tstp is None:
                t[:] = 0
            else:
                t[tstp] = 0

    def normAll(self) -> None:
        for t in self.data.values():
            t /= self.Nmc[:, None]

    def collectAll(self) -> None:
        import torch
        import torch.distributed as dist
        if not (dist.is_available() and dist.is_initialized()):
            return
        n = dist.get_world_size()
        for name in sorted(self.data):
            t = torch.from_numpy(self.data[name].view(np.float64).copy())
            dist.all_reduce(t)
            self.data[name] = (t.numpy() / n).view(np.complex128)

    def obsValue(self, name: str, tstp: int, idx: int) -> complex:
        return complex(self.data[name][tstp, idx])

    def outFile(self, h: float, fname: str, obs_names, precision: int = 6) -> None:
        """The TSV table of mc_manager.hpp:147-196: "#time[\tindex]" and one column per
        real observable or two (real, imag) per complex one, values as std::to_string
        writes them; with dim > 1 a row per index and a blank line after each time."""
        if self.report() != 0:
            return
        with open(fname, "w") as f:
            if obs_names[0] not in self.data:
                raise KeyError("outFile: wrong name!!")
            dim = self.data[obs_names[0]].shape[1]
            label = "#time\tindex" if dim > 1 else "#time"
            for n in obs_names:
                if n not in self.type:
                    raise KeyError("outFile: wrong name!!")
                label += ("\t" + n) if self.type[n] == MC_REAL else ("\t" + n + "(real)" + "\t" + n + "(imag)")
                if self.data[n].shape[1] != dim:
                    print("mismatched dimensions")
                    return
            f.write(label + "\n")
            for t in range(self.nt):
                for idx in range(dim):
                    row = _to_string(t * h) + ("\t" + _to_string(idx) if dim > 1 else "")
                    for n in obs_names:
                        v = self.data[n][t, idx]
                        row += "\t" + _to_string(float(v.real))
                        if self.type[n] == MC_COMPLEX:
                            row += "\t" + _to_string(float(v.imag))
                    f.write(row + "\n")
                if dim > 1:
                    f.write("\n")


def seeded_start(seed: int, dim: int) -> np.ndarray:
    """The start vector the request loop draws for `seed` (Philox4x32-10, host copy)."""
    out = np.empty(dim)
    A.call("qd_seeded_start", C.c_uint64(seed), dim, out.ctypes.data_as(A._DP))
    return out


class Server:
    """The request loop (qd_server_*): submit ground-state and evolution
    requests as operator descriptions, poll finished results.

    mode "plain" runs every request with the FP64 reference algorithms;
    "mixed" batches small real ground states (FP32 products, FP64 refinement)
    and evolves Hermitian operators with the short-recurrence exponential.
    """

    def __init__(self, mode: str = "mixed", small_lanes: int = 4, large_lanes: int = 3, batch_lanes: int = 2,
                 batch_max: int = 64, small_dim: int = 65536, hbm_budget: int = 0, batch_dim: int = 3432,
                 batch_min: int = 4, ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        o = A.qd_server_opts()
        o.mode = A.QD_SERVE_MIXED if mode == "mixed" else A.QD_SERVE_PLAIN
        o.small_lanes = small_lanes
        o.large_lanes = large_lanes
        o.batch_lanes = batch_lanes
        o.batch_max = batch_max
        o.batch_min = batch_min
        o.small_dim = small_dim
        o.hbm_budget = hbm_budget
        o.batch_dim = batch_dim
        self.handle = C.c_void_p()
        A.call("qd_server_create", self.ctx.handle, C.byref(o), C.byref(self.handle))
        self.mode = mode
        self._keep = {}

    def _submit(self, kind: int, spec: SectorSpec, opsum: OperatorSum, krylov_dim: int, nsteps: int,
                dt: float, psi0, seed: int, want_state: bool, dim_hint: int, tag: int) -> int:
        q = A.qd_request()
        q.kind = kind
        q.nbits = spec.nbits
        cons, nc = spec.constraint_array()
        q.ncons = nc
        q.tight = spec.tight
        q.cons = C.cast(cons, C.POINTER(A.qd_constraint))
        terms, nt, gates, ng = opsum.pack()
        q.terms = C.cast(terms, C.POINTER(A.qd_term))
        q.gates = C.cast(gates, C.POINTER(A.qd_gate))
        q.nterms = nt
        q.ngates = ng
        q.krylov_dim = krylov_dim
        q.nsteps = nsteps
        q.dt = dt
        q.seed = seed
        q.tag = tag
        keep = [cons, terms, gates]
        if psi0 is not None:
            p0 = np.ascontiguousarray(np.asarray(psi0, dtype=np.complex128))
            q.psi0 = p0.ctypes.data_as(A._DP)
            q.psi0_len = len(p0)
            keep.append(p0)
        out = None
        if want_state:
            n = dim_hint if dim_hint else (len(psi0) if psi0 is not None else 0)
            if n <= 0:
                raise ValueError("want_state needs the sector dimension (dim_hint) or psi0")
            out = np.zeros(n, dtype=np.complex128)
            q.psi_out = out.ctypes.data_as(A._DP)
            q.psi_out_len = n
        rid = C.c_uint64()
        A.call("qd_server_submit", self.handle, C.byref(q), C.byref(rid))
        self._keep[rid.value] = out
        return rid.value

    def submit_ground(self, spec: SectorSpec, opsum: OperatorSum, krylov_dim: int = 100, psi0=None, seed: int = 0,
                      want_state: bool = False, dim_hint: int = 0, tag: int = 0) -> int:
        return self._submit(A.QD_REQ_GROUND, spec, opsum, krylov_dim, 0, 0.0, psi0, seed, want_state, dim_hint, tag)

    def submit_evolve(self, spec: SectorSpec, opsum: OperatorSum, dt: float, nsteps: int, m: int = 16, psi0=None,
                      seed: int = 0, want_state: bool = False, dim_hint: int = 0, tag: int = 0) -> int:
        return self._submit(A.QD_REQ_EVOLVE, spec, opsum, m, nsteps, dt, psi0, seed, want_state, dim_hint, tag)

    def poll(self, max_results: int = 256, timeout_ms: int = 0):
        buf = (A.qd_result * max_results)()
        n = C.c_int(0)
        A.call("qd_server_poll", self.handle, buf, max_results, C.byref(n), timeout_ms)
        out = []
        for i in range(n.value):
            r = buf[i]
            d = {f: getattr(r, f) for f, _ in A.qd_result._fields_}
            d["state"] = self._keep.pop(r.id, None)
            out.append(d)
        return out

    def wait_all(self, ids, timeout_s: float = 600.0):
        want = set(ids)
        got = {}
        import time as _t
        t_end = _t.monotonic() + timeout_s
        while want - set(got):
            if _t.monotonic() > t_end:
                raise TimeoutError(f"{len(want - set(got))} requests still pending")
            for r in self.poll(256, 100):
                got[r["id"]] = r
        return got

    def now(self) -> float:
        t = C.c_double()
        A.call("qd_server_now", self.handle, C.byref(t))
        return t.value

    def stats(self) -> dict:
        st = A.qd_server_stats()
        A.call("qd_server_get_stats", self.handle, C.byref(st))
        return {f: getattr(st, f) for f, _ in A.qd_server_stats._fields_}

    def close(self):
        if getattr(self, "handle", None) and self.handle.value and not _SHUTDOWN[0]:
            A.call("qd_server_destroy", self.handle)
        self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
