"""ctypes view of the C ABI declared in include/qudrip_gb300.h.

The structures are defined without loading the shared library so that host
logic (operator algebra, argument packing) works on machines without a GPU.
`lib()` loads the in-tree library and fails loudly when it is missing: the
engine has no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libqudrip_gb300.so")

# status codes (qudrip_gb300.h)
QD_OK = 0
QD_ERR_INVALID = 1
QD_ERR_OOM = 2
QD_ERR_CUDA = 3
QD_ERR_BREAKDOWN = 4
QD_ERR_TIMEOUT = 5
QD_ERR_UNSUPPORTED = 6
QD_ERR_OVERFLOW = 7
QD_ERR_NOT_HERMITIAN = 8
QD_ERR_BUSY = 9

QD_CQ_NSET = 0
QD_CQ_ND = 1
QD_GATE_BIT = 0
QD_GATE_HOP = 1
QD_HAM_REAL = 1
QD_HAM_HERMITIAN = 2
QD_SPMV_CSR = 0
QD_SPMV_MATRIX_FREE = 1
QD_RITZ_STORED_BASIS = 0
QD_RITZ_SECOND_PASS = 1
QD_SPMV_FX = 120  # uniform-coupling form with exact fixed-point row sums
QD_SPMV_FX_SLOTS = 121  # the same with the columns computed on the fly from the terms
QD_SPMV_FX_BLOCK = 122  # the same on the block layout of the sector (no column read)
SPMV_KERNELS = {100: "tile", 101: "balanced", 102: "vector2", 103: "vector4", 104: "vector8",
                105: "scalar", 106: "row4", 107: "row8", 108: "row4_stream", 109: "row8_stream",
                110: "row_exact", 111: "row_sorted"}


class qd_cq_term(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nsite", C.c_int32), ("hole", C.c_int32),
                ("coef", C.c_int32), ("mask", C.c_uint64)]


class qd_constraint(C.Structure):
    _fields_ = [("nterms", C.c_int32), ("reserved", C.c_int32), ("target", C.c_int64),
                ("term", qd_cq_term * 4)]


class qd_gate(C.Structure):
    _fields_ = [("kind", C.c_int32), ("site", C.c_int32), ("site_b", C.c_int32),
                ("string", C.c_int32), ("u", C.c_double * 8)]


class qd_term(C.Structure):
    _fields_ = [("coeff_re", C.c_double), ("coeff_im", C.c_double),
                ("gate_offset", C.c_int32), ("ngates", C.c_int32)]


class qd_ham_info(C.Structure):
    _fields_ = [("dim", C.c_int64), ("nnz", C.c_int64), ("flags", C.c_int32),
                ("max_row_nnz", C.c_int32), ("has_matrix_free", C.c_int32),
                ("product_kernel", C.c_int32), ("step_launches", C.c_int32)]


class qd_lanczos_opts(C.Structure):
    _fields_ = [("krylov_dim", C.c_int32), ("spmv", C.c_int32), ("ritz", C.c_int32),
                ("add_dim", C.c_int32)]


class qd_lanczos_result(C.Structure):
    _fields_ = [("act_dim", C.c_int32), ("breakdown", C.c_int32), ("matvecs", C.c_int32),
                ("reserved", C.c_int32), ("ritz_value", C.c_double), ("err", C.c_double)]


class qd_traj_desc(C.Structure):
    _fields_ = [("ntraj", C.c_int32), ("nsteps", C.c_int32), ("dt", C.c_double), ("gamma", C.c_double),
                ("seed", C.c_uint64), ("m", C.c_int32), ("nchan", C.c_int32),
                ("chan_bits", C.POINTER(C.c_int32)), ("nobs", C.c_int32), ("reserved", C.c_int32),
                ("obs_a", C.POINTER(C.c_int32)), ("obs_b", C.POINTER(C.c_int32))]


class qd_traj_stats(C.Structure):
    _fields_ = [("jumps", C.c_int64), ("setup_ms", C.c_double), ("ensemble_ms", C.c_double),
                ("path", C.c_int32), ("products", C.c_int32)]


QD_REQ_GROUND = 0
QD_REQ_EVOLVE = 1
QD_SERVE_PLAIN = 0
QD_SERVE_MIXED = 1
QD_PATH_GRID = 0
QD_PATH_BATCH = 1


class qd_server_opts(C.Structure):
    _fields_ = [("mode", C.c_int32), ("small_lanes", C.c_int32), ("large_lanes", C.c_int32),
                ("batch_lanes", C.c_int32), ("batch_max", C.c_int32), ("batch_min", C.c_int32),
                ("small_dim", C.c_int64), ("hbm_budget", C.c_int64), ("batch_dim", C.c_int64),
                ("reserved", C.c_int32 * 2)]


class qd_request(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nbits", C.c_int32), ("ncons", C.c_int32), ("tight", C.c_int32),
                ("cons", C.POINTER(qd_constraint)), ("terms", C.POINTER(qd_term)),
                ("gates", C.POINTER(qd_gate)), ("nterms", C.c_int32), ("ngates", C.c_int32),
                ("krylov_dim", C.c_int32), ("nsteps", C.c_int32), ("dt", C.c_double),
                ("psi0", C.POINTER(C.c_double)), ("psi0_len", C.c_int64), ("seed", C.c_uint64),
                ("psi_out", C.POINTER(C.c_double)), ("psi_out_len", C.c_int64), ("tag", C.c_uint64)]


class qd_result(C.Structure):
    _fields_ = [("id", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("kind", C.c_int32),
                ("path", C.c_int32), ("act_dim", C.c_int32), ("dim", C.c_int64), ("nnz", C.c_int64),
                ("matvecs", C.c_int64), ("bytes", C.c_int64), ("energy", C.c_double),
                ("ritz", C.c_double), ("norm", C.c_double), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double)]


class qd_server_stats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "completed", "failed", "queued", "active",
                                         "max_active", "batches", "batched", "bytes_in_use",
                                         "bytes_peak", "budget")]


class QDError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: status {code} ({msg})")
        self.code = code


_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)

# name -> (argtypes); every function returns qd_status (int) unless listed in _RESTYPES
_SIGNATURES = {
    "qd_ctx_create": [C.c_int, _PP],
    "qd_ctx_destroy": [_P],
    "qd_ctx_sync": [_P],
    "qd_ctx_stream": [_P, _PP],
    "qd_ctx_launch_count": [_P, _I64P],
    "qd_ctx_record": [_P, C.c_int],
    "qd_ctx_elapsed": [_P, C.c_int, C.c_int, C.POINTER(C.c_float)],
    "qd_host_alloc": [C.c_int64, _PP],
    "qd_host_free": [_P],
    "qd_ham_time_spmv": [_P, C.c_int, C.c_int, _DP, _DP],
    "qd_ham_set_spmv_kernel": [_P, C.c_int],
    "qd_ham_autotune": [_P, C.c_int, C.POINTER(C.c_int), _DP],
    "qd_csr_expect_noalloc": [_P, _P, _P, C.c_int64, _P, _P, _P],
    "qd_arnoldi_evolve": [_P, _P, C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int)],
    "qd_batch_lanczos": [_P, C.c_int, C.POINTER(C.c_void_p), C.POINTER(_DP), C.c_int, _DP],
    "qd_krylov_evolve_batch": [_P, _P, C.c_int64, C.c_int, C.c_double, C.c_int, _P, C.c_int64,
                               C.POINTER(C.c_int)],
    "qd_traj_run": [_P, C.POINTER(qd_traj_desc), _DP, _DP, _DP, C.POINTER(qd_traj_stats)],
    "qd_status_string": [C.c_int],
    "qd_last_error": [],
    "qd_api_version": [],
    "qd_sector_create": [_P, C.c_int, C.POINTER(qd_constraint), C.c_int, C.c_int, _PP],
    "qd_sector_destroy": [_P],
    "qd_sector_dim": [_P, _I64P],
    "qd_sector_rank_kind": [_P, C.POINTER(C.c_int)],
    "qd_sector_basis": [_P, C.POINTER(C.c_uint64)],
    "qd_sector_rank": [_P, C.POINTER(C.c_uint64), C.c_int64, _I64P],
    "qd_ham_lower": [_P, C.POINTER(qd_term), C.c_int, C.POINTER(qd_gate), C.c_int, _PP],
    "qd_ham_destroy": [_P],
    "qd_ham_get_info": [_P, C.POINTER(qd_ham_info)],
    "qd_ham_add": [_P, _P, _PP],
    "qd_ham_copy": [_P, _PP],
    "qd_ham_scale": [_P, C.c_double, C.c_double],
    "qd_ham_build_matrix_free": [_P],
    "qd_ham_apply_matrix_free": [_P, _P, C.c_int, _P, C.c_int],
    "qd_ham_download_csc": [_P, _I64P, C.POINTER(C.c_int32), _DP],
    "qd_ham_download_csr": [_P, _I64P, C.POINTER(C.c_int32), _DP],
    "qd_state_create": [_P, C.c_int64, C.c_int, _PP],
    "qd_state_destroy": [_P],
    "qd_state_upload": [_P, C.c_int, _DP],
    "qd_state_download": [_P, C.c_int, _DP],
    "qd_state_device_ptr": [_P, C.c_int, _PP],
    "qd_state_copy": [_P, C.c_int, _P, C.c_int],
    "qd_ham_apply": [_P, _P, C.c_int, _P, C.c_int],
    "qd_state_eval": [_P, C.c_int, _P, _DP],
    "qd_obs_eval": [_P, C.c_int, C.c_int, C.POINTER(C.c_void_p), _DP],
    "qd_lanczos_ground": [_P, _P, C.c_int, C.POINTER(qd_lanczos_opts), _DP,
                          C.POINTER(qd_lanczos_result)],
    "qd_lanczos_extend": [_P, _P, C.c_int, C.POINTER(qd_lanczos_opts), _DP, C.POINTER(qd_lanczos_result)],
    "qd_arnoldi_ground": [_P, _P, C.c_int, C.POINTER(qd_lanczos_opts), _DP, C.POINTER(qd_lanczos_result)],
    "qd_arnoldi_extend": [_P, _P, C.c_int, C.POINTER(qd_lanczos_opts), _DP, C.POINTER(qd_lanczos_result)],
    "qd_hermitian_lanczos_ground": [_P, _P, C.c_int, C.c_int, _DP, C.POINTER(qd_lanczos_result)],
    "qd_lanczos_evolve": [_P, _P, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int)],
    "qd_seeded_start": [C.c_uint64, C.c_int64, _DP],
    "qd_server_create": [_P, C.POINTER(qd_server_opts), _PP],
    "qd_server_submit": [_P, C.POINTER(qd_request), C.POINTER(C.c_uint64)],
    "qd_server_poll": [_P, C.POINTER(qd_result), C.c_int, C.POINTER(C.c_int), C.c_int],
    "qd_server_now": [_P, _DP],
    "qd_server_get_stats": [_P, C.POINTER(qd_server_stats)],
    "qd_server_destroy": [_P],
}
_RESTYPES = {"qd_status_string": C.c_char_p, "qd_last_error": C.c_char_p,
             "qd_api_version": C.c_int}

_lib = None
_lock = threading.Lock()


def declared_symbols():
    """Names of every entry point this module binds (all declared in the header)."""
    return sorted(_SIGNATURES)


def lib():
    """Load libqudrip_gb300.so (built in-tree by __graft_entry__.build())."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"qudrip_gb300 CUDA library not found at {LIB_PATH}; "
                    "run `python -c 'import __graft_entry__ as g; g.build()'` first "
                    "(there is no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, args in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = _RESTYPES.get(name, C.c_int)
            _lib = L
    return _lib


def check(code: int, where: str):
    if code != QD_OK:
        L = lib()
        msg = (L.qd_last_error() or b"").decode() or (L.qd_status_string(code) or b"").decode()
        raise QDError(code, where, msg)


def call(name: str, *args):
    fn = getattr(lib(), name)
    check(fn(*args), name)
