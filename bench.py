"""Benchmark: Lanczos ground state of the periodic XXZ chain, L = 24, Sz = 0.

Workload (the reference's headline case): H = sum_i [Jxy/2 (S+_i S-_{i+1} + h.c.)
+ Jz S^z_i S^z_{i+1}], Jxy = Jz = 1, dim 2,704,156, nnz 36,564,892 (explicit
zeros kept), FP64 Lanczos with krylov_dim = 100 from a seeded uniform[-1, 1]
start vector.  One step = one getGroundState solve (100 sparse products and
the fused dot / axpy / norm kernels, the tridiagonal solve and the Ritz
vector) with the Hamiltonian and start vector already in HBM.

  value    matvecs/s over the timed steps (CUDA events on the engine stream)
  e2e      the same metric through the public API with host buffers: each step
           uploads the start vector from pinned memory, solves, evaluates
           psi.eval and downloads the Ritz vector
  roofline achieved HBM GB/s of the kernel the recurrence launches, per launch
           over its CUDA-event time: for the one-launch Lanczos step (the
           default for uniform couplings) the step's algorithmic bytes
           nnz*(8+4) + (dim+1)*4 + dim*24 (matrix, v1, v2, v_k); for a product
           launched alone one FP64 CSR matvec, nnz*(8+4) + (dim+1)*4 + dim*16
  cpu_baseline  the CPU oracle port (the reference's CSC column-push product,
           complex128, one core like the reference) on a bounded sample

--impl reference times that CPU port alone on the same workload.
Multi-GPU: each rank solves its own copy (replicas; no data-path collective).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L = 24
KRY = 100
SEED = 12345
METRIC = "matvecs/s (Lanczos ground state, XXZ L=24 Sz=0, FP64)"
UNIT = "matvecs/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Replica bookkeeping across ranks: a barrier and max/sum of per-rank
    numbers (NCCL between GPUs; gloo on CPU for the host-side tests)."""

    def __init__(self, world, local, backend="nccl"):
        self.world = world
        self.pg = None
        self.device = "cuda" if backend == "nccl" else "cpu"
        if world > 1:
            import torch
            import torch.distributed as dist
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend)
            self.dist = dist
            self.torch = torch

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def _reduce(self, x: float, op) -> float:
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x: float) -> float:
        return x if self.world == 1 else self._reduce(x, self.dist.ReduceOp.MAX)

    def sum(self, x: float) -> float:
        return x if self.world == 1 else self._reduce(x, self.dist.ReduceOp.SUM)

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # wait (at most 3 s) for the first sample so the timed region is covered
        t_end = time.monotonic() + 3.0
        while time.monotonic() < t_end and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
            time.sleep(0.01)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sms.append(float(p[1]))
                    mx = float(p[2])
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sms)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel_key: str):
    """dram bytes per launch recorded from an ncu capture in profiles/ (line
    `traffic_bytes_per_launch: <n>` in the summary named for the kernel)."""
    path = os.path.join(ROOT, "profiles", f"{kernel_key}.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.strip().startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].strip().split()[0])
                except ValueError:
                    return None
    return None


# ----------------------------------------------------------------- CPU legs
def cpu_sample(kry: int, budget_s: float):
    """The oracle port on one core: repeated Lanczos solves of kry steps at L=24."""
    import oracle as O
    from qudrip_gb300 import chains
    spec, ham = chains.xxz_chain(L)
    sec = O.Sector(spec)
    H = O.Ham(sec, ham)
    v0 = np.random.Generator(np.random.PCG64(SEED)).uniform(-1.0, 1.0, sec.dim)
    return H, v0


def run_cpu_steps(H, v0, kry, steps):
    mv = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        r = H.lanczos_ground(v0, kry)
        mv += r["matvecs"]
    dt = time.perf_counter() - t0
    return mv, dt


def run_cpu_threads(H, v0, kry, steps, nthreads):
    """`nthreads` host threads each run `steps` oracle Lanczos solves on the
    shared read-only Hamiltonian (ctypes releases the GIL inside the oracle)."""
    import threading
    counts = [0] * nthreads

    def work(i):
        counts[i] = run_cpu_steps(H, v0, kry, steps)[0]

    th = [threading.Thread(target=work, args=(i,)) for i in range(nthreads)]
    t0 = time.perf_counter()
    for t in th:
        t.start()
    for t in th:
        t.join()
    return sum(counts), time.perf_counter() - t0


def reference_arm(args, rank, world):
    if rank != 0:
        return 0
    H, v0 = cpu_sample(4, 0)
    kry = 4  # bounded sample: 2*4 products per solve (first pass + getState pass)
    nthreads = max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)
    run_cpu_threads(H, v0, kry, 1, nthreads)
    t_all = 0.0
    mv_all = 0
    for _ in range(args.steps):
        mv, dt = run_cpu_threads(H, v0, kry, 1, nthreads)
        mv_all += mv
        t_all += dt
    value = mv_all / t_all
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_all / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded uniform[-1,1] start vector)",
        "config": {"workload": "xxz_chain_L24_periodic_Sz0_lanczos", "L": L, "dim": H.dim, "nnz": H.nnz,
                   "krylov_dim_sample": kry, "spmv": "csc_column_push_complex128", "threads": nthreads,
                   "compared_as": "matvecs/s: the reference's State is complex128, so each product here is a "
                                  "complex128 CSC column push (about 4x the flops and 1.7x the bytes of the GPU "
                                  "arm's real FP64 product); each solve runs krylov_dim=4 (a bounded sample), the "
                                  "GPU arm krylov_dim=100"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"each step: {nthreads} concurrent Lanczos solves (one per host thread) with "
                                   f"krylov_dim={kry} at L=24 on one shared CSC matrix (CPU restatement of the "
                                   "reference, which is single-threaded per solve)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------- GPU arm
def gpu_arm(args, rank, world, local):
    import qudrip_gb300 as q
    from qudrip_gb300 import _capi as A
    from qudrip_gb300 import chains

    dist = Dist(world, local)
    ctx = q.Context(local)
    spec, ham = chains.xxz_chain(L)
    sec = q.Sector(spec.index, spec.constraints, ctx=ctx)
    H = sec.lower(ham)
    if args.product is not None:
        A.call("qd_ham_set_spmv_kernel", H.handle, args.product)
    dim = sec.dim
    v0 = q.start_vector(dim, SEED).astype(np.complex128)
    psi = q.getState(sec, 2)
    psi.set(1, v0)  # resident start vector

    def solve_resident():  # a fresh solver per solve (a solver keeps its Krylov space between calls)
        A.call("qd_state_copy", psi.handle, 1, psi.handle, 0)
        return q.Arnoldi.getLanczosSolver(sec, KRY).getGroundState(H, psi(0), 0)

    for _ in range(args.warmup):
        solve_resident()
    ctx.sync()
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    ctx.sync()
    l0 = ctx.launches()
    A.call("qd_ctx_record", ctx.handle, 0)
    mv = 0
    ritz = None
    for _ in range(args.steps):
        r = solve_resident()
        mv += r.matvecs
        ritz = r.ritz_value
    A.call("qd_ctx_record", ctx.handle, 1)
    ms = C.c_float(0)
    A.call("qd_ctx_elapsed", ctx.handle, 0, 1, C.byref(ms))
    ctx.sync()
    launches = ctx.launches() - l0
    dist.barrier()
    clk = clocks.stop()
    t_max = dist.max(ms.value / 1e3)
    mv_all = dist.sum(float(mv))
    value = mv_all / t_max

    # roofline of the product kernel, timed live on the engine stream
    avg_ms = C.c_double(0)
    nbytes = C.c_double(0)
    A.call("qd_ham_time_spmv", H.handle, A.QD_SPMV_CSR, 50, C.byref(avg_ms), C.byref(nbytes))
    hbm_peak, peak_kind = peaks()
    # Algorithmic bytes of one L=24 matvec (the unit of the metric): the FP64
    # CSR figure nnz*(8+4) + (dim+1)*4 + dim*(8+8) = 492,861,828 B, whatever
    # format the kernel reads (the uniform-coupling form reads fewer bytes for
    # the same unit; its own byte count is reported beside).  Where the whole
    # Lanczos step is one launch the unit is one step: the matrix, v1 and v2
    # read once, v_k written once (w never leaves the chip):
    # nnz*12 + (dim+1)*4 + dim*24 = 514,495,076 B.
    info = A.qd_ham_info()
    A.call("qd_ham_get_info", H.handle, C.byref(info))
    one_launch = info.step_launches == 1
    unit_bytes = H.nnz * 12 + (dim + 1) * 4 + dim * (24 if one_launch else 16)
    achieved = unit_bytes / (avg_ms.value * 1e-3) / 1e9
    if info.product_kernel == 120:
        kernel_name = "lz_fx_step_kernel<SellRows,true>" if one_launch else "spmv_fx_dots_kernel<true>"
        spmv_name = ("uniform_coupling_fixed_point_sums_sliced_columns_one_launch_step" if one_launch else
                     "uniform_coupling_fixed_point_sums_sliced_columns_fused_dots")
        traffic = profile_traffic("lz_fx_step_xxz_L24" if one_launch else "spmv_fx_dots_xxz_L24")
    elif info.product_kernel == 122:
        kernel_name = "lz_fx_step_kernel<BlockRows,true>" if one_launch else "spmv_fx_block_dots_kernel<true>"
        spmv_name = ("uniform_coupling_fixed_point_sums_block_layout_one_launch_step" if one_launch else
                     "uniform_coupling_fixed_point_sums_block_layout_fused_dots")
        traffic = profile_traffic("lz_fx_step_block_xxz_L24" if one_launch else "spmv_fx_block_dots_xxz_L24")
    elif info.product_kernel == 121:
        kernel_name = "lz_fx_step_kernel<SlotRows,true>" if one_launch else "spmv_fx_slots_dots_kernel<true>"
        spmv_name = ("uniform_coupling_fixed_point_sums_columns_from_terms_one_launch_step" if one_launch else
                     "uniform_coupling_fixed_point_sums_columns_from_terms_fused_dots")
        traffic = None
    else:
        kernel_name, spmv_name = "spmv_rowexact_kernel<double,double>", "csr_row_exact_fp64"
        traffic = profile_traffic("spmv_csr_f64_xxz_L24")

    # end to end through the public API with pinned host buffers
    hb = C.c_void_p()
    A.call("qd_host_alloc", dim * 16, C.byref(hb))
    hv = np.ctypeslib.as_array((C.c_double * (2 * dim)).from_address(hb.value)).view(np.complex128)
    hv[:] = v0
    ho = C.c_void_p()
    A.call("qd_host_alloc", dim * 16, C.byref(ho))
    dptr = C.cast(hb, C.POINTER(C.c_double))
    optr = C.cast(ho, C.POINTER(C.c_double))
    e_steps = args.steps  # the same step count as the device-timed value

    def e2e_step():
        A.call("qd_state_upload", psi.handle, 0, dptr)
        r = q.Arnoldi.getLanczosSolver(sec, KRY).getGroundState(H, psi(0), 0)
        E = psi.eval(0, H)
        A.call("qd_state_download", psi.handle, 0, optr)
        return r, E

    e2e_step()
    dist.barrier()
    t0 = time.perf_counter()
    e_mv = 0
    energy = None
    for _ in range(e_steps):
        r, energy = e2e_step()
        e_mv += r.matvecs + 1
    ctx.sync()
    t_e2e = dist.max(time.perf_counter() - t0)
    e2e_value = dist.sum(float(e_mv)) / t_e2e
    A.call("qd_host_free", hb)
    A.call("qd_host_free", ho)

    extras = {}
    if not args.no_extras:
        extras["matrix_free_L24"] = matrix_free_leg(ctx, H, sec, psi, ritz)
        extras["xy_chain_L24"] = xy_leg(ctx)
        extras["batched_disorder_sweep"] = batched_sweep(ctx)
        extras["jump_trajectories"] = trajectory_ensemble(ctx, with_oracle=not args.no_cpu)
        extras["serving_mix"] = serving_mix(args.serve_requests)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        Ho, ov0 = cpu_sample(4, 0)
        mv_c, dt_c = run_cpu_steps(Ho, ov0, 4, 6)
        cpu = {"value": mv_c / dt_c, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "6 Lanczos solves with krylov_dim=4 at L=24 (48 complex128 CSC products plus "
                         "vector work, CPU restatement of the reference, single-threaded like it)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded uniform[-1,1] start vector; Hamiltonian built from the operator tree)",
            "config": {"workload": "xxz_chain_L24_periodic_Sz0_lanczos_k100", "L": L, "Jxy": 1.0, "Jz": 1.0,
                       "dim": dim, "nnz": H.nnz, "krylov_dim": KRY, "spmv": spmv_name,
                       "ritz": "stored_basis", "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (CSR 493 MB); no flush",
                       "ritz_value": ritz, "psi_eval": energy.real if energy is not None else None},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": dim * 16,
                    "d2h_bytes_per_step": dim * 16 + 16},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "kernel": kernel_name, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": unit_bytes,
                         "format_bytes_per_launch": nbytes.value, "launch_ms": avg_ms.value},
            "cpu_baseline": cpu,
            "clocks": clk,
            "extras": extras,
        }
        print(json.dumps(line))
    dist.close()
    return 0


def xy_leg(ctx):
    """The XY chain of the README at L=24 (open boundary, Nset=12, dim 2,704,156, real FP64,
    Lanczos k=100 from the seeded start vector): matvecs/s of the solve and the product kernel
    against the per-matvec algorithmic bytes of the FP64 CSR product, as for the XXZ workload."""
    import qudrip_gb300 as q
    from qudrip_gb300 import _capi as A
    from qudrip_gb300 import chains
    spec, ham = chains.xy_chain(L)
    sec = q.Sector(spec.index, spec.constraints, ctx=ctx)
    H = sec.lower(ham)
    dim = sec.dim
    psi = q.getState(sec, 2)
    psi.set(1, q.start_vector(dim, SEED).astype(np.complex128))

    def solve():
        A.call("qd_state_copy", psi.handle, 1, psi.handle, 0)
        return q.Arnoldi.getLanczosSolver(sec, KRY).getGroundState(H, psi(0), 0)

    solve()
    ctx.sync()
    A.call("qd_ctx_record", ctx.handle, 2)
    mv, n = 0, 5
    for _ in range(n):
        r = solve()
        mv += r.matvecs
    A.call("qd_ctx_record", ctx.handle, 3)
    ms = C.c_float(0)
    A.call("qd_ctx_elapsed", ctx.handle, 2, 3, C.byref(ms))
    pm, pb = C.c_double(), C.c_double()
    A.call("qd_ham_time_spmv", H.handle, A.QD_SPMV_CSR, 30, C.byref(pm), C.byref(pb))
    unit_bytes = H.nnz * 12 + (dim + 1) * 4 + dim * 16
    step_bytes = H.nnz * 12 + (dim + 1) * 4 + dim * 24  # one Lanczos step: v2 read, v_k written too
    hbm_peak, _ = peaks()
    achieved = unit_bytes / (pm.value * 1e-3) / 1e9
    exact = -2.0 * sum(np.cos(np.pi * k / (L + 1)) for k in range(1, L + 1) if np.cos(np.pi * k / (L + 1)) > 0)
    return {"workload": "XY chain L=24 open (README model), Nset=12, dim 2,704,156, FP64 Lanczos k=100",
            "nnz": int(H.nnz), "matvecs_per_s": mv / (ms.value * 1e-3), "ms_per_solve": ms.value / n,
            "product_ms": pm.value, "algorithmic_bytes_per_matvec": unit_bytes,
            "achieved_GBps": achieved, "frac_of_measured_hbm": achieved / hbm_peak,
            "algorithmic_bytes_per_step": step_bytes,
            "frac_of_measured_hbm_step_bytes": step_bytes / (pm.value * 1e-3) / 1e9 / hbm_peak,
            "ritz_value": r.ritz_value, "free_fermion_E0": exact,
            "rel_dE_vs_free_fermion_E0": abs(r.ritz_value - exact) / abs(exact)}


def matrix_free_leg(ctx, H, sec, psi, ritz_csr):
    """The L=24 XXZ workload's second product: the same Lanczos solve through the
    matrix-free form (no stored matrix), timed, and checked against the FP64
    reference energy (scipy eigsh, tests/golden) and the CSR-path Ritz value."""
    import qudrip_gb300 as q
    from qudrip_gb300 import _capi as A
    def solve():
        A.call("qd_state_copy", psi.handle, 1, psi.handle, 0)
        return q.LanczosSolver(sec, KRY, spmv=A.QD_SPMV_MATRIX_FREE).getGroundState(H, psi(0), 0)

    solve()
    ctx.sync()
    A.call("qd_ctx_record", ctx.handle, 2)
    mv = 0
    n = 2
    for _ in range(n):
        r = solve()
        mv += r.matvecs
    A.call("qd_ctx_record", ctx.handle, 3)
    ms = C.c_float(0)
    A.call("qd_ctx_elapsed", ctx.handle, 2, 3, C.byref(ms))
    pm, pb = C.c_double(), C.c_double()
    A.call("qd_ham_time_spmv", H.handle, A.QD_SPMV_MATRIX_FREE, 20, C.byref(pm), C.byref(pb))
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        e0 = json.load(f)["heisenberg_periodic_e0"]["24"]["e0"]
    return {"matvecs_per_s": mv / (ms.value * 1e-3), "ms_per_solve": ms.value / n, "product_ms": pm.value,
            "bytes_per_product": pb.value, "ritz_value": r.ritz_value,
            "rel_dE_vs_reference_E0": abs(r.ritz_value - e0) / abs(e0),
            "rel_dE_vs_csr_path": abs(r.ritz_value - ritz_csr) / abs(ritz_csr),
            "device_bytes_of_the_operator": ("uniform couplings: 32-bit states 4 B/row + diagonal 8 B/row + slot "
                                             "tables of a few KB (no CSR is read); otherwise basis 8 B/row + "
                                             "diagonal 8 B/row")}


def batched_sweep(ctx, n_inst=512, steps=80, seed=2024, chain_L=None):
    """Disorder sweep: n_inst random-field XXZ chains, L uniform in {14,16,18,20} (or all
    of length chain_L), Sz=0, Jz=1, h_i ~ U[-2,2]; mixed-precision batched solve vs the
    plain FP64 solver run instance by instance.  Returns solves/s of both forms and the
    energy deviations."""
    import qudrip_gb300 as q
    from qudrip_gb300 import chains
    rng = np.random.Generator(np.random.PCG64(seed))
    t0 = time.perf_counter()
    hams, v0s, dims = [], [], []
    for i in range(n_inst):
        L = int(rng.choice([14, 16, 18, 20])) if chain_L is None else int(chain_L)
        h = rng.uniform(-2.0, 2.0, L)
        spec, ham = chains.xxz_chain(L, 1.0, 1.0, True, h)
        sec = q.Sector(spec.index, spec.constraints, ctx=ctx)
        hams.append(sec.lower(ham))
        v0s.append(q.start_vector(sec.dim, seed + i))
        dims.append(sec.dim)
    lower_s = time.perf_counter() - t0
    q.batch_lanczos(hams[:8], v0s[:8], steps)  # warm-up
    ctx.sync()
    t0 = time.perf_counter()
    out = q.batch_lanczos(hams, v0s, steps)
    mixed_s = time.perf_counter() - t0
    psi = {}
    plain_e = np.empty(n_inst)
    # plain FP64 form: the reference's algorithm, one instance after another
    for i in range(min(4, n_inst)):
        st = q.getState(hams[i].sector, 1)
        st.set(0, v0s[i])
        q.Arnoldi.getLanczosSolver(hams[i].sector, steps).getGroundState(hams[i], st(0), 0)
    ctx.sync()
    t0 = time.perf_counter()
    for i in range(n_inst):
        d = dims[i]
        st = psi.get(d)
        if st is None:
            st = psi[d] = q.getState(hams[i].sector, 1)
        st.set(0, v0s[i])
        r = q.Arnoldi.getLanczosSolver(hams[i].sector, steps).getGroundState(hams[i], st(0), 0)
        plain_e[i] = r.ritz_value
    ctx.sync()
    plain_s = time.perf_counter() - t0
    rel = np.abs(out[:, 1] - plain_e) / np.abs(plain_e)
    lset = "{14,16,18,20}" if chain_L is None else "{%d}" % chain_L
    # the device's own span of the call (out[:, 5:7]: each instance's start and end, ns) and the
    # reorthogonalisation's bytes: two passes over the stored FP32 basis, act (act + 1) / 2 vectors each
    span_s = (out[:, 6].max() - out[:, 5].min()) * 1e-9
    act = out[:, 3]
    dimf = np.array(dims, dtype=float)
    nnzf = np.array([float(h.nnz) for h in hams])
    reorth_bytes = float(np.sum(act * (act + 1) * dimf * 4.0))
    # per step k, as the kernel table counts it: the FP32 CSR product (nnz 8 B) and (2k + 3) vector
    # passes of dim 4 B (the basis read twice, w, v1, v2)
    step_bytes = float(np.sum(act * nnzf * 8.0 + (act * (act + 1) + 3 * act) * dimf * 4.0))
    hbm_peak, _ = peaks()
    return {"workload": f"{n_inst} random-field XXZ chains L in {lset}, {steps} Lanczos steps",
            "mixed_solves_per_s": n_inst / mixed_s, "plain_fp64_solves_per_s": n_inst / plain_s,
            "speedup": plain_s / mixed_s, "max_rel_dE": float(rel.max()), "median_rel_dE": float(np.median(rel)),
            "device_span_ms": span_s * 1e3, "algorithmic_step_bytes": step_bytes,
            "step_bytes_frac_of_measured_hbm": step_bytes / span_s / 1e9 / hbm_peak,
            "reorth_basis_bytes": reorth_bytes,
            "reorth_GBps_over_device_span": reorth_bytes / span_s / 1e9,
            "reorth_frac_of_measured_hbm": reorth_bytes / span_s / 1e9 / hbm_peak,
            "lowering_s_all_instances": lower_s, "mixed_form": "fp32 products/basis, fp64 accumulation, "
            "full reorthogonalisation, device tridiagonal, fp64 Rayleigh refinement; one persistent launch",
            "plain_form": "fp64 Lanczos (reference algorithm), one solve after another"}


def trajectory_ensemble(ctx, with_oracle=True, ntraj=4096, nsteps=1000):
    """Dissipative Hubbard chain: L=8, N_up=N_dn=4 (dim 4900), t=1, U=4, open, jumps
    sqrt(gamma) n_{i,s} on all 16 site-spins, gamma=0.1, 4096 trajectories, m=30,
    dt=0.01, T=10; observable <n_{i,up} n_{i,dn}>(t).  Starts from the ground state of
    Hermitian::LanczosSolver, as the reference program does (programs/hubbard_diss.cpp:382-384)."""
    import qudrip_gb300 as q
    from qudrip_gb300 import chains
    from qudrip_gb300.operators import getHopFermiGate
    Lh, gamma, dt, m, seed = 8, 0.1, 0.01, 30, 4242
    spec, ham = chains.hubbard_chain(Lh, 4, 4, 4.0, -1.0)
    sec = q.Sector(spec.index, spec.constraints, ctx=ctx)
    H = sec.lower(ham)
    psi = q.getState(sec, 1)
    psi.set(0, q.start_vector(sec.dim, 11))
    q.Hermitian.LanczosSolver(sec, 100).getGroundState(H, psi, 0)
    psi0 = psi.get(0)
    psi0 = psi0 / np.linalg.norm(psi0)
    gate = getHopFermiGate(spec.index)
    heff = ham
    for s in range(2 * Lh):
        heff = heff + (-0.5j * gamma) * gate(s, s)
    Heff = sec.lower(heff)
    chan = list(range(2 * Lh))
    obs = [(i, i + Lh) for i in range(Lh)]
    t0 = time.perf_counter()
    mean, err, st = q.traj_run(Heff, psi0, ntraj, nsteps, dt, gamma, seed, m, chan, obs)
    wall = time.perf_counter() - t0
    form = {0: "resident: one CTA per trajectory, operator and complex64 vectors in shared memory, "
               "truncated Taylor exp(-i dt (H - mu)) with the degree from its remainder bound",
            1: "FP64 Arnoldi exponential per trajectory and step (batched kernel)"}[int(st.path)]
    out = {"workload": f"dissipative Hubbard L=8 (dim 4900), {ntraj} trajectories x {nsteps} steps, m=30, dt=0.01",
           "trajectory_steps_per_s": ntraj * nsteps / wall, "wall_s": wall, "form": form,
           "products_per_step": int(st.products),
           "products_per_s": ntraj * nsteps * int(st.products) / (st.ensemble_ms * 1e-3),
           "setup_ms": st.setup_ms, "ensemble_ms": st.ensemble_ms, "jumps": int(st.jumps),
           "docc_t0": float(mean[0].mean()), "docc_T": float(mean[-1].mean()),
           "docc_T_stderr": float(err[-1].mean())}
    if with_oracle:
        import oracle as O
        osec = O.Sector(spec)
        oh = O.Ham(osec, heff)
        nt_c, ns_c = 16, 100
        ref, rj = O.traj_run(oh, osec.basis(), nt_c, ns_c, dt, gamma, seed, m, chan, obs, psi0)
        m2, _, st2 = q.traj_run(Heff, psi0, nt_c, ns_c, dt, gamma, seed, m, chan, obs)
        out["oracle_check"] = {"ntraj": nt_c, "nsteps": ns_c, "max_abs_diff": float(np.abs(m2 - ref).max()),
                               "jumps_gpu": int(st2.jumps), "jumps_oracle": int(rj)}
    return out


def spmv_only(args, local):
    """Time CSR product kernels alone on the L=24 matrix (also the ncu target)."""
    import qudrip_gb300 as q
    from qudrip_gb300 import _capi as A
    from qudrip_gb300 import chains
    ctx = q.Context(local)
    spec, ham = chains.xxz_chain(L)
    sec = q.Sector(spec.index, spec.constraints, ctx=ctx)
    H = sec.lower(ham)
    if args.product is not None:
        A.call("qd_ham_set_spmv_kernel", H.handle, args.product)
    kernels = sorted(A.SPMV_KERNELS) + [A.QD_SPMV_MATRIX_FREE] if args.spmv_only == 9999 else [args.spmv_only]
    hbm_peak, _ = peaks()
    for k in kernels:
        ms = C.c_double(0)
        nb = C.c_double(0)
        A.call("qd_ham_time_spmv", H.handle, k, args.iters, C.byref(ms), C.byref(nb))
        gbs = nb.value / (ms.value * 1e-3) / 1e9
        print(json.dumps({"kernel": ("matrix_free" if k == A.QD_SPMV_MATRIX_FREE else "") + A.SPMV_KERNELS.get(k % 1000, "") + ("+dot" if 2000 <= k < 3000 else "") + ({3001: "lanczos_k2", 3002: "lanczos_k3"}.get(k, "")), "id": k, "ms": ms.value, "GBps": gbs,
                          "frac": gbs / hbm_peak, "matvecs_per_s": 1e3 / ms.value}))
    return 0


def serving_requests(n_req, rate, seed):
    """The serving mix: Poisson arrivals (mean `rate`/s), 70% ground states
    (Lanczos k=100) and 30% real-time evolutions (T=5, dt=0.05: 100 Krylov
    steps of dimension 16) on XXZ chains with L uniform in {12,...,22} (Sz=0),
    Jz ~ U[0,2], and random fields h_i ~ U[-1,1] on half of them."""
    from qudrip_gb300 import chains
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    reqs = []
    for i in range(n_req):
        t += rng.exponential(1.0 / rate)
        L = int(rng.choice([12, 14, 16, 18, 20, 22]))
        Jz = float(rng.uniform(0.0, 2.0))
        h = rng.uniform(-1.0, 1.0, size=L) if rng.uniform() < 0.5 else None
        kind = "ground" if rng.uniform() < 0.7 else "evolve"
        spec, ham = chains.xxz_chain(L, 1.0, Jz, periodic=True, fields=h)
        reqs.append(dict(t=t, L=L, kind=kind, spec=spec, ham=ham, seed=int(rng.integers(1 << 62))))
    return reqs


def serve_stream(mode, reqs, **opts):
    """Submits `reqs` at their arrival times; returns results by request index."""
    import qudrip_gb300 as q
    srv = q.Server(mode=mode, **opts)
    try:
        # warm-up: one request of each kind and size class
        warm = [srv.submit_ground(r["spec"], r["ham"], 100, seed=1) for r in reqs[:4]]
        warm += [srv.submit_evolve(r["spec"], r["ham"], 0.05, 2, m=16, seed=1) for r in reqs[:2]]
        srv.wait_all(warm)
        t0 = srv.now()
        out = {}
        ids = {}
        i = 0
        while i < len(reqs) or len(out) < len(reqs):
            now = srv.now() - t0
            while i < len(reqs) and reqs[i]["t"] <= now:
                r = reqs[i]
                if r["kind"] == "ground":
                    rid = srv.submit_ground(r["spec"], r["ham"], 100, seed=r["seed"], tag=i)
                else:  # keep the evolved state to compare the two forms in 2-norm
                    rid = srv.submit_evolve(r["spec"], r["ham"], 0.05, 100, m=16, seed=r["seed"], tag=i,
                                            want_state=True, dim_hint=math.comb(r["L"], r["L"] // 2))
                ids[rid] = i
                i += 1
            wait_ms = 1 if i < len(reqs) else 50
            for res in srv.poll(256, wait_ms):
                out[res["tag"]] = res
        st = srv.stats()
    finally:
        srv.close()
    return out, st


def serving_mix(n_req=400, rate=200.0, seed=77, **opts):
    reqs = serving_requests(n_req, rate, seed)
    summary = {"workload": f"Poisson {rate:.0f} req/s, {n_req} requests: 70% ground state (Lanczos k=100), "
                           "30% evolution (T=5, dt=0.05, m=16); XXZ L in {12..22} Sz=0, Jz~U[0,2], "
                           "fields h_i~U[-1,1] on half"}
    results = {}
    for mode in ("mixed", "plain"):
        out, st = serve_stream(mode, reqs, **opts)
        lat = np.array([out[i]["t_done"] - out[i]["t_submit"] for i in range(n_req)])
        t_first = min(out[i]["t_submit"] for i in range(n_req))
        t_last = max(out[i]["t_done"] for i in range(n_req))
        bad = sum(1 for i in range(n_req) if out[i]["status"] != 0)
        by_kind = {}
        for kind in ("ground", "evolve"):
            idx = [i for i in range(n_req) if reqs[i]["kind"] == kind]
            lk = lat[idx]
            by_kind[kind] = {"n": len(idx), "p50_ms": 1e3 * float(np.percentile(lk, 50)),
                             "p99_ms": 1e3 * float(np.percentile(lk, 99))}
        results[mode] = out
        service = {}
        for kind in ("ground", "evolve"):
            for L in (12, 14, 16, 18, 20, 22):
                idx = [i for i in range(n_req) if reqs[i]["kind"] == kind and reqs[i]["L"] == L]
                if idx:
                    sv = [out[i]["t_done"] - out[i]["t_admit"] for i in idx]
                    service[f"{kind}_L{L}"] = round(1e3 * float(np.median(sv)), 2)
        busy = {kind: round(sum(out[i]["t_done"] - out[i]["t_admit"] for i in range(n_req)
                                if reqs[i]["kind"] == kind), 3) for kind in ("ground", "evolve")}
        summary[mode] = {"service_p50_ms": service, "service_s_total_by_kind": busy,
                         "solves_per_s": n_req / (t_last - t_first), "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                         "p99_ms": 1e3 * float(np.percentile(lat, 99)), "failed": bad, "by_kind": by_kind,
                         "batches": st["batches"], "batched": st["batched"], "max_active": st["max_active"],
                         "bytes_peak": st["bytes_peak"], "budget": st["budget"]}
    dE = [abs(results["mixed"][i]["energy"] - results["plain"][i]["energy"]) / abs(results["plain"][i]["energy"])
          for i in range(n_req) if reqs[i]["kind"] == "ground"]
    dEv = [abs(results["mixed"][i]["energy"] - results["plain"][i]["energy"]) / abs(results["plain"][i]["energy"])
           for i in range(n_req) if reqs[i]["kind"] == "evolve"]
    dpsi = [float(np.linalg.norm(results["mixed"][i]["state"] - results["plain"][i]["state"]))
            for i in range(n_req) if reqs[i]["kind"] == "evolve"]
    summary["max_rel_dE_ground_mixed_vs_plain"] = float(max(dE)) if dE else None
    summary["max_rel_dE_evolved_mixed_vs_plain"] = float(max(dEv)) if dEv else None
    summary["max_l2_dpsi_evolved_mixed_vs_plain"] = max(dpsi) if dpsi else None
    summary["speedup_solves_per_s"] = summary["mixed"]["solves_per_s"] / summary["plain"]["solves_per_s"]
    return summary


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--spmv-only", type=int, default=None, metavar="KERNEL",
                    help="only time product KERNEL on the L=24 matrix (100..111 CSR kernels, 1 matrix-free, "
                         "9999 all)")
    ap.add_argument("--iters", type=int, default=50)
    ap.add_argument("--product", type=int, default=None, metavar="KERNEL",
                    help="product kernel of the Lanczos solves (qd_ham_set_spmv_kernel code; default: the engine's)")
    ap.add_argument("--serve-only", action="store_true", help="only run the serving mix")
    ap.add_argument("--xy-only", action="store_true", help="only run the XY chain's Lanczos leg")
    ap.add_argument("--batch-only", type=int, default=None, metavar="N",
                    help="only run the batched disorder sweep with N instances")
    ap.add_argument("--batch-L", type=int, default=None, metavar="L",
                    help="with --batch-only: every chain of length L instead of L in {14,16,18,20}")
    ap.add_argument("--serve-requests", type=int, default=400)
    ap.add_argument("--traj-only", type=int, nargs=2, default=None, metavar=("NTRAJ", "NSTEPS"),
                    help="only run the trajectory ensemble with NTRAJ trajectories of NSTEPS steps")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return reference_arm(args, rank, world)
    if args.spmv_only is not None:
        return spmv_only(args, local)
    if args.serve_only:
        print(json.dumps(serving_mix(args.serve_requests)))
        return 0
    if args.xy_only:
        import qudrip_gb300 as q
        print(json.dumps(xy_leg(q.Context(local))))
        return 0
    if args.traj_only is not None:
        import qudrip_gb300 as q
        print(json.dumps(trajectory_ensemble(q.Context(local), with_oracle=False, ntraj=args.traj_only[0],
                                             nsteps=args.traj_only[1])))
        return 0
    if args.batch_only is not None:
        import qudrip_gb300 as q
        print(json.dumps(batched_sweep(q.Context(local), n_inst=args.batch_only, chain_L=args.batch_L)))
        return 0
    return gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
