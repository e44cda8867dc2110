"""Benchmark of the scirs2-sparse iterative-solve path on one GB300.

Metric: time to an FP64-verified relative residual of 1e-8, learned vs
Jacobi PCG, plus SpMV HBM GB/s.

Headline workload (the learned-SAI evaluation): 2D anisotropic diffusion on
Q1 elements, 1024 x 1024 grid (n = 1,048,576, nnz = 9,424,900), held-out
seed 1000001 of the training distribution (eps = 845.08, theta = 0.9632),
b ~ N(0, 1) from the seed, x0 = 0.  A step is one complete solve from b to
x including its setup: the FP32 copy of A, the network's forward pass and
the factor G, and FP32 PCG with FP64 residual replacement until
||b - A x||_2 <= 1e-8 ||b||_2 in FP64.  `value` times that step with A, b
and x resident on the device; `e2e` times the same step through the C ABI
with b copied from pinned host memory and x copied back inside the timed
region.  `jacobi_pcg_fp64` times plain FP64 Jacobi-PCG (the reference's
method) on the same problem and device, `speedup_vs_jacobi_fp64` is their
ratio; `jacobi_pcg_fp64_fused` and `speedup_vs_jacobi_fp64_fused` the same
method in two kernels per iteration (A p by the recurrence q = A z + beta q);
IC(0)-PCG (the reference's quirky factorisation and the textbook
one) is reported beside them.

`roofline` times the dominant kernel of the step, the FP32 SpMV of A,
alone with CUDA events on the library stream; `spmv_sweep` adds the 3D
7-point 128^3 Laplacian and the 4M-row power-law matrix in FP32 and FP64.
`workloads` reports the other configurations once each: 2D Poisson 256^2
FP64 Jacobi-PCG, the 128^3 Laplacian and the 160^3 variable-coefficient
problem with mixed precision and in FP64, and 4096 batched 2D systems.
`cpu_baseline` is one complete solve of the headline problem by the CPU
oracle (a restatement of the reference's cg with Jacobi; row-parallel SpMV
and elementwise loops on the host cores, bit-identical to one thread,
reductions serial like the reference's); `cpu_rows` times the other
configurations the same way.  `--impl reference` times complete oracle
solves of the headline problem, built by the oracle's own generators.

  python bench.py [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "Time to 1e-8 FP64 residual: learned vs Jacobi PCG on GB300; SpMV HBM GB/s"
TOL = 1e-8
SIDE = 1024            # headline grid side
PROBLEM_SEED = 1000001  # held-out seed of the training distribution
GRID = 128             # 3D Laplacian of the SpMV sweep
SEED = 0


def spmv_bytes(n: int, nnz: int, w: int) -> int:
    # nnz (w + 4) + 4 (n + 1) + 2 n w  (int32 indices, x read once, y written once)
    return nnz * (w + 4) + 4 * (n + 1) + 2 * n * w


def dia_bytes(n: int, ndiag: int, w: int, wv: int = 0) -> int:
    # diagonal layout: ndiag n values (wv bytes each, w when 0), the 2-byte
    # row masks, x read once, y written once; no column indices
    return ndiag * n * (wv or w) + 2 * n + 2 * n * w


def kernel_bytes(S, op, ip, ix, w, exact=True):
    """Algorithmic bytes of the kernel the library runs for op, and its format."""
    name = S.spmv_kernel(op, exact=exact)
    n = len(ip) - 1
    if name.startswith("spmv_dia_kernel"):
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(ip))
        nd = len(np.unique(np.asarray(ix, dtype=np.int64) - rows))
        return dia_bytes(n, nd, w, 2 if "FP16" in name else 0), "diagonal", name
    return spmv_bytes(n, len(ix), w), "csr", name


def headline_problem():
    """The headline problem from the library's own generators (device arm)."""
    import scirs_gb300 as S
    from scirs_gb300 import learned as LR

    prob = LR.sample_problem(PROBLEM_SEED)
    ip, ix, v = S.generate("aniso_q1", SIDE, SIDE, param0=prob.eps, param1=prob.theta)
    n = len(ip) - 1
    b = S.rhs_normal(PROBLEM_SEED, n)
    return prob.eps, prob.theta, ip, ix, v, n, b


def oracle_headline_problem():
    """The same problem from the oracle's restatement of the generators
    (bit-identical arrays), so that the reference arm never loads the device
    library."""
    from oracle import oracle_ffi as O

    _, eps, theta = O.sample_problem(PROBLEM_SEED)
    ip, ix, v = O.generate("aniso_q1", SIDE, SIDE, param0=eps, param1=theta)
    n = len(ip) - 1
    b = O.rhs_normal(PROBLEM_SEED, n)
    return eps, theta, ip, ix, v, n, b


def workload_desc(eps, theta, n, nnz):
    return (f"2D anisotropic Q1 diffusion {SIDE}x{SIDE} (n={n:,}, nnz={nnz:,}), eps={eps:.2f}, "
            f"theta={theta:.4f} (held-out seed {PROBLEM_SEED}), b~N(0,1) from the seed, x0=0, "
            f"stop at FP64 true relative residual {TOL:g}")


def host_info():
    """CPU model, logical CPUs and the CPUs this process may use."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if model is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    usable = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    return {"cpu_model": model, "nproc": os.cpu_count(), "usable_cpus": usable,
            "machine": os.uname().machine}


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, name in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def build_problem():
    import scirs_gb300 as S

    ip, ix, v = S.generate("laplace3d", GRID, GRID, GRID)
    n = len(ip) - 1
    b = S.rhs_normal(SEED, n)
    return ip, ix, v, n, b


# ------------------------------------------------------------ reference arm
def oracle_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def cpu_reference_solve(ip, ix, v, n, b, max_iter, threads):
    """The oracle's restatement of the reference cg + Jacobi (FP64), timed.
    Row-parallel SpMV and elementwise loops on `threads` host threads
    (bit-identical to one thread); every reduction is the reference's serial
    left fold."""
    from oracle import oracle_ffi as O

    O.set_threads(threads)
    a = O.op_csr_i32(ip, ix, v, (n, n))
    m = O.op_jacobi(a)
    t0 = time.perf_counter()
    r = O.cg(a, b, max_iter=max_iter, rtol=TOL, atol=0.0, preconditioner=m)
    dt = time.perf_counter() - t0
    return r, dt


def max_over_ranks(value, dist, device):
    """The slowest rank's time: with replicas every rank times the same step,
    and the job's step ends when the last replica's does."""
    if not dist:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """The reference's method -- cg with a Jacobi preconditioner in FP64
    (iterative.rs:40-162, preconditioners.rs:14-92) -- as the oracle restates
    it, on the host cores, on the headline problem.  Every timed step is one
    complete solve from x0 = 0 to the FP64 target; the warm-up steps are
    short solves.  Inputs come from the oracle's generators: the device
    library is never loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle_ffi as O

    eps, theta, ip, ix, v, n, b = oracle_headline_problem()
    nnz = len(v)
    threads = oracle_threads()
    for _ in range(args.warmup):
        cpu_reference_solve(ip, ix, v, n, b, 20, threads)
    times, iters, r = [], [], None
    for _ in range(args.steps):
        r, dt = cpu_reference_solve(ip, ix, v, n, b, 200000, threads)
        times.append(dt)
        iters.append(int(r["iterations"]))
    value = statistics.mean(times)
    true_res = O.true_rel_residual(ip, ix, v, b, r["x"]) if r is not None else None
    sample = (f"complete solves: oracle cg+Jacobi FP64 (restatement of iterative.rs:40-162) from x0=0 to "
              f"the FP64 target, {iters[-1] if iters else 0} iterations each; SpMV and elementwise loops on "
              f"{threads} host threads (bit-identical to one thread), dot products and norms serial left "
              f"folds as in the reference")
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": workload_desc(eps, theta, n, nnz), "method": "Jacobi-PCG FP64 (reference cg)",
                   "iterations": iters[-1] if iters else None, "converged": bool(r["converged"]) if r else None,
                   "fp64_true_rel_residual": true_res, "step_s": times, "host": host_info()},
        "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------- device arm
def run_ours(args):
    import ctypes as C

    import torch

    import scirs_gb300 as S
    from scirs_gb300 import _lib as L
    from scirs_gb300 import learned as LR

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    eps, theta, ip, ix, v, n, b = headline_problem()
    nnz = len(v)
    ctx = S.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    a64 = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    net = LR.load_weights(ctx, WEIGHTS)
    b_dev = torch.from_numpy(b).to(dev)
    x_dev = torch.empty(n, dtype=torch.float64, device=dev)
    b_pin = torch.from_numpy(b).pin_memory()
    x_pin = torch.empty(n, dtype=torch.float64).pin_memory()
    flush = torch.ones(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    flush_out = torch.empty((), dtype=torch.float32, device=dev)

    def l2_flush():
        # read 512 MB (4x L2): evicts the previous step's lines without
        # leaving dirty lines behind for the next kernel to write back
        torch.sum(flush, dim=0, out=flush_out)

    torch.cuda.synchronize()

    def learned_step(b_ptr, x_ptr, mem):
        """FP32 copy of A, network forward + factor G, FP32 PCG with FP64
        residual replacement to the FP64 target."""
        a32 = a64.astype(np.float32)
        g32 = net.preconditioner(a32)
        o = L.IROptions()
        L.lib.sx_ir_options_default(C.byref(o))
        o.tol = TOL
        o.max_inner = 200000
        o.preconditioner = g32.handle
        o.a32 = a32.handle
        o.mode = L.SX_IR_REPLACE
        r = L.IRResult()
        rc = L.lib.sx_cg_mixed(ctx.handle, a64.handle, C.c_void_p(b_ptr), n, C.byref(o), C.c_void_p(x_ptr),
                               mem, C.byref(r))
        g32.close()
        a32.close()
        S.sparse._check(rc)
        return r

    def jacobi_step(b_ptr, x_ptr, mem):
        """The reference's method on the device: FP64 Jacobi-PCG."""
        m64 = S.jacobi(ctx, a64)
        o = L.CGOptions()
        L.lib.sx_cg_options_default(C.byref(o))
        o.max_iter, o.rtol, o.atol, o.preconditioner = 200000, TOL, 0.0, m64.handle
        r = L.IterResult()
        rc = L.lib.sx_cg(ctx.handle, a64.handle, C.c_void_p(b_ptr), n, C.byref(o), C.c_void_p(x_ptr), mem,
                         C.byref(r))
        m64.close()
        S.sparse._check(rc)
        return r

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        times = []
        launches0 = ctx.kernel_launches
        out = None
        for _ in range(steps):
            l2_flush()  # between steps, outside the events
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return times, out, ctx.kernel_launches - launches0

    dev_b, dev_x = b_dev.data_ptr(), x_dev.data_ptr()
    with ClockSampler(local) as clk:
        t_dev, res, launches = timed(lambda: learned_step(dev_b, dev_x, L.SX_MEM_DEVICE), args.steps,
                                     args.warmup)
    x_learned = x_dev.cpu().numpy()
    true_res = S.true_rel_residual(a64, b, x_learned)
    # e2e: b from pinned host memory in, x back to pinned host memory, inside the events
    t_e2e, _, _ = timed(lambda: learned_step(b_pin.data_ptr(), x_pin.data_ptr(), L.SX_MEM_HOST),
                        max(2, args.steps // 2), 1)
    # the reference's method on the same device
    t_jac, r_jac, _ = timed(lambda: jacobi_step(dev_b, dev_x, L.SX_MEM_DEVICE), max(2, args.steps // 2), 1)
    true_res_jac = S.true_rel_residual(a64, b, x_dev.cpu().numpy())
    # the same method in two kernels per iteration (A p by the recurrence
    # q = A z + beta q, the p-update in the SpMV's epilogue): the FP64 loop
    # fused as far as the FP32 one
    ctx.set_cg_recurrence(True)
    t_jacf, r_jacf, _ = timed(lambda: jacobi_step(dev_b, dev_x, L.SX_MEM_DEVICE), max(2, args.steps // 2), 1)
    ctx.set_cg_recurrence(False)
    true_res_jacf = S.true_rel_residual(a64, b, x_dev.cpu().numpy())

    def once(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1) / 1e3

    # setup share of the learned step, and the other preconditioners
    a32 = a64.astype(np.float32)
    g32, t_setup = once(lambda: net.preconditioner(a32))
    r_lm, t_lm_solve = once(lambda: S.cg_mixed(a64, b, tol=TOL, max_inner=200000, preconditioner=g32, a32=a32))
    g32.close()
    m32 = S.jacobi(ctx, a32)
    r_jm, t_jm = once(lambda: S.cg_mixed(a64, b, tol=TOL, max_inner=200000, preconditioner=m32, a32=a32))
    m32.close()
    ic0 = {}
    # textbook IC(0) always (54 iterations); the reference's factorisation
    # needs ~1,400 iterations of a level-scheduled triangular solve (--ic0)
    for variant, tb in ((("reference", False), ("textbook", True)) if args.ic0 else (("textbook", True),)):
        try:
            mi, t_mi = once(lambda: S.ic0(ctx, a64, textbook=tb))
        except S.SparseError as e:
            ic0[variant] = {"error": str(e)}
            continue
        r_ic, t_ic = once(lambda: S.cg(a64, b, max_iter=args.ic0_max_iter, rtol=TOL, atol=0.0, preconditioner=mi))
        ic0[variant] = {"s": t_ic + t_mi, "setup_s": t_mi, "iterations": r_ic.iterations,
                        "converged": r_ic.converged, "fp64_true_rel_residual": S.true_rel_residual(a64, b, r_ic.x)}
        mi.close()

    # roofline: the dominant kernel of the step, the FP32 SpMV of A, alone
    peak, peak_kind = load_peaks()

    def spmv_time(op, nn, dt, flags=1, reps=20):
        tdt = torch.float32 if dt == np.float32 else torch.float64
        xb = torch.randn(nn, dtype=tdt, device=dev)
        yb = torch.empty(nn, dtype=tdt, device=dev)
        for _ in range(3):
            L.lib.sx_spmv_ex(ctx.handle, op.handle, C.c_void_p(xb.data_ptr()), C.c_void_p(yb.data_ptr()), flags)
        ts = []
        for _ in range(reps):
            l2_flush()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            # a ~0.1 ms spin on the stream first: the host enqueues the start
            # event and the launch while it runs, so the events bracket the
            # kernel and not the host's call overhead
            with torch.cuda.stream(stream):
                torch.cuda._sleep(200000)
            e0.record(stream)
            S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, op.handle, C.c_void_p(xb.data_ptr()),
                                             C.c_void_p(yb.data_ptr()), flags))
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return statistics.median(ts)

    def spmv_stream_time(ops, nn, dt, flags=1, launches=60, reps=5):
        """Average launch duration over back-to-back launches that rotate
        over copies of the matrix and its vectors whose total exceeds L2, so
        every launch reads its operands from HBM; events bracket the whole run
        of launches (L2 flushed before each run)."""
        tdt = torch.float32 if dt == np.float32 else torch.float64
        xs = [torch.randn(nn, dtype=tdt, device=dev) for _ in ops]
        ys = [torch.empty(nn, dtype=tdt, device=dev) for _ in ops]
        for k in range(len(ops)):
            S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, ops[k].handle, C.c_void_p(xs[k].data_ptr()),
                                             C.c_void_p(ys[k].data_ptr()), flags))
        ts = []
        for _ in range(reps):
            l2_flush()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            # the device waits (about 40 us per launch at 2 GHz) until the host
            # has queued every launch, so the timed run measures the kernels
            # back to back, not the host's issue rate
            with torch.cuda.stream(stream):
                torch.cuda._sleep(80000 * launches)
            e0.record(stream)
            for j in range(launches):
                k = j % len(ops)
                L.lib.sx_spmv_ex(ctx.handle, ops[k].handle, C.c_void_p(xs[k].data_ptr()),
                                 C.c_void_p(ys[k].data_ptr()), flags)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3 / launches)
        return statistics.median(ts)

    b_a32, fmt_a32, kname = kernel_bytes(S, a32, ip, ix, 4)
    t_a32 = spmv_time(a32, n, np.float32)
    # copies of A in FP32 (with their own x, y) totalling more than twice L2
    copies = [a32] + [a64.astype(np.float32) for _ in range(max(1, int(2.2 * 129e6 / b_a32)))]
    t_a32_stream = spmv_stream_time(copies, n, np.float32)
    for op in copies:
        op.close()

    def sweep_entry(nbytes, t, t_stream=None):
        e = {"GB/s": nbytes / t / 1e9, "frac": nbytes / t / 1e9 / peak, "us": t * 1e6}
        if t_stream is not None:
            e.update({"stream_us": t_stream * 1e6, "stream_GB/s": nbytes / t_stream / 1e9,
                      "stream_frac": nbytes / t_stream / 1e9 / peak})
        return e

    sweep = {f"aniso_q1_{SIDE}_fp32": sweep_entry(b_a32, t_a32, t_a32_stream)}
    if args.sweep:
        lip, lix, lv = S.generate("laplace3d", GRID, GRID, GRID)
        ln = len(lip) - 1
        l64 = S.csr_from_arrays(ctx, lip, lix, lv, (ln, ln))
        l32 = l64.astype(np.float32)
        l32c = [l32] + [l64.astype(np.float32) for _ in range(3)]
        l64c = [l64] + [l64.astype(np.float64) for _ in range(2)]
        sweep[f"laplace3d_{GRID}_fp32"] = sweep_entry(kernel_bytes(S, l32, lip, lix, 4)[0],
                                                      spmv_time(l32, ln, np.float32),
                                                      spmv_stream_time(l32c, ln, np.float32))
        sweep[f"laplace3d_{GRID}_fp64"] = sweep_entry(kernel_bytes(S, l64, lip, lix, 8)[0],
                                                      spmv_time(l64, ln, np.float64),
                                                      spmv_stream_time(l64c, ln, np.float64))
        sweep[f"laplace3d_{GRID}_fp64_fma"] = sweep_entry(kernel_bytes(S, l64, lip, lix, 8, exact=False)[0],
                                                          spmv_time(l64, ln, np.float64, flags=0),
                                                          spmv_stream_time(l64c, ln, np.float64, flags=0))
        for op in l32c[1:] + l64c[1:]:
            op.close()
        # the same matrix stored as its lower triangle (SymCsrMatrix): merged
        # rows read as many bytes as the full CSR; the half-storage product
        # reads the lower triangle once (its bytes: lower entries, x, y)
        s64 = S.sym_csr_from_csr(l64)
        s32 = s64.astype(np.float32)
        lnnz = s64.nnz_stored()
        half_b = lambda w: lnnz * (w + 4) + 4 * (ln + 1) + 2 * ln * w  # noqa: E731
        sweep[f"laplace3d_{GRID}_sym_fp64"] = sweep_entry(kernel_bytes(S, l64, lip, lix, 8)[0],
                                                          spmv_time(s64, ln, np.float64))
        sweep[f"laplace3d_{GRID}_sym_fp32"] = sweep_entry(kernel_bytes(S, l32, lip, lix, 4)[0],
                                                          spmv_time(s32, ln, np.float32))
        sweep[f"laplace3d_{GRID}_sym_half_fp64"] = sweep_entry(half_b(8), spmv_time(s64, ln, np.float64, flags=2))
        sweep[f"laplace3d_{GRID}_sym_half_fp32"] = sweep_entry(half_b(4), spmv_time(s32, ln, np.float32, flags=2))
        s32.close()
        s64.close()
        l32.close()
        l64.close()
        pip, pix, pv = S.generate("powerlaw", 4194304, seed=1, param0=16.0, param1=4096.0)
        pn, pnnz = len(pip) - 1, len(pv)
        p64 = S.csr_from_arrays(ctx, pip, pix, pv, (pn, pn))
        p32 = p64.astype(np.float32)
        sweep["powerlaw_4M_fp32"] = sweep_entry(spmv_bytes(pn, pnnz, 4), spmv_time(p32, pn, np.float32, reps=10))
        sweep["powerlaw_4M_fp64"] = sweep_entry(spmv_bytes(pn, pnnz, 8), spmv_time(p64, pn, np.float64, reps=10))
        sweep["powerlaw_4M_fp64_fma"] = sweep_entry(spmv_bytes(pn, pnnz, 8),
                                                    spmv_time(p64, pn, np.float64, flags=0, reps=10))
        p32.close()
        p64.close()
        # the matrix's columns are uniform random: every nonzero gathers x at
        # an unpredictable address, so the bound is this GPU's random-gather
        # rate (measured live: pnnz gathers from an L2-resident x of pn
        # elements), not HBM
        rates = {}
        for dt in (0, 1):
            rate = C.c_double(0.0)
            S.sparse._check(L.lib.sx_probe_gather_rate(ctx.handle, dt, pn, pnnz, C.byref(rate)))
            rates[dt] = rate.value
        for key, dt in (("powerlaw_4M_fp32", 0), ("powerlaw_4M_fp64", 1), ("powerlaw_4M_fp64_fma", 1)):
            bound_us = pnnz / rates[dt] * 1e6
            sweep[key]["gather_bound"] = {"Ggathers_per_s": rates[dt] / 1e9, "bound_us": bound_us,
                                          "frac": bound_us / sweep[key]["us"]}

    workloads = run_workloads(ctx, S, once, args) if args.workloads else None

    traffic = None
    prof = os.path.join(REPO, "profiles", f"spmv_aniso_q1_{SIDE}_fp32.txt")
    if os.path.exists(prof):
        for line in open(prof):
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = float(line.split(":")[1])

    # CPU baseline: one complete oracle solve of the headline problem (the
    # reference arm's step), then the other configurations' CPU rows
    cpu, cpu_rows = None, None
    if rank == 0 and not args.no_cpu_baseline:
        threads = oracle_threads()
        rc_, dt = cpu_reference_solve(ip, ix, v, n, b, 200000, threads)
        cpu = {"value": dt, "unit": "s", "cores": threads, "kind": "port",
               "sample": f"one complete oracle cg+Jacobi FP64 solve of the headline problem "
                         f"({int(rc_['iterations'])} iterations); SpMV and elementwise loops on {threads} host "
                         f"threads (bit-identical to one thread), reductions serial as in the reference"}
        cpu_rows = run_cpu_rows(threads, workloads or {})

    value = max_over_ranks(statistics.mean(t_dev), dist, dev)
    jac = statistics.mean(t_jac)
    jacf = statistics.mean(t_jacf)
    jacf_iter_s = jacf / max(int(r_jacf.iterations), 1)
    # K1: A (layout), z gathered once, p read and written, q read (written as y);
    # K2: x, r read and written, p, q, D read, z written
    jacf_bytes = dia_bytes(n, 9, 8) + 11 * n * 8
    # FP64 Jacobi-PCG per iteration on the diagonal layout: A (9 FP64 values
    # + the 2-byte mask per row), p read and Ap written by the SpMV; the
    # update reads x, p, r, Ap, 1/diag and writes x, r; the p step reads r,
    # 1/diag, p and writes p
    jac_iter_s = jac / max(int(r_jac.iterations), 1)
    jac_bytes = dia_bytes(n, 9, 8) + 7 * n * 8 + 4 * n * 8
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 Krylov vectors and A copy / f16 values of the learned factor G (widened to f32) / "
                 "f64 residual, outer inner products and solution",
        "data": "synthetic",
        "config": {"workload": workload_desc(eps, theta, n, nnz),
                   "method": "learned factorised SAI (GNN weights scirs_gb300/weights/aniso_q1.npz) + FP32 PCG "
                             "with FP64 residual replacement; step includes the FP32 copy and the network setup",
                   "outer_iterations": int(res.outer_iterations), "inner_iterations": int(res.inner_iterations),
                   "fp64_true_rel_residual": true_res,
                   "setup_s": t_setup, "solve_s": t_lm_solve,
                   "l2": "working set > L2 (129 MB) and a 512 MB L2 flush between steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "speedup_vs_jacobi_fp64": jac / value,
        "speedup_vs_jacobi_fp64_fused": jacf / value,
        "baseline_note": (f"the fastest FP64 Jacobi-PCG here (two kernels per iteration) runs at "
                          f"{jacf_bytes / jacf_iter_s / 1e9 / peak:.2f} of HBM, not 0.6: its SpMV keeps "
                          f"GB300's FP64 pipe busy (two FP64 lanes per clock per SM), so the speed-up over "
                          f"it, {jacf / value:.2f}x, is against an FP64-pipe-bound baseline"),
        "learned_vs_jacobi_mixed": t_jm / value,
        "jacobi_pcg_fp64": {"value": jac, "unit": "s", "iterations": int(r_jac.iterations),
                            "us_per_iteration": jac_iter_s * 1e6, "bytes_per_iteration": jac_bytes,
                            "GB/s": jac_bytes / jac_iter_s / 1e9, "frac": jac_bytes / jac_iter_s / 1e9 / peak,
                            "fp64_true_rel_residual": true_res_jac},
        "jacobi_pcg_fp64_fused": {"value": jacf, "unit": "s", "iterations": int(r_jacf.iterations),
                                  "us_per_iteration": jacf_iter_s * 1e6, "bytes_per_iteration": jacf_bytes,
                                  "GB/s": jacf_bytes / jacf_iter_s / 1e9,
                                  "frac": jacf_bytes / jacf_iter_s / 1e9 / peak,
                                  "kernels_per_iteration": 2, "fp64_true_rel_residual": true_res_jacf},
        "jacobi_pcg_mixed": {"value": t_jm, "unit": "s", "outer_iterations": r_jm.outer_iterations,
                             "inner_iterations": r_jm.inner_iterations, "fp64_true_rel_residual": r_jm.rel_residual},
        "e2e": {"value": statistics.mean(t_e2e), "unit": "s", "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": n * 8},
        "roofline": {"bound": "hbm", "kernel": f"FP32 SpMV of A (aniso Q1 {SIDE}^2), {kname}",
                     "achieved": b_a32 / t_a32_stream / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": b_a32 / t_a32_stream / 1e9 / peak, "peak_source": peak_kind,
                     "algorithmic_bytes": b_a32, "format": fmt_a32,
                     "launch_us": t_a32_stream * 1e6,
                     "timing": "average launch duration over 60 back-to-back launches rotating over "
                               f"{len(copies)} copies of A, x, y (> 2x L2), L2 flushed before each run; "
                               "each launch programmatic (it loads its values while the previous one "
                               "finishes, and waits for it on the device before reading x); "
                               f"a single event-bracketed launch takes {t_a32 * 1e6:.2f} us "
                               f"({b_a32 / t_a32 / 1e9 / peak:.3f} of peak)",
                     "csr_equivalent_bytes": spmv_bytes(n, nnz, 4), "traffic": traffic},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "host": host_info(),
        "ic0_pcg_fp64": ic0,
        "spmv_sweep": sweep,
        "workloads": workloads,
        "cpu_rows": cpu_rows,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    net.close()
    a64.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()


def run_cpu_rows(threads, dev):
    """The other configurations on the host cores through the oracle (the
    reference's algorithms restated; SpMV and elementwise loops on `threads`
    threads, bit-identical to one).  Solves that take minutes on the CPU are
    sampled and scaled, and say so."""
    from oracle import oracle_ffi as O

    O.set_threads(threads)
    rows = {"threads": threads}

    def med(fn, reps):
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts)

    # 2D Poisson 256^2, FP64 Jacobi-PCG, complete solve
    ip, ix, v = O.generate("poisson2d", 256, 256)
    n = len(ip) - 1
    b = O.rhs_normal(0, n)
    a = O.op_csr_i32(ip, ix, v, (n, n))
    t0 = time.perf_counter()
    r = O.cg(a, b, max_iter=5000, rtol=TOL, atol=0.0, preconditioner=O.op_jacobi(a))
    t = time.perf_counter() - t0
    row = {"s": t, "iterations": int(r["iterations"]), "converged": bool(r["converged"])}
    g = dev.get("poisson2d_256_jacobi_fp64")
    if g:
        row["gpu_s"] = g["s"]
        row["gpu_iterations"] = g["iterations"]
    rows["poisson2d_256_jacobi_fp64"] = row
    # SpMV: 3D 7-point 128^3 and the 4M-row power-law matrix, FP64 and FP32
    for name, gen in ((f"laplace3d_{GRID}", lambda: O.generate("laplace3d", GRID, GRID, GRID)),
                      ("powerlaw_4M", lambda: O.generate("powerlaw", 4194304, seed=1, param0=16.0, param1=4096.0))):
        ip, ix, v = gen()
        n = len(ip) - 1
        x = O.rhs_normal(3, n)
        for dt in (np.float64, np.float32):
            vv, xx = v.astype(dt), x.astype(dt)
            w = 8 if dt == np.float64 else 4
            tm = med(lambda: O.spmv_i32(ip, ix, vv, xx), 3)
            rows[f"spmv_{name}_{'fp64' if w == 8 else 'fp32'}"] = {
                "ms": tm * 1e3, "GB/s": spmv_bytes(n, len(ix), w) / tm / 1e9}
        del ip, ix, v
    # 3D variable-coefficient 160^3, FP64 cg + Jacobi to 1e-10: the first
    # iterations, scaled to the device's FP64 count
    ip, ix, v = O.generate("varcoef3d", 160, 160, 160, seed=SEED, param0=1.5)
    n = len(ip) - 1
    b = O.rhs_normal(SEED, n)
    a = O.op_csr_i32(ip, ix, v, (n, n))
    m = O.op_jacobi(a)
    k = 100
    t0 = time.perf_counter()
    O.cg(a, b, max_iter=k, rtol=1e-10, atol=0.0, preconditioner=m)
    t = time.perf_counter() - t0
    g = dev.get("varcoef3d_160_fp64_1e-10")
    full = g["iterations"] if g else None
    rows["varcoef3d_160_cg_fp64_1e-10"] = {
        "s_per_iteration": t / k, "s": t / k * full if full else None, "iterations": full,
        "sample": f"first {k} iterations timed, scaled to the device FP64 Jacobi-PCG iteration count"}
    del a, m, ip, ix, v
    # batched: the reference runs one cg per system; complete solves of the
    # first systems, scaled to the 4096 by the sum of side^3 (rows x iterations)
    sides = O.batch_sides(4096, 32, 256, SEED)
    ns, t = 8, 0.0
    its = []
    offs = np.concatenate([[0], np.cumsum(sides[:ns] ** 2)])
    b_all = O.rhs_normal(SEED, int(offs[-1]))  # the batch's b restricted to these systems
    for sidx in range(ns):
        ip, ix, v = O.batch_system(sidx, int(sides[sidx]), SEED, 1.0)
        n = len(ip) - 1
        b = b_all[offs[sidx]:offs[sidx + 1]]
        a = O.op_csr_i32(ip, ix, v, (n, n))
        t0 = time.perf_counter()
        r = O.cg(a, b, max_iter=20000, rtol=TOL, atol=0.0, preconditioner=O.op_jacobi(a))
        t += time.perf_counter() - t0
        its.append(int(r["iterations"]))
    cube = sides.astype(np.float64) ** 3
    rows["batched_4096_cg_fp64"] = {"s_sample": t, "systems_sampled": ns, "iterations": its,
                                    "s": t * cube.sum() / cube[:ns].sum(),
                                    "sample": f"complete FP64 Jacobi-PCG solves of the first {ns} systems, "
                                              f"scaled to 4096 by the sum of side^3"}
    # the reference IC(0) apply (ic.rs:163-214: the backward solve scans every
    # row for each unknown, O(n^2)) on 2D Q1 problems, extrapolated to 1024^2
    pts = []
    for side in (48, 64, 96):
        ip, ix, v = O.generate("aniso_q1", side, side, param0=845.08, param1=0.9632)
        n = len(ip) - 1
        a = O.op_csr_i32(ip, ix, v, (n, n))
        try:
            mi = O.op_ic0(a, fast=False)
        except Exception as e:  # the quirky factorisation may break down
            rows["ic0_reference_apply"] = {"error": str(e)}
            pts = []
            break
        x = O.rhs_normal(5, n)
        pts.append((n, med(lambda: mi.matvec(x), 2)))
    if pts:
        ex = float(np.polyfit(np.log([q[0] for q in pts]), np.log([q[1] for q in pts]), 1)[0])
        n_big = SIDE * SIDE
        t_big = pts[-1][1] * (n_big / pts[-1][0]) ** ex
        rows["ic0_reference_apply"] = {"points": [{"n": q[0], "s": q[1]} for q in pts], "exponent": ex,
                                       "s_per_apply_at_1024^2": t_big,
                                       "sample": "apply times on 48^2, 64^2, 96^2 Q1 grids, power-law fit, "
                                                 "extrapolated to n = 1,048,576"}
    return rows


def run_workloads(ctx, S, once, args):
    """The other configurations, one timed run each (FP64 true residuals)."""
    out = {}
    # 2D 5-point Poisson 256^2, FP64 Jacobi-PCG (L2-resident, latency-bound)
    ip, ix, v = S.generate("poisson2d", 256, 256)
    n = len(ip) - 1
    b = S.rhs_normal(0, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    m = S.jacobi(ctx, a)
    S.cg(a, b, max_iter=5000, rtol=TOL, atol=0.0, preconditioner=m)  # graph capture outside the timing
    r, t = once(lambda: S.cg(a, b, max_iter=5000, rtol=TOL, atol=0.0, preconditioner=m))
    out["poisson2d_256_jacobi_fp64"] = {"s": t, "iterations": r.iterations, "us_per_iteration": t / max(r.iterations, 1) * 1e6,
                                        "fp64_true_rel_residual": S.true_rel_residual(a, b, r.x)}
    m.close()
    a.close()
    # 3D 7-point Laplacian 128^3: mixed precision vs FP64 Jacobi-PCG
    ip, ix, v = S.generate("laplace3d", GRID, GRID, GRID)
    n = len(ip) - 1
    b = S.rhs_normal(SEED, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    a32 = a.astype(np.float32)
    m32, m64 = S.jacobi(ctx, a32), S.jacobi(ctx, a)
    S.cg_mixed(a, b, tol=TOL, preconditioner=m32, a32=a32)
    r, t = once(lambda: S.cg_mixed(a, b, tol=TOL, preconditioner=m32, a32=a32))
    S.cg(a, b, max_iter=20000, rtol=TOL, atol=0.0, preconditioner=m64)
    r64, t64 = once(lambda: S.cg(a, b, max_iter=20000, rtol=TOL, atol=0.0, preconditioner=m64))
    out["laplace3d_128_jacobi"] = {"mixed_s": t, "mixed_inner_iterations": r.inner_iterations,
                                   "mixed_outer_iterations": r.outer_iterations,
                                   "mixed_fp64_true_rel_residual": r.rel_residual,
                                   "fp64_s": t64, "fp64_iterations": r64.iterations}
    for op in (m32, m64, a32, a):
        op.close()
    # 3D variable-coefficient 160^3, mixed precision to 1e-10
    ip, ix, v = S.generate("varcoef3d", 160, 160, 160, seed=SEED, param0=1.5)
    n = len(ip) - 1
    b = S.rhs_normal(SEED, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    a32 = a.astype(np.float32)
    m32 = S.jacobi(ctx, a32)
    S.cg_mixed(a, b, tol=1e-10, max_inner=100000, preconditioner=m32, a32=a32)
    r, t = once(lambda: S.cg_mixed(a, b, tol=1e-10, max_inner=100000, preconditioner=m32, a32=a32))
    out["varcoef3d_160_mixed_1e-10"] = {"s": t, "inner_iterations": r.inner_iterations,
                                        "outer_iterations": r.outer_iterations, "converged": r.converged,
                                        "fp64_true_rel_residual": r.rel_residual}
    # the same problem in plain FP64 Jacobi-PCG (the reference's method)
    m64 = S.jacobi(ctx, a)
    S.cg(a, b, max_iter=100000, rtol=1e-10, atol=0.0, preconditioner=m64)
    r, t = once(lambda: S.cg(a, b, max_iter=100000, rtol=1e-10, atol=0.0, preconditioner=m64))
    out["varcoef3d_160_fp64_1e-10"] = {"s": t, "iterations": r.iterations, "converged": r.converged,
                                       "fp64_true_rel_residual": S.true_rel_residual(a, b, r.x)}
    m64.close()
    m32.close()
    a32.close()
    a.close()
    if args.batched:
        sys_ptr, ip, ix, v = S.generate_batch(4096, 32, 256, seed=SEED, sigma=1.0)
        n = len(ip) - 1
        b = S.rhs_normal(SEED, n)
        a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        del ix, v
        a32 = a.astype(np.float32)
        S.batched_pcg(a, sys_ptr, b, rtol=TOL, a32=a32)  # autotune and first-launch costs outside the timing
        r, t = once(lambda: S.batched_pcg(a, sys_ptr, b, rtol=TOL, a32=a32))
        # algorithmic bytes of the FP32 inner iterations (the dominant part):
        # per iteration of a system with m rows and z nonzeros, 8 z (values,
        # columns) + 4 (m + 1) (row pointers) + 52 m (z gathered once, p and q
        # read and written, then d, r read and written, p, q, 1/diag read, z
        # written)
        rows_s = np.diff(sys_ptr)
        nnz_s = ip[sys_ptr[1:]] - ip[sys_ptr[:-1]]
        inner_bytes = float(np.sum(r.inner_iterations * (8.0 * nnz_s + 4.0 * (rows_s + 1) + 52.0 * rows_s)))
        out["batched_4096_varcoef2d"] = {"s": t, "systems": 4096, "rows": n, "nnz": a.nnz,
                                         "converged": int(r.converged.sum()),
                                         "max_rel_residual": float(r.rel_residual.max()),
                                         "max_inner_iterations": int(r.inner_iterations.max()),
                                         "total_inner_iterations": int(r.inner_iterations.sum()),
                                         "outer_iterations": r.outer_iterations,
                                         "inner_algorithmic_bytes": inner_bytes,
                                         "inner_GB/s": inner_bytes / t / 1e9,
                                         "frac": inner_bytes / t / 1e9 / load_peaks()[0],
                                         "launch_shape": {"threads_per_block": r.threads_per_block,
                                                          "blocks_per_sm": r.blocks_per_sm,
                                                          "chosen_by": "autotuner"}}
        a32.close()
        a.close()
    return out


def run_profile(args):
    """A few launches of one kernel for ncu (small, self-contained)."""
    import torch

    import scirs_gb300 as S
    from scirs_gb300 import _lib as L
    import ctypes as C

    ctx = S.Context(0)
    if args.profile == "solve":
        ip, ix, v, n, b = build_problem()
        a64 = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        a32 = a64.astype(np.float32)
        m32 = S.jacobi(ctx, a32)
        for _ in range(args.steps):
            r = S.cg_mixed(a64, b, tol=TOL, inner_rtol=args.inner_rtol, preconditioner=m32, a32=a32)
        print(json.dumps({"profile": "solve", "n": n, "outer": r.outer_iterations,
                          "inner": r.inner_iterations, "rel_residual": r.rel_residual}))
        for op in (m32, a32, a64):
            op.close()
        ctx.close()
        return
    if args.profile == "learned":
        from scirs_gb300 import learned as LR

        _, _, ip, ix, v, n, b = headline_problem()
        a64 = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        net = LR.load_weights(ctx, WEIGHTS)
        for _ in range(args.steps):
            a32 = a64.astype(np.float32)
            g32 = net.preconditioner(a32)
            r = S.cg_mixed(a64, b, tol=TOL, max_inner=200000, preconditioner=g32, a32=a32)
            g32.close()
            a32.close()
        print(json.dumps({"profile": "learned", "n": n, "outer": r.outer_iterations,
                          "inner": r.inner_iterations, "rel_residual": r.rel_residual}))
        net.close()
        a64.close()
        ctx.close()
        return
    if args.profile in ("jacobi64", "jacobi64fused", "jacobi32mixed"):
        _, _, ip, ix, v, n, b = headline_problem()
        a64 = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
        a32 = a64.astype(np.float32)
        m = S.jacobi(ctx, a64 if args.profile != "jacobi32mixed" else a32)
        ctx.set_cg_recurrence(args.profile == "jacobi64fused")
        for _ in range(args.steps):
            if args.profile != "jacobi32mixed":
                r = S.cg(a64, b, max_iter=200000, rtol=TOL, atol=0.0, preconditioner=m)
                its = r.iterations
            else:
                r = S.cg_mixed(a64, b, tol=TOL, max_inner=200000, preconditioner=m, a32=a32)
                its = r.inner_iterations
        print(json.dumps({"profile": args.profile, "n": n, "iterations": its}))
        for op in (m, a32, a64):
            op.close()
        ctx.close()
        return
    if args.profile in ("spmv32", "spmv64") or args.profile.startswith("sym"):
        ip, ix, v = S.generate("laplace3d", GRID, GRID, GRID)
    elif args.profile == "aniso32":
        _, _, ip, ix, v, _, _ = headline_problem()
    else:
        ip, ix, v = S.generate("powerlaw", 4194304, seed=1, param0=16.0, param1=4096.0)
    n = len(ip) - 1
    dt = np.float64 if args.profile.endswith("64") else np.float32
    a = S.csr_from_arrays(ctx, ip, ix, v.astype(dt), (n, n))
    flags = 1
    if args.profile.startswith("sym"):
        # lower-triangle storage: merged rows (exact) or the half-storage scatter
        full = a
        a = S.sym_csr_from_csr(full)
        full.close()
        flags = 2 if "half" in args.profile else 1
    tdt = torch.float64 if dt == np.float64 else torch.float32
    x = torch.randn(n, dtype=tdt, device="cuda")
    y = torch.empty(n, dtype=tdt, device="cuda")
    for _ in range(args.steps):
        S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, a.handle, C.c_void_p(x.data_ptr()),
                                         C.c_void_p(y.data_ptr()), flags))
    ctx.synchronize()
    print(json.dumps({"profile": args.profile, "n": n, "nnz": len(v), "launches": args.steps}))
    a.close()
    ctx.close()


# ---------------- learned SAI vs Jacobi (2D anisotropic Q1, held-out seeds)
WEIGHTS = os.path.join(REPO, "scirs_gb300", "weights", "aniso_q1.npz")


def eval_learned(ctx, net, side, seeds, max_iter=400000, with_fp64_learned=True, log=None, ic0_max_iter=0):
    """Held-out anisotropic Q1 problems: time to FP64 relative residual 1e-8 for
    FP64 Jacobi-PCG, mixed-precision Jacobi-PCG and mixed-precision learned PCG
    (falling back to FP64 learned PCG if refinement stagnates)."""
    import torch

    import scirs_gb300 as S
    from scirs_gb300 import learned as LR

    stream = torch.cuda.ExternalStream(ctx.stream)

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1) / 1e3

    rows = []
    for sd in seeds:
        prob = LR.sample_problem(sd)
        a64 = LR.build(ctx, prob, side=side)
        a32 = a64.astype(np.float32)
        n = a64.shape[0]
        b = S.rhs_normal(sd, n)
        row = {"seed": sd, "eps": prob.eps, "theta": prob.theta, "n": n, "nnz": a64.nnz}
        m64 = S.jacobi(ctx, a64)
        r, t = timed(lambda: S.cg(a64, b, max_iter=max_iter, rtol=TOL, atol=0.0, preconditioner=m64))
        row["jacobi_fp64"] = {"s": t, "iters": r.iterations, "conv": r.converged,
                              "true_res": S.true_rel_residual(a64, b, r.x)}
        for variant, tb in ((("ic0_reference_fp64", False), ("ic0_textbook_fp64", True)) if ic0_max_iter else ()):
            try:
                mi, t_setup = timed(lambda: S.ic0(ctx, a64, textbook=tb))
            except S.SparseError as e:
                row[variant] = {"error": str(e)}
                continue
            r, t = timed(lambda: S.cg(a64, b, max_iter=ic0_max_iter, rtol=TOL, atol=0.0, preconditioner=mi))
            row[variant] = {"s": t, "setup_s": t_setup, "iters": r.iterations, "conv": r.converged,
                            "true_res": S.true_rel_residual(a64, b, r.x)}
            mi.close()
        m32 = S.jacobi(ctx, a32)
        r, t = timed(lambda: S.cg_mixed(a64, b, tol=TOL, inner_rtol=1e-4, max_inner=max_iter,
                                        preconditioner=m32, a32=a32))
        row["jacobi_mixed"] = {"s": t, "outer": r.outer_iterations, "inner": r.inner_iterations,
                               "conv": r.converged, "true_res": r.rel_residual}
        if net is not None:
            g32, t_setup = timed(lambda: net.preconditioner(a32))
            r, t = timed(lambda: S.cg_mixed(a64, b, tol=TOL, inner_rtol=1e-4, max_inner=max_iter,
                                            preconditioner=g32, a32=a32))
            row["learned_mixed"] = {"s": t, "setup_s": t_setup, "outer": r.outer_iterations,
                                    "inner": r.inner_iterations, "conv": r.converged,
                                    "true_res": r.rel_residual}
            if with_fp64_learned or not r.converged:
                g64, t_setup64 = timed(lambda: net.preconditioner(a64))
                r, t = timed(lambda: S.cg(a64, b, max_iter=max_iter, rtol=TOL, atol=0.0,
                                          preconditioner=g64))
                row["learned_fp64"] = {"s": t, "setup_s": t_setup64, "iters": r.iterations,
                                       "conv": r.converged, "true_res": S.true_rel_residual(a64, b, r.x)}
                g64.close()
            g32.close()
        for op in (m32, m64, a32, a64):
            op.close()
        rows.append(row)
        if log:
            log(json.dumps(row))
    return rows


def run_learned(args):
    import scirs_gb300 as S
    from scirs_gb300 import learned as LR

    ctx = S.Context(0)
    log = lambda s: print(s, file=sys.stderr, flush=True)  # noqa: E731
    train_log = None
    if args.train_gnn:
        t0 = time.perf_counter()
        net, train_log = LR.train(ctx, args.train_gnn, seed=args.train_seed, log_every=100)
        t_train = time.perf_counter() - t0
        out = os.path.abspath(args.weights_out)
        os.makedirs(os.path.dirname(out), exist_ok=True)
        LR.save_weights(out, net, {"steps": args.train_gnn, "seed": args.train_seed, "train_s": t_train})
        log(json.dumps({"trained_steps": args.train_gnn, "train_s": t_train, "log": train_log[-5:]}))
    elif os.path.exists(WEIGHTS):
        net = LR.load_weights(ctx, WEIGHTS)
    else:
        net = None
    seeds = [int(s) for s in args.eval_seeds.split(",")]
    rows = eval_learned(ctx, net, args.eval_side, seeds, log=log,
                        ic0_max_iter=args.ic0_max_iter if args.ic0 else 0)
    print(json.dumps({"eval_side": args.eval_side, "rows": rows}), flush=True)
    if net is not None:
        net.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--inner-rtol", type=float, default=1e-4)
    ap.add_argument("--no-sweep", dest="sweep", action="store_false")
    ap.add_argument("--no-workloads", dest="workloads", action="store_false")
    ap.add_argument("--no-batched", dest="batched", action="store_false")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ic0", action="store_true", help="also time IC(0)-PCG with the reference's factorisation")
    ap.add_argument("--ic0-max-iter", type=int, default=3000)
    ap.add_argument("--profile", default=None,
                    choices=["spmv32", "spmv64", "powerlaw32", "powerlaw64", "aniso32", "solve", "learned",
                             "jacobi64", "jacobi64fused", "jacobi32mixed", "sym64", "sym32", "symhalf64", "symhalf32"],
                    help="run a few launches of one SpMV for an ncu capture and exit")
    ap.add_argument("--workload", default="laplace3d", choices=["laplace3d", "learned"])
    ap.add_argument("--train-gnn", type=int, default=0, help="train the network for N steps first")
    ap.add_argument("--weights-out", default=os.path.join(REPO, "trained", "aniso_q1.npz"),
                    help="where --train-gnn writes the trained weights")
    ap.add_argument("--train-seed", type=int, default=0)
    ap.add_argument("--eval-side", type=int, default=1024)
    ap.add_argument("--eval-seeds", default="1000001,1000002,1000003,1000004")
    args = ap.parse_args()
    if args.workload == "learned":
        run_learned(args)
    elif args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
