"""Benchmark of the scirs2-sparse iterative-solve path on one GB300.

Metric: time to an FP64-verified relative residual of 1e-8 (learned vs
Jacobi PCG), plus SpMV HBM GB/s.  Workload: 3D 7-point Laplacian on a 128^3
grid (n = 2,097,152, nnz = 14,581,760), b ~ N(0, 1) from seed 0, x0 = 0.

A step is one complete solve from b to x.  `value` times the solve with A,
b and x resident on the device; `e2e` times the same solve through the
C ABI with b copied from pinned host memory and x copied back inside the
timed region.  `roofline` times the dominant kernel (the FP32 CSR SpMV of
the inner solver) alone with CUDA events on the library's stream.
`cpu_baseline` times the CPU oracle (a restatement of the reference's cg
with Jacobi, single-threaded like the reference) on a bounded sample.

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
GRID = 128
SEED = 0
TOL = 1e-8


def spmv_bytes(n: int, nnz: int, w: int) -> int:
    # nnz (w + 4) + 4 (n + 1) + 2 n w  (int32 indices, x read once, y written once)
    return nnz * (w + 4) + 4 * (n + 1) + 2 * n * w


def workload_desc(n, nnz):
    return (f"3D 7-point Laplacian {GRID}^3 (n={n:,}, nnz={nnz:,}), b~N(0,1) seed {SEED}, x0=0, "
            f"stop at FP64 true relative residual {TOL:g}")


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
def cpu_reference_solve(ip, ix, v, n, b, max_iter):
    """The oracle's restatement of the reference cg + Jacobi (FP64), timed."""
    from oracle import oracle_ffi as O

    a = O.op_csr_i32(ip, ix, v, (n, n))
    m = O.op_jacobi(a)
    t0 = time.perf_counter()
    r = O.cg(a, b, max_iter=max_iter, rtol=TOL, atol=0.0, preconditioner=m)
    dt = time.perf_counter() - t0
    return r, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    ip, ix, v, n, b = build_problem()
    nnz = len(v)
    # warm-up: one full solve gives the iteration count at convergence
    full, t_full = cpu_reference_solve(ip, ix, v, n, b, 100000)
    iters = full["iterations"]
    per_iter = t_full / max(iters, 1)
    sample_iters = iters if t_full <= 20.0 else max(20, int(20.0 / per_iter))
    for _ in range(max(0, args.warmup - 1)):
        cpu_reference_solve(ip, ix, v, n, b, sample_iters)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_reference_solve(ip, ix, v, n, b, sample_iters)
        times.append(dt * iters / sample_iters)
    value = statistics.mean(times)
    sample = (f"oracle cg+Jacobi FP64 (restatement of iterative.rs:40-162), {sample_iters} of {iters} "
              f"iterations per step, scaled to {iters}; single thread like the reference")
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": workload_desc(n, nnz), "method": "Jacobi-PCG FP64 (reference cg)",
                   "iterations": iters},
        "cpu_baseline": {"value": value, "unit": "s", "cores": 1, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------- device arm
def run_ours(args):
    import torch

    import scirs_gb300 as S
    from scirs_gb300 import _lib as L

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    ip, ix, v, n, b = build_problem()
    nnz = len(v)
    ctx = S.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    a64 = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    a32 = a64.astype(np.float32)
    m32 = S.jacobi(ctx, a32)
    m64 = S.jacobi(ctx, a64)
    dev = torch.device("cuda", local)
    b_dev = torch.from_numpy(b).to(dev)
    x_dev = torch.empty(n, dtype=torch.float64, device=dev)
    b_pin = torch.from_numpy(b).pin_memory()
    x_pin = torch.empty(n, dtype=torch.float64).pin_memory()
    flush = torch.ones(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    flush_out = torch.empty(1, dtype=torch.float32, device=dev)

    def l2_flush():
        # read 512 MB (4x L2): evicts the previous step's lines without
        # leaving dirty lines behind for the next kernel to write back
        torch.sum(flush, dim=0, out=flush_out)

    torch.cuda.synchronize()

    import ctypes as C

    def solve_mixed(b_ptr, x_ptr, mem):
        o = L.IROptions()
        L.lib.sx_ir_options_default(C.byref(o))
        o.tol = TOL
        o.inner_rtol = args.inner_rtol
        o.max_inner = 20000
        o.preconditioner = m32.handle
        o.a32 = a32.handle
        r = L.IRResult()
        rc = L.lib.sx_cg_mixed(ctx.handle, a64.handle, C.c_void_p(b_ptr), n, C.byref(o), C.c_void_p(x_ptr),
                               mem, C.byref(r))
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

    # device-resident solve (value)
    with ClockSampler(local) as clk:
        t_dev, res, launches = timed(lambda: solve_mixed(b_dev.data_ptr(), x_dev.data_ptr(), L.SX_MEM_DEVICE),
                                     args.steps, args.warmup)
    x = x_dev.cpu().numpy()
    true_res = S.true_rel_residual(a64, b, x)
    # end-to-end through the C ABI with host buffers (e2e)
    t_e2e, res_e2e, _ = timed(lambda: solve_mixed(b_pin.data_ptr(), x_pin.data_ptr(), L.SX_MEM_HOST),
                              args.steps, max(1, args.warmup // 2))
    # plain FP64 Jacobi-PCG on the same GPU (the comparison method)
    def solve_fp64():
        o = L.CGOptions()
        L.lib.sx_cg_options_default(C.byref(o))
        o.max_iter, o.rtol, o.atol, o.preconditioner = 100000, TOL, 0.0, m64.handle
        r = L.IterResult()
        S.sparse._check(L.lib.sx_cg(ctx.handle, a64.handle, C.c_void_p(b_dev.data_ptr()), n, C.byref(o),
                                    C.c_void_p(x_dev.data_ptr()), L.SX_MEM_DEVICE, C.byref(r)))
        return r

    t_j64, r_j64, _ = timed(solve_fp64, max(2, args.steps // 2), 1)
    true_res_j64 = S.true_rel_residual(a64, b, x_dev.cpu().numpy())

    # roofline: the inner FP32 SpMV alone, CUDA events on the library stream
    def spmv_time(op, xbuf, ybuf, reps=20):
        for _ in range(3):
            L.lib.sx_spmv_ex(ctx.handle, op.handle, C.c_void_p(xbuf.data_ptr()), C.c_void_p(ybuf.data_ptr()), 1)
        total = 0.0
        for _ in range(reps):
            l2_flush()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, op.handle, C.c_void_p(xbuf.data_ptr()),
                                             C.c_void_p(ybuf.data_ptr()), 1))
            e1.record(stream)
            e1.synchronize()
            total += e0.elapsed_time(e1) / 1e3
        return total / reps

    peak, peak_kind = load_peaks()
    # sanity reference for the timing method: a plain device copy of 1 GiB
    cbuf_a = torch.empty(256 * 1024 * 1024, dtype=torch.float32, device=dev)
    cbuf_b = torch.empty_like(cbuf_a)
    for _ in range(3):
        cbuf_b.copy_(cbuf_a)
    torch.cuda.synchronize()
    ce0, ce1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ce0.record()
    for _ in range(5):
        cbuf_b.copy_(cbuf_a)
    ce1.record()
    ce1.synchronize()
    copy_gbs = 5 * 2 * cbuf_a.numel() * 4 / (ce0.elapsed_time(ce1) / 1e3) / 1e9
    del cbuf_a, cbuf_b
    x32 = torch.randn(n, dtype=torch.float32, device=dev)
    y32 = torch.empty(n, dtype=torch.float32, device=dev)
    x64 = torch.randn(n, dtype=torch.float64, device=dev)
    y64 = torch.empty(n, dtype=torch.float64, device=dev)
    t32 = spmv_time(a32, x32, y32)
    t64 = spmv_time(a64, x64, y64)
    b32 = spmv_bytes(n, nnz, 4)
    b64 = spmv_bytes(n, nnz, 8)
    sweep = {
        "laplace3d_128_fp32": {"GB/s": b32 / t32 / 1e9, "frac": b32 / t32 / 1e9 / peak, "us": t32 * 1e6},
        "laplace3d_128_fp64": {"GB/s": b64 / t64 / 1e9, "frac": b64 / t64 / 1e9 / peak, "us": t64 * 1e6},
    }
    if args.sweep:
        pip, pix, pv = S.generate("powerlaw", 4194304, seed=1, param0=16.0, param1=4096.0)
        pn, pnnz = len(pip) - 1, len(pv)
        p64 = S.csr_from_arrays(ctx, pip, pix, pv, (pn, pn))
        p32 = p64.astype(np.float32)
        px32 = torch.randn(pn, dtype=torch.float32, device=dev)
        py32 = torch.empty(pn, dtype=torch.float32, device=dev)
        px64 = torch.randn(pn, dtype=torch.float64, device=dev)
        py64 = torch.empty(pn, dtype=torch.float64, device=dev)
        pt32 = spmv_time(p32, px32, py32, 10)
        pt64 = spmv_time(p64, px64, py64, 10)
        pb32, pb64 = spmv_bytes(pn, pnnz, 4), spmv_bytes(pn, pnnz, 8)
        sweep["powerlaw_4M_fp32"] = {"GB/s": pb32 / pt32 / 1e9, "frac": pb32 / pt32 / 1e9 / peak, "us": pt32 * 1e6}
        sweep["powerlaw_4M_fp64"] = {"GB/s": pb64 / pt64 / 1e9, "frac": pb64 / pt64 / 1e9 / peak, "us": pt64 * 1e6}
        p32.close()
        p64.close()

    traffic = None
    prof = os.path.join(REPO, "profiles", "spmv_laplace3d_128_fp32.txt")
    if os.path.exists(prof):
        for line in open(prof):
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = float(line.split(":")[1])

    # CPU baseline: the oracle on a bounded sample, scaled to the FP64 Jacobi-PCG count
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        iters = int(r_j64.iterations)
        sample_iters = min(iters, args.cpu_sample_iters)
        _, dt = cpu_reference_solve(ip, ix, v, n, b, sample_iters)
        cpu = {"value": dt * iters / sample_iters, "unit": "s", "cores": 1, "kind": "port",
               "sample": f"oracle cg+Jacobi FP64, first {sample_iters} of {iters} iterations, scaled"}

    value = statistics.mean(t_dev)
    if dist:
        tt = torch.tensor([value], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        value = float(tt.item())
    e2e = statistics.mean(t_e2e)
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 refinement", "data": "synthetic",
        "config": {"workload": workload_desc(n, nnz),
                   "method": "Jacobi-PCG, FP32 inner solve + FP64 iterative refinement",
                   "inner_rtol": args.inner_rtol, "outer_iterations": int(res.outer_iterations),
                   "inner_iterations": int(res.inner_iterations), "fp64_true_rel_residual": true_res,
                   "l2": "working set > L2 (129 MB) and a 512 MB L2 flush between steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "jacobi_pcg_fp64": {"value": statistics.mean(t_j64), "unit": "s", "iterations": int(r_j64.iterations),
                            "fp64_true_rel_residual": true_res_j64},
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8},
        "roofline": {"bound": "hbm", "kernel": "spmv_stream_kernel<float> (laplace3d 128^3)",
                     "achieved": b32 / t32 / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": b32 / t32 / 1e9 / peak, "peak_source": peak_kind,
                     "algorithmic_bytes": b32, "traffic": traffic},
        "spmv_sweep": sweep,
        "copy_gbs_same_run": copy_gbs,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    for op in (m64, m32, a32, a64):
        op.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()


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
    if args.profile in ("spmv32", "spmv64"):
        ip, ix, v = S.generate("laplace3d", GRID, GRID, GRID)
    else:
        ip, ix, v = S.generate("powerlaw", 4194304, seed=1, param0=16.0, param1=4096.0)
    n = len(ip) - 1
    dt = np.float64 if args.profile.endswith("64") else np.float32
    a = S.csr_from_arrays(ctx, ip, ix, v.astype(dt), (n, n))
    tdt = torch.float64 if dt == np.float64 else torch.float32
    x = torch.randn(n, dtype=tdt, device="cuda")
    y = torch.empty(n, dtype=tdt, device="cuda")
    for _ in range(args.steps):
        S.sparse._check(L.lib.sx_spmv_ex(ctx.handle, a.handle, C.c_void_p(x.data_ptr()),
                                         C.c_void_p(y.data_ptr()), 1))
    ctx.synchronize()
    print(json.dumps({"profile": args.profile, "n": n, "nnz": len(v), "launches": args.steps}))
    a.close()
    ctx.close()


# ------------------------------------------- learned SAI vs Jacobi (configs[4])
WEIGHTS = os.path.join(REPO, "scirs_gb300", "weights", "aniso_q1.npz")


def eval_learned(ctx, net, side, seeds, max_iter=400000, with_fp64_learned=True, log=None):
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
        out = os.path.join(REPO, "gpurun_out", "aniso_q1.npz")
        os.makedirs(os.path.dirname(out), exist_ok=True)
        LR.save_weights(out, net, {"steps": args.train_gnn, "seed": args.train_seed, "train_s": t_train})
        log(json.dumps({"trained_steps": args.train_gnn, "train_s": t_train, "log": train_log[-5:]}))
    elif os.path.exists(WEIGHTS):
        net = LR.load_weights(ctx, WEIGHTS)
    else:
        net = None
    seeds = [int(s) for s in args.eval_seeds.split(",")]
    rows = eval_learned(ctx, net, args.eval_side, seeds, log=log)
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
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-iters", type=int, default=60)
    ap.add_argument("--profile", default=None,
                    choices=["spmv32", "spmv64", "powerlaw32", "powerlaw64", "solve"],
                    help="run a few launches of one SpMV for an ncu capture and exit")
    ap.add_argument("--workload", default="laplace3d", choices=["laplace3d", "learned"])
    ap.add_argument("--train-gnn", type=int, default=0, help="train the network for N steps first")
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
