"""Training and evaluation helpers for the learned factorised SAI.

Training problems are 2D anisotropic diffusion on Q1 elements:
K = R(theta) diag(1, 1/eps) R(theta)^T with eps log-uniform in [1, 1e3] and
theta uniform in [0, pi), on square grids whose side is drawn from
`sides`.  Every step is an Adam step of the device's own forward/backward
kernels on one problem (4 Gaussian probes).  Weights are stored as a small
versioned .npz.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import sparse as S

WEIGHTS_VERSION = 1


@dataclass
class Problem:
    side: int
    eps: float
    theta: float
    seed: int


def sample_problem(seed: int, sides=(64, 512)) -> Problem:
    rng = np.random.default_rng(seed)
    side = int(rng.integers(sides[0], sides[1] + 1))
    eps = float(10.0 ** rng.uniform(0.0, 3.0))
    theta = float(rng.uniform(0.0, np.pi))
    return Problem(side, eps, theta, seed)


def build(ctx: S.Context, prob: Problem, side: int | None = None, dtype=np.float64) -> S.Operator:
    nside = side or prob.side
    ip, ix, v = S.generate("aniso_q1", nside, nside, param0=prob.eps, param1=prob.theta)
    n = len(ip) - 1
    return S.csr_from_arrays(ctx, ip, ix, v.astype(dtype), (n, n))


def train(ctx: S.Context, steps: int, seed: int = 0, n_problems: int = 48, sides=(64, 512),
          lr: float = 2e-3, net: S.LearnedSAI | None = None, log_every: int = 0):
    """Train on `n_problems` seeded problems (seeds seed*1000 + k); returns (net, log)."""
    net = net or S.LearnedSAI(ctx, seed=seed)
    probs = [sample_problem(seed * 1000 + k, sides) for k in range(n_problems)]
    ops = [build(ctx, p, dtype=np.float32) for p in probs]
    log = []
    t0 = time.perf_counter()
    for step in range(steps):
        k = step % n_problems
        # cosine decay of the step size
        cur = lr * 0.5 * (1.0 + np.cos(np.pi * step / max(steps, 1)))
        loss = net.train_step(ops[k], seed=seed * 7919 + step, lr=max(cur, lr * 0.02))
        if log_every and step % log_every == 0:
            log.append((step, float(loss), time.perf_counter() - t0))
    for op in ops:
        op.close()
    return net, log


def save_weights(path: str, net: S.LearnedSAI, meta: dict) -> None:
    np.savez(path, version=WEIGHTS_VERSION, params=net.params, **{k: np.asarray(v) for k, v in meta.items()})


def load_weights(ctx: S.Context, path: str) -> S.LearnedSAI:
    d = np.load(path)
    if int(d["version"]) != WEIGHTS_VERSION:
        raise ValueError(f"weights version {int(d['version'])} != {WEIGHTS_VERSION}")
    return S.LearnedSAI(ctx, params=d["params"])


@dataclass
class SolveResult:
    """Outcome of `solve`: method is "learned-mixed" when the learned mixed
    loop reached tol, "learned-mixed+jacobi-pcg" when the fallback ran."""
    x: np.ndarray
    converged: bool
    method: str
    outer_iterations: int
    inner_iterations: int
    fallback_iterations: int
    rel_residual: float


def solve(net: S.LearnedSAI, a64: S.Operator, b, tol: float = 1e-8, max_inner: int = 200000,
          max_outer: int = 30, fallback_max_iter: int = 200000) -> SolveResult:
    """A x = b to an FP64 relative residual of tol: the learned factor G of
    the FP32 copy of A, FP32 PCG with M = G G^T inside the FP64
    residual-replacement loop, and, when that loop stops short of tol
    (stagnation, an FP32 p.Ap <= 0 or the outer limit), plain FP64
    Jacobi-PCG from its last iterate (converged by its own FP64 test,
    ||r|| <= tol ||b||; rel_residual is then the FP64 true residual)."""
    a32 = a64.astype(np.float32)
    g32 = None
    try:
        g32 = net.preconditioner(a32)
        r = S.cg_mixed(a64, b, tol=tol, max_inner=max_inner, max_outer=max_outer, preconditioner=g32, a32=a32)
    finally:
        if g32 is not None:
            g32.close()
        a32.close()
    if r.converged:
        return SolveResult(r.x, True, "learned-mixed", r.outer_iterations, r.inner_iterations, 0, r.rel_residual)
    m = S.jacobi(a64.ctx, a64)
    try:
        f = S.cg(a64, b, x0=r.x, max_iter=fallback_max_iter, rtol=tol, atol=0.0, preconditioner=m)
    finally:
        m.close()
    rel = float(S.true_rel_residual(a64, b, f.x))
    return SolveResult(f.x, bool(f.converged), "learned-mixed+jacobi-pcg", r.outer_iterations,
                       r.inner_iterations, f.iterations, rel)
