"""Learned factorised SAI: device forward/backward vs the PyTorch CPU oracle,
training, and the gain of the trained network over Jacobi."""
import numpy as np
import pytest
import torch

from tests import gnn_reference as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _aniso(S, ctx, nx, ny, eps, theta, dtype=np.float64):
    ip, ix, v = S.generate("aniso_q1", nx, ny, param0=eps, param1=theta)
    n = len(ip) - 1
    return ip, ix, v, S.csr_from_arrays(ctx, ip, ix, v.astype(dtype), (n, n))


def test_forward_matches_pytorch(S, ctx):
    ip, ix, v, a = _aniso(S, ctx, 20, 17, 30.0, 0.7)
    net = S.LearnedSAI(ctx, seed=3)
    p = net.params
    # a perturbed, non-trivial network (the initial one is near the identity)
    rng = np.random.default_rng(1)
    p = (p + 0.2 * rng.standard_normal(p.size).astype(np.float32)).astype(np.float32)
    net.params = p
    g_dev = net.edge_values(a)
    prep = R.prepare(ip, ix, v)
    g_ref = R.forward(torch.tensor(p), prep).detach().numpy()
    assert g_dev.shape == g_ref.shape
    scale = np.abs(g_ref).max()
    assert np.max(np.abs(g_dev - g_ref)) <= 3e-2 * scale
    assert np.corrcoef(g_dev, g_ref)[0, 1] > 0.999


def test_gradient_matches_autograd(S, ctx):
    ip, ix, v, a = _aniso(S, ctx, 16, 15, 10.0, 1.1)
    net = S.LearnedSAI(ctx, seed=5)
    rng = np.random.default_rng(2)
    p = (net.params + 0.1 * rng.standard_normal(net.num_params)).astype(np.float32)
    net.params = p
    prep = R.prepare(ip, ix, v)
    z = rng.standard_normal((prep["n"], 4)).astype(np.float32)
    loss_dev, grad_dev = net.loss_grad(a, probes=z)
    pt = torch.tensor(p, requires_grad=True)
    loss_ref = R.probe_loss(R.forward(pt, prep), prep, z)
    loss_ref.backward()
    grad_ref = pt.grad.numpy()
    assert abs(loss_dev - loss_ref.item()) <= 2e-2 * abs(loss_ref.item())
    # per parameter group: direction and magnitude
    o = 0
    for name, shape in R.param_layout():
        k = int(np.prod(shape))
        gd, gr = grad_dev[o:o + k], grad_ref[o:o + k]
        o += k
        nr = np.linalg.norm(gr)
        if nr < 1e-6 * np.linalg.norm(grad_ref):
            continue
        cos = float(gd @ gr / (np.linalg.norm(gd) * nr + 1e-30))
        assert cos > 0.995, (name, cos)
        assert abs(np.linalg.norm(gd) / nr - 1) < 0.05, (name, np.linalg.norm(gd), nr)


def test_training_reduces_loss_and_iterations(S, ctx):
    rng = np.random.default_rng(7)
    train = []
    for _ in range(6):
        eps = float(10 ** rng.uniform(0, 3))
        theta = float(rng.uniform(0, np.pi))
        train.append(_aniso(S, ctx, 48, 48, eps, theta)[3])
    net = S.LearnedSAI(ctx, seed=11)
    first = np.mean([net.loss_grad(a, seed=99)[0] for a in train])
    for step in range(600):
        net.train_step(train[step % len(train)], seed=step, lr=2e-3)
    last = np.mean([net.loss_grad(a, seed=99)[0] for a in train])
    assert last < 0.8 * first, (first, last)
    # held-out matrix: PCG iterations with the learned G G^T vs Jacobi
    ip, ix, v, a = _aniso(S, ctx, 64, 64, 300.0, 0.4)
    n = a.shape[0]
    b = S.rhs_normal(5, n)
    r_j = S.cg(a, b, max_iter=20000, rtol=1e-8, atol=0.0, preconditioner=S.jacobi(ctx, a))
    m = net.preconditioner(a)
    r_l = S.cg(a, b, max_iter=20000, rtol=1e-8, atol=0.0, preconditioner=m)
    assert r_j.converged and r_l.converged
    assert r_l.iterations < r_j.iterations, (r_l.iterations, r_j.iterations)


def test_learned_preconditioner_is_spd_apply(S, ctx):
    # M^-1 = G G^T: symmetric and positive on random vectors
    ip, ix, v, a = _aniso(S, ctx, 12, 12, 5.0, 0.3)
    net = S.LearnedSAI(ctx, seed=1)
    m = net.preconditioner(a)
    n = a.shape[0]
    rng = np.random.default_rng(0)
    for _ in range(3):
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        mx, my = m.matvec(x), m.matvec(y)
        assert abs(x @ my - y @ mx) <= 1e-10 * np.linalg.norm(x) * np.linalg.norm(my)
        assert x @ mx > 0


@pytest.mark.parametrize("dtype,symmetric", [(np.float64, True), (np.float32, True), (np.float64, False)])
def test_learned_factor_matches_dense_g(S, ctx, dtype, symmetric):
    # M^-1 x = G (G^T x) with G = D^-1/2 G^ on the network's pattern (each
    # row's strict-lower columns, then the diagonal): G^T comes from the
    # graph's transposed pattern (read off A's upper triangle when A's
    # pattern is symmetric, a sort otherwise), so a wrong entry permutation
    # would break the product (and its symmetry), not just round it
    ip, ix, v, a = _aniso(S, ctx, 20, 17, 30.0, 0.6, dtype)
    if not symmetric:
        # drop some upper entries: a pattern without (j, i) for some (i, j)
        n = a.shape[0]
        a.close()
        rows = np.repeat(np.arange(n), np.diff(ip))
        keep = ~((ix > rows) & ((rows + ix) % 5 == 0))
        ix, v = ix[keep], v[keep]
        ip = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=n))]).astype(ip.dtype)
        a = S.csr_from_arrays(ctx, ip, ix, v.astype(dtype), (n, n))
    net = S.LearnedSAI(ctx, seed=2)
    m = net.preconditioner(a)
    g = net.edge_values(a).astype(np.float64)
    n = a.shape[0]
    G = np.zeros((n, n))
    pos = 0
    for i in range(n):
        row = ix[ip[i]:ip[i + 1]]
        d = np.float64(v.astype(dtype)[ip[i]:ip[i + 1]][row == i][0])
        dis = np.float64(np.float32(1.0 / np.sqrt(d)))
        for c in list(row[row < i]) + [i]:
            G[i, c] = np.float64(dtype(g[pos] * dis))
            pos += 1
    assert pos == len(g)
    rng = np.random.default_rng(5)
    for _ in range(2):
        x = rng.standard_normal(n)
        ref = G @ (G.T @ x.astype(dtype).astype(np.float64))
        out = m.matvec(x.astype(dtype)).astype(np.float64)
        tol = 1e-12 if dtype == np.float64 else 2e-5
        assert np.abs(out - ref).max() <= tol * np.abs(ref).max()
    m.close()
    net.close()
    a.close()


def test_fp16_factor_matches_fp32_factor_iterations(S, ctx):
    # the learned preconditioner's solver applies read G in FP16; the same G
    # in FP32 (a user FSAI operator) needs about as many PCG iterations
    ip, ix, v, a64 = _aniso(S, ctx, 96, 80, 200.0, 0.8)
    a32 = a64.astype(np.float32)
    n = a64.shape[0]
    net = S.LearnedSAI(ctx, seed=4)
    rng = np.random.default_rng(3)
    net.params = (net.params + 0.05 * rng.standard_normal(net.num_params)).astype(np.float32)
    g = net.edge_values(a32)
    # G pattern: each row's strict-lower columns, then the diagonal
    lens, cols = [], []
    for i in range(n):
        row = ix[ip[i]:ip[i + 1]]
        low = row[row < i]
        cols.append(np.concatenate([low, [i]]))
        lens.append(len(low) + 1)
    gp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    gi = np.concatenate(cols).astype(np.int32)
    diag = np.array([v[ip[i]:ip[i + 1]][ix[ip[i]:ip[i + 1]] == i][0] for i in range(n)])
    dis = 1.0 / np.sqrt(diag.astype(np.float32).astype(np.float64))
    gv = (g.astype(np.float64) * np.repeat(dis, lens)).astype(np.float32)
    G = S.csr_from_arrays(ctx, gp, gi, gv, (n, n))
    m32 = S.fsai(ctx, G)
    m16 = net.preconditioner(a32)
    b = S.rhs_normal(2, n).astype(np.float32)
    r32 = S.cg(a32, b, max_iter=20000, rtol=1e-5, atol=0.0, preconditioner=m32)
    r16 = S.cg(a32, b, max_iter=20000, rtol=1e-5, atol=0.0, preconditioner=m16)
    assert r32.converged and r16.converged
    assert abs(r16.iterations - r32.iterations) <= 0.05 * r32.iterations + 3, (r16.iterations, r32.iterations)
    for op in (m16, m32, G, a32, a64):
        op.close()
    net.close()
