"""CPU checks of the PyTorch restatement used as the network's gradient oracle."""
import numpy as np
import scipy.sparse as sp
import torch

from tests import gnn_reference as R


def _aniso(nx, ny, eps, theta):
    import scirs_gb300 as S

    return S.generate("aniso_q1", nx, ny, param0=eps, param1=theta)


def test_identity_g_gives_scaled_matrix_loss():
    ip, ix, v = _aniso(9, 8, 20.0, 0.5)
    prep = R.prepare(ip, ix, v)
    n = prep["n"]
    g = np.where(prep["g_rows"] == prep["g_cols"], 1.0, 0.0).astype(np.float32)
    rng = np.random.default_rng(0)
    z = rng.standard_normal((n, 4)).astype(np.float32)
    loss = R.probe_loss(torch.tensor(g), prep, z).item()
    a = sp.csr_matrix((v, ix, ip), shape=(n, n)).toarray()
    d = 1 / np.sqrt(np.diag(a))
    ahat = d[:, None] * a * d[None, :]
    ref = np.sum(((ahat - np.eye(n)) @ z) ** 2) / (4 * n)
    assert abs(loss - ref) <= 1e-4 * ref


def test_pattern_is_lower_with_diagonal_last():
    ip, ix, v = _aniso(7, 6, 3.0, 1.0)
    prep = R.prepare(ip, ix, v)
    rows, cols = prep["g_rows"], prep["g_cols"]
    assert np.all(cols <= rows)
    for i in range(prep["n"]):
        c = cols[rows == i]
        assert c[-1] == i and np.all(np.diff(c) > 0)


def test_autograd_matches_finite_differences():
    ip, ix, v = _aniso(6, 6, 10.0, 0.8)
    prep = R.prepare(ip, ix, v)
    rng = np.random.default_rng(1)
    z = rng.standard_normal((prep["n"], 4)).astype(np.float32)
    g0 = torch.tensor(rng.uniform(-0.2, 0.2, len(prep["g_rows"])), dtype=torch.float64)
    g0[prep["g_rows"] == prep["g_cols"]] += 1.0
    g = g0.clone().requires_grad_(True)
    prep64 = dict(prep)
    loss = R.probe_loss(g.float(), prep64, z)
    loss.backward()
    e = 3
    h = 1e-3
    gp, gm = g0.clone(), g0.clone()
    gp[e] += h
    gm[e] -= h
    fd = (R.probe_loss(gp.float(), prep64, z) - R.probe_loss(gm.float(), prep64, z)).item() / (2 * h)
    assert abs(fd - g.grad[e].item()) <= 2e-2 * abs(fd) + 1e-6
