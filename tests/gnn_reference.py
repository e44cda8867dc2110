"""PyTorch CPU restatement of the learned factorised-SAI network (test oracle).

Mirrors scirs_gb300/csrc/sx_gnn.cu operation by operation: the same
parameter layout, BF16 rounding of weights and of the GEMM inputs (node
features and hidden states), FP32 accumulation, and the random-probe loss
||(G^T A G - I) Z||_F^2 / (k n) on the Jacobi-scaled matrix.  Autograd of this
module is the gradient oracle for the device's hand-written backward pass.
"""
from __future__ import annotations

import numpy as np
import torch

F0, K0, H, L, C = 4, 16, 64, 3, 32


def param_layout():
    """(name, shape) in the flat FP32 parameter vector order."""
    out = []
    kin = F0
    for layer in range(L):
        out += [(f"Ws{layer}", (H, kin)), (f"Wn{layer}", (H, kin)), (f"b{layer}", (H,))]
        kin = H
    out += [("P1", (C, H)), ("P2", (C, H)), ("p3", (C,)), ("p0", (C,)), ("q", (C,)),
            ("wd", (H,)), ("bd", (1,))]
    return out


def num_params():
    return int(sum(np.prod(s) for _, s in param_layout()))


def unflatten(flat: torch.Tensor):
    p, o = {}, 0
    for name, shape in param_layout():
        k = int(np.prod(shape))
        p[name] = flat[o:o + k].view(*shape)
        o += k
    return p


def bf16(t: torch.Tensor) -> torch.Tensor:
    """Round to BF16 (nearest even) and back; identity for the gradient."""
    r = t.detach().to(torch.bfloat16).to(torch.float32)
    return t + (r - t).detach()


def prepare(indptr, indices, vals):
    """Jacobi scaling, off-diagonal scaled matrix, node features, G pattern."""
    n = len(indptr) - 1
    indptr = np.asarray(indptr, dtype=np.int64)
    indices = np.asarray(indices, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    rows = np.repeat(np.arange(n), np.diff(indptr))
    diag = np.zeros(n)
    diag_mask = rows == indices
    diag[rows[diag_mask]] = vals[diag_mask]
    dis = (1.0 / np.sqrt(diag)).astype(np.float32)
    off = ~diag_mask
    orow, ocol = rows[off], indices[off]
    # scaled off-diagonal value in FP32: (a_ij * dis_i) * dis_j
    ahat = (vals[off].astype(np.float32) * dis[orow]) * dis[ocol[...]]
    feats = np.zeros((n, K0), dtype=np.float32)
    feats[:, 0] = 1.0
    np.add.at(feats[:, 1], orow, np.abs(ahat))
    np.add.at(feats[:, 2], orow, ahat)
    np.maximum.at(feats[:, 3], orow, np.abs(ahat))
    low = off & (indices < rows)
    # G pattern: strictly lower entries of each row in column order, then the diagonal
    g_rows, g_cols, g_ahat = [], [], []
    ahat_full = {}
    for r_, c_, v_ in zip(orow, ocol, ahat):
        ahat_full[(r_, c_)] = v_
    for i in range(n):
        cols = sorted(int(c) for c in indices[indptr[i]:indptr[i + 1]] if c < i)
        for c in cols:
            g_rows.append(i)
            g_cols.append(c)
            g_ahat.append(ahat_full[(i, c)])
        g_rows.append(i)
        g_cols.append(i)
        g_ahat.append(0.0)
    del low
    return dict(n=n, dis=dis, orow=orow, ocol=ocol, ahat=ahat.astype(np.float32), feats=feats,
                g_rows=np.array(g_rows), g_cols=np.array(g_cols),
                g_ahat=np.array(g_ahat, dtype=np.float32))


def forward(flat: torch.Tensor, prep):
    """Edge values g_hat on the G pattern (torch, differentiable in flat)."""
    p = unflatten(flat)
    n = prep["n"]
    orow = torch.as_tensor(prep["orow"])
    ocol = torch.as_tensor(prep["ocol"])
    ahat = torch.as_tensor(prep["ahat"])
    h = torch.as_tensor(prep["feats"])[:, :F0]
    h = bf16(h)
    for layer in range(L):
        ws, wn, b = bf16(p[f"Ws{layer}"]), bf16(p[f"Wn{layer}"]), p[f"b{layer}"]
        s_self = h @ ws.T
        s_nb = h @ wn.T
        agg = torch.zeros(n, H).index_add_(0, orow, ahat[:, None] * s_nb[ocol])
        pre = s_self + agg + b
        h = bf16(torch.relu(pre))
    y1 = h @ bf16(p["P1"]).T
    y2 = h @ bf16(p["P2"]).T
    yd = h @ bf16(p["wd"])
    gr = torch.as_tensor(prep["g_rows"])
    gc = torch.as_tensor(prep["g_cols"])
    ga = torch.as_tensor(prep["g_ahat"])
    is_diag = gr == gc
    z = torch.relu(y1[gr] + y2[gc] + ga[:, None] * p["p3"] + p["p0"])
    g_off = z @ p["q"]
    g_diag = torch.nn.functional.softplus(yd[gr] + p["bd"])
    return torch.where(is_diag, g_diag, g_off)


def probe_loss(g: torch.Tensor, prep, z: np.ndarray):
    """||(G^T A_hat G - I) Z||^2 / (k n) with A_hat = I + offdiag."""
    n = prep["n"]
    k = z.shape[1]
    Z = torch.as_tensor(z, dtype=torch.float32)
    gr = torch.as_tensor(prep["g_rows"])
    gc = torch.as_tensor(prep["g_cols"])
    orow = torch.as_tensor(prep["orow"])
    ocol = torch.as_tensor(prep["ocol"])
    ahat = torch.as_tensor(prep["ahat"])
    y = torch.zeros(n, k).index_add_(0, gr, g[:, None] * Z[gc])
    w = y + torch.zeros(n, k).index_add_(0, orow, ahat[:, None] * y[ocol])
    v = torch.zeros(n, k).index_add_(0, gc, g[:, None] * w[gr])
    r = v - Z
    return (r * r).sum() / (k * n)
