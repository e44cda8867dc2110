"""CPU checks of the C ABI library: it loads, exports every declared symbol,
and its host-side generators produce the documented matrices."""
import ctypes as C
import os
import re

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(REPO, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(REPO, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(sx_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    from scirs_gb300 import _lib as L

    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(L.lib, n)]
    assert not missing, missing
    assert not L.MISSING


def test_status_and_message_strings():
    from scirs_gb300 import _lib as L

    assert L.lib.sx_status_string(9) == b"ValueError"
    assert L.lib.sx_status_string(14) == b"IndexCastOverflow"
    assert L.lib.sx_message_string(2) == b"Matrix not positive definite (p^T*A*p <= 0)"
    assert L.lib.sx_message_string(4).decode() == "BiCGSTAB breakdown: rho ≈ 0"


def test_option_defaults_match_reference():
    # CGOptions / BiCGSTABOptions / GMRESOptions defaults (iterative.rs:25-35, 358-368, 623-634)
    from scirs_gb300 import _lib as L

    o = L.CGOptions()
    L.lib.sx_cg_options_default(C.byref(o))
    assert (o.max_iter, o.rtol, o.atol) == (1000, 1e-8, 1e-12) and not o.x0
    g = L.GMRESOptions()
    L.lib.sx_gmres_options_default(C.byref(g))
    assert (g.max_iter, g.restart, g.rtol, g.atol) == (1000, 30, 1e-8, 1e-12)


def test_context_without_gpu_fails_loudly():
    import torch

    import scirs_gb300 as S

    if torch.cuda.is_available():
        return
    try:
        S.Context(0)
    except S.SparseError as e:
        assert e.variant == "CudaError"
    else:
        raise AssertionError("a context was created without a GPU")


def test_generator_sizes():
    import scirs_gb300 as S

    ip, ix, v = S.generate("poisson2d", 256, 256)
    assert len(ip) - 1 == 65536 and len(v) == 326656
    ip, ix, v = S.generate("laplace3d", 16, 16, 16)
    assert len(v) == 7 * 16 ** 3 - 6 * 16 ** 2
    ip, ix, v = S.generate("aniso_q1", 64, 64, param0=10.0, param1=0.3)
    assert len(v) == 9 * 64 * 64 - (6 * 64 + 6 * 64 - 4)


def _dense(ip, ix, v):
    n = len(ip) - 1
    d = np.zeros((n, n))
    for r in range(n):
        d[r, ix[ip[r]:ip[r + 1]]] = v[ip[r]:ip[r + 1]]
    return d


def test_generators_are_spd_and_sorted():
    import scirs_gb300 as S

    for kind, dims, p0, p1 in [("poisson2d", (6, 5, 1), 0, 0), ("laplace3d", (4, 3, 5), 0, 0),
                               ("varcoef3d", (4, 4, 3), 1.5, 0), ("varcoef2d", (7, 5, 1), 1.0, 0),
                               ("aniso_q1", (6, 7, 1), 1000.0, 1.1)]:
        ip, ix, v = S.generate(kind, *dims, seed=4, param0=p0, param1=p1)
        d = _dense(ip, ix, v)
        assert np.allclose(d, d.T), kind
        assert np.linalg.eigvalsh(d).min() > 0, kind
        for r in range(len(ip) - 1):
            assert np.all(np.diff(ix[ip[r]:ip[r + 1]]) > 0)


def test_generators_are_deterministic():
    import scirs_gb300 as S

    a = S.generate("varcoef3d", 20, 20, 20, seed=9, param0=1.5)
    b = S.generate("varcoef3d", 20, 20, 20, seed=9, param0=1.5)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert np.array_equal(S.rhs_normal(3, 100000), S.rhs_normal(3, 100000))


def test_powerlaw_statistics():
    import scirs_gb300 as S

    ip, ix, v = S.generate("powerlaw", 200000, seed=2, param0=16.0, param1=4096.0)
    lens = np.diff(ip)
    assert lens.min() >= 1 and lens.max() <= 4096
    assert abs(lens.mean() - 16.0) < 0.6
    assert np.all((v >= -1) & (v < 1))
    for r in range(0, 200000, 997):
        row = ix[ip[r]:ip[r + 1]]
        assert np.all(np.diff(row) > 0)
