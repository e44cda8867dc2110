"""Batched PCG on the device vs the oracle, one system at a time."""
import numpy as np
import pytest

from oracle import oracle_ffi as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import scirs_gb300

    return scirs_gb300


def _slice(sp, ip, ix, v, s):
    r0, r1 = sp[s], sp[s + 1]
    k0, k1 = ip[r0], ip[r1]
    return ip[r0:r1 + 1] - k0, ix[k0:k1] - r0, v[k0:k1]


def test_batched_matches_per_system_oracle(S, ctx):
    sp, ip, ix, v = S.generate_batch(23, 4, 36, seed=7, sigma=1.0)
    n = len(ip) - 1
    b = S.rhs_normal(11, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    r = S.batched_pcg(a, sp, b, rtol=1e-8, inner_rtol=1e-4)
    assert r.converged.all()
    for s in range(len(sp) - 1):
        sip, six, sv = _slice(sp, ip, ix, v, s)
        bs = b[sp[s]:sp[s + 1]]
        xs = r.x[sp[s]:sp[s + 1]]
        res = O.true_rel_residual(sip, six, sv, bs, xs)
        assert res <= 1e-8 * 1.0001, (s, res)
        assert abs(res - r.rel_residual[s]) <= 1e-3 * res + 1e-16
        ro = O.cg_mixed_ir(sip, six, sv, bs, tol=1e-8, inner_rtol=1e-4)
        assert ro["converged"]
        assert np.linalg.norm(xs - ro["x"]) / np.linalg.norm(ro["x"]) < 1e-6


def test_batched_zero_and_trivial_systems(S, ctx):
    # a zero right-hand side converges at once; 1x1 systems solve in one step
    sp, ip, ix, v = S.generate_batch(5, 1, 6, seed=3)
    n = len(ip) - 1
    b = S.rhs_normal(2, n)
    b[sp[1]:sp[2]] = 0.0
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    r = S.batched_pcg(a, sp, b)
    assert r.converged.all()
    assert np.all(r.x[sp[1]:sp[2]] == 0.0)
    for s in range(5):
        sip, six, sv = _slice(sp, ip, ix, v, s)
        bs = b[sp[s]:sp[s + 1]]
        if np.any(bs):
            assert O.true_rel_residual(sip, six, sv, bs, r.x[sp[s]:sp[s + 1]]) <= 1e-8


def test_batched_rejects_bad_offsets(S, ctx):
    sp, ip, ix, v = S.generate_batch(3, 4, 6, seed=1)
    n = len(ip) - 1
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    bad = sp.copy()
    bad[-1] -= 1
    with pytest.raises(S.SparseError) as e:
        S.batched_pcg(a, bad, np.ones(n))
    assert e.value.variant == "DimensionMismatch"


def test_batched_every_launch_shape(S, ctx):
    # each candidate shape of the autotuner (forced) solves the batch to the
    # tolerance; one shape run twice gives the same bits; the tuned shape is
    # one of them and is cached for the next call on the same batch
    import os

    sp, ip, ix, v = S.generate_batch(40, 8, 64, seed=5, sigma=1.0)
    n = len(ip) - 1
    b = S.rhs_normal(2, n)
    a = S.csr_from_arrays(ctx, ip, ix, v, (n, n))
    shapes = set()
    try:
        for k in range(6):
            os.environ["SX_TUNE_FORCE"] = str(k)
            r = S.batched_pcg(a, sp, b, rtol=1e-8)
            assert r.converged.all(), k
            shapes.add((r.threads_per_block, r.blocks_per_sm))
            for s in range(len(sp) - 1):
                sip, six, sv = _slice(sp, ip, ix, v, s)
                assert O.true_rel_residual(sip, six, sv, b[sp[s]:sp[s + 1]], r.x[sp[s]:sp[s + 1]]) <= 1.0001e-8
            if k == 2:
                r2 = S.batched_pcg(a, sp, b, rtol=1e-8)
                assert np.array_equal(r.x.view(np.uint8), r2.x.view(np.uint8))
    finally:
        os.environ.pop("SX_TUNE_FORCE", None)
    assert len(shapes) == 6
    r1 = S.batched_pcg(a, sp, b, rtol=1e-8)
    r2 = S.batched_pcg(a, sp, b, rtol=1e-8)
    assert (r1.threads_per_block, r1.blocks_per_sm) == (r2.threads_per_block, r2.blocks_per_sm)
    assert (r1.threads_per_block, r1.blocks_per_sm) in shapes
    assert np.array_equal(r1.x.view(np.uint8), r2.x.view(np.uint8))
    a.close()
