"""GPU tests of the batched solver: independent chunks of uneven size with
several right-hand sides each, against per-(chunk, RHS) FP64 solves.

Every (chunk, RHS) is its own exact-kernel system.  Bars:
  * each solution within 1e-6 relative of the CPU oracle's FP64 PCG on that
    chunk and right-hand side (converged to 1e-10);
  * the FP64 true residual |b - A x| / |b|, recomputed by the oracle's FP64
    operator, at most tol (1e-8) and equal to the reported one within 1e-3
    relative;
  * the FP32 batched product within 2e-5 relative (max norm) of the
    oracle's FP64 product.
"""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (BatchSolver, MixedParams, SignalCovarParams, WFVectorW,
                             pixel_to_npixel, pixel_to_wpixel, synth)

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA
EXACT = SignalCovarParams(VS, LP, LQ, eval="exact")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def small_batch(n_chunks, n_rhs, seed, sk=(3, 10), per=(16, 40)):
    return synth.chunks(n_chunks, seed, sk_range=sk, per_range=per, n_rhs=n_rhs)


def to_form(form, pixes, rhs):
    """Records and right-hand sides in the form's convention (W: wd = d / n)."""
    conv = pixel_to_wpixel if form == "w" else pixel_to_npixel
    recs = [conv(p) for p in pixes]
    if form == "w":
        n = np.concatenate([p[:, 3] for p in pixes])
        rhs = rhs / n[:, None]
    return recs, np.ascontiguousarray(rhs)


def oracle_solutions(form, recs, rhs, tol=1e-10):
    out = np.empty_like(rhs)
    off = 0
    for rec in recs:
        n = rec.shape[0]
        for r in range(rhs.shape[1]):
            rr = rec.copy()
            rr[:, 4] = rhs[off:off + n, r]
            x, ok, _, _ = oracle.solve_pcg(form, rr, VS, LP, LQ, 5000, 50, tol, exact=True)
            assert ok
            out[off:off + n, r] = x
        off += n
    return out


def oracle_rel_resid(form, recs, rhs, x):
    """|b - A y| / |b| per (chunk, RHS) with the FP64 oracle operator
    (y = x / w in the W form)."""
    res = np.zeros((len(recs), rhs.shape[1]))
    off = 0
    for c, rec in enumerate(recs):
        n = rec.shape[0]
        for r in range(rhs.shape[1]):
            rr = rec.copy()
            rr[:, 4] = rhs[off:off + n, r]
            y = x[off:off + n, r] / rec[:, 3] if form == "w" else x[off:off + n, r]
            resid = oracle.A_residual(form, rr, y, VS, LP, LQ, exact=True)
            res[c, r] = np.linalg.norm(resid) / np.linalg.norm(rr[:, 4])
        off += n
    return res


@pytest.mark.parametrize("form", ["w", "sn"])
def test_batch_matches_per_chunk_fp64(ctx, form):
    pixes, rhs = small_batch(5, 8, seed=3)
    recs, b = to_form(form, pixes, rhs)
    bs = BatchSolver(ctx, form, recs, EXACT, n_rhs=8)
    x, res = bs.solve_mixed(b, MixedParams(tol=1e-8))
    assert res.status == 0 and res.converged.all()
    assert (res.n_updates >= 1).all() and (res.iters > 0).all()
    assert res.rel_resid.max() <= 1e-8
    true = oracle_rel_resid(form, recs, b, x)
    assert true.max() <= 1e-8 * (1 + 1e-6)
    assert np.allclose(true, res.rel_resid, rtol=1e-3, atol=0)
    xo = oracle_solutions(form, recs, b)
    off = 0
    for c, rec in enumerate(recs):
        n = rec.shape[0]
        for r in range(8):
            assert rel(x[off:off + n, r], xo[off:off + n, r]) < 1e-6, (c, r)
        off += n
    bs.close()


def test_batch_rhs_blocks_and_odd_rhs_counts(ctx):
    pixes, rhs = small_batch(4, 6, seed=5)
    recs, b = to_form("w", pixes, rhs)
    xo = oracle_solutions("w", recs, b)
    bs = BatchSolver(ctx, "w", recs, EXACT, n_rhs=6)
    sols = []
    for rb in (1, 2):
        bs.set_variant("cuda_core", rb)
        assert bs.info()["rhs_block"] == rb
        x, res = bs.solve_mixed(b, MixedParams(tol=1e-8))
        assert res.converged.all()
        assert rel(x, xo) < 1e-6
        sols.append(x)
    assert rel(sols[0], sols[1]) < 1e-6
    # a single right-hand side and an odd count
    for R in (1, 3):
        bs1 = BatchSolver(ctx, "w", recs, EXACT, n_rhs=R)
        x1, res1 = bs1.solve_mixed(np.ascontiguousarray(b[:, :R]), MixedParams(tol=1e-8))
        assert res1.converged.all()
        assert rel(x1, xo[:, :R]) < 1e-6
        bs1.close()
    bs.close()


def test_batch_matches_single_operator_mixed_solve(ctx):
    # one chunk, one RHS: the same system as WFVectorW.solve_mixed
    w = synth.small(12, 40, 10.0, seed=9)
    rec = pixel_to_wpixel(w.pixels)
    op = WFVectorW(ctx, rec, EXACT)
    xs, rs = op.solve_mixed(MixedParams(tol=1e-8))
    bs = BatchSolver(ctx, "w", [rec], EXACT, n_rhs=1)
    xb, rb = bs.solve_mixed(rec[:, 4:5].copy(), MixedParams(tol=1e-8))
    assert rs.success and rb.converged.all()
    assert rel(xb[:, 0], xs) < 1e-6
    # the iteration counts follow the same recurrence up to FP32 rounding
    assert abs(int(rb.iters[0, 0]) - rs.num_iters) <= max(3, rs.num_iters // 10)
    bs.close()


def test_batch_product_f32_vs_fp64(ctx):
    import torch

    pixes, rhs = small_batch(6, 4, seed=11, sk=(2, 14), per=(8, 64))
    recs, b = to_form("sn", pixes, rhs)
    bs = BatchSolver(ctx, "sn", recs, EXACT, n_rhs=4)
    p = np.random.default_rng(1).standard_normal(b.shape)
    pt = torch.tensor(p, dtype=torch.float64, device="cuda")
    qt = torch.zeros_like(pt)
    for rb in (1, 2, 4):
        bs.set_variant("cuda_core", rb)
        bs.product_f32_dev(pt, qt)
        torch.cuda.synchronize()
        q = qt.cpu().numpy()
        off = 0
        for rec in recs:
            n = rec.shape[0]
            for r in range(4):
                qo = oracle.A_product("sn", rec, p[off:off + n, r], VS, LP, LQ, exact=True)
                assert rel(q[off:off + n, r], qo) < 2e-5
            off += n
    bs.close()


def test_batch_zero_rhs_cap_and_determinism(ctx):
    pixes, rhs = small_batch(3, 4, seed=17)
    recs, b = to_form("w", pixes, rhs)
    b[:, 2] = 0.0  # x = 0 is exact: converged with no iteration
    bs = BatchSolver(ctx, "w", recs, EXACT, n_rhs=4)
    x, res = bs.solve_mixed(b, MixedParams(tol=1e-8))
    assert res.converged.all()
    assert (res.iters[:, 2] == 0).all() and not np.any(x[:, 2])
    x2, res2 = bs.solve_mixed(b, MixedParams(tol=1e-8))
    assert np.array_equal(x, x2) and np.array_equal(res.iters, res2.iters)
    # the profiled solve (iterations launched one by one, not from the
    # graph) takes the same steps
    ctx.set_profiling(True)
    x3, res3 = bs.solve_mixed(b, MixedParams(tol=1e-8))
    ctx.set_profiling(False)
    prof = ctx.profile()
    assert np.array_equal(x, x3) and np.array_equal(res.iters, res3.iters)
    assert prof["f32_launches"] >= res.iters.max() and prof["f32_evaluated"] > 0
    assert prof["f64_launches"] >= res.n_updates.max() and prof["f64_evaluated"] > 0
    # an iteration cap ends with an FP64 update and converged = False
    _, res3 = bs.solve_mixed(b, MixedParams(max_iter=4, tol=1e-12))
    assert res3.status == 3
    nz = [0, 1, 3]
    assert not res3.converged[:, nz].any() and (res3.iters[:, nz] == 4).all()
    assert (res3.n_updates[:, nz] >= 1).all()
    bs.close()


def test_batch_autotuner_choice(ctx):
    pixes, rhs = small_batch(8, 16, seed=23, sk=(4, 16), per=(32, 64))
    recs, b = to_form("w", pixes, rhs)
    bs = BatchSolver(ctx, "w", recs, EXACT, n_rhs=16)
    bs.set_variant("auto")
    inf = bs.info()
    assert inf["variant"] in (0, 1) and 16 % inf["rhs_block"] == 0
    x, res = bs.solve_mixed(b, MixedParams(tol=1e-8))
    assert res.converged.all() and res.rel_resid.max() <= 1e-8
    assert inf["n_chunks"] == 8 and inf["n_total"] == sum(r.shape[0] for r in recs)
    assert inf["n_pad"] % 128 == 0 and inf["inner_tile_pairs"] <= inf["outer_tile_pairs"]
    bs.close()


def test_tensor_core_wait_timeout_is_reported_and_recoverable(ctx):
    """The tcgen05 matvec's bounded waits: with a bound of 1 SM clock cycle
    the first wait that is not already satisfied runs out, the kernel records
    its code, waits (with the default bound) for its own MMAs and copies in
    flight, frees its tensor memory and returns, and the solve raises
    DS_ERR_TIMEOUT.  With the default bound restored the same batch on the
    same context solves to tolerance and agrees with the CUDA-core variant,
    so the failed launches left the context and the tensor memory usable."""
    from dachshund_gb300 import _lib
    from dachshund_gb300._lib import DsError

    pixes, rhs = small_batch(3, 16, seed=77, sk=(3, 8), per=(16, 40))
    recs, b = to_form("w", pixes, rhs)
    bs = BatchSolver(ctx, "w", recs, EXACT, n_rhs=16)
    bs.set_variant("tensor")
    assert bs.info()["variant"] == 1
    try:
        ctx.set_wait_limit(1)
        with pytest.raises(DsError) as ei:
            bs.solve_mixed(b, MixedParams(max_iter=20, tol=1e-8))
        assert ei.value.code == _lib.DS_ERR_TIMEOUT
    finally:
        ctx.set_wait_limit(0)
    for _ in range(2):
        x, res = bs.solve_mixed(b, MixedParams(tol=1e-8))
        assert res.status == 0 and res.converged.all() and res.rel_resid.max() <= 1e-8
    bs.set_variant("cuda_core")
    xc, resc = bs.solve_mixed(b, MixedParams(tol=1e-8))
    assert resc.converged.all()
    assert rel(x, xc) < 1e-6
    bs.close()


@pytest.mark.parametrize("n_rhs", [16, 32, 64])
def test_batch_tensor_core_product_and_solve(ctx, n_rhs):
    """The tcgen05 BF16 hi/lo matvec: product within 1e-4 of the FP64 oracle
    (max norm, relative to the largest entry), the solve within 1e-6 of the
    oracle's converged solutions and at most tol in FP64 residual."""
    import torch

    pixes, rhs = small_batch(4, n_rhs, seed=31 + n_rhs, sk=(3, 12), per=(16, 48))
    recs, b = to_form("w", pixes, rhs)
    bs = BatchSolver(ctx, "w", recs, EXACT, n_rhs=n_rhs)
    bs.set_variant("tensor")
    assert bs.info()["variant"] == 1
    p = np.random.default_rng(2).standard_normal(b.shape)
    pt = torch.tensor(p, dtype=torch.float64, device="cuda")
    qt = torch.zeros_like(pt)
    bs.product_f32_dev(pt, qt)
    torch.cuda.synchronize()
    q = qt.cpu().numpy()
    off = 0
    for rec in recs:
        n = rec.shape[0]
        for r in range(n_rhs):
            qo = oracle.A_product("w", rec, p[off:off + n, r], VS, LP, LQ, exact=True)
            assert rel(q[off:off + n, r], qo) < 1e-4, r
        off += n
    cols = [0, n_rhs // 2, n_rhs - 1]
    x, res = bs.solve_mixed(b, MixedParams(tol=1e-8))
    assert res.status == 0 and res.converged.all() and res.rel_resid.max() <= 1e-8
    xo = oracle_solutions("w", recs, np.ascontiguousarray(b[:, cols]))
    assert rel(x[:, cols], xo) < 1e-6
    true = oracle_rel_resid("w", recs, np.ascontiguousarray(b[:, cols]),
                            np.ascontiguousarray(x[:, cols]))
    assert true.max() <= 1e-8 * (1 + 1e-6)
    bs.close()
