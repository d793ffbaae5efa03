"""GPU tests of the mixed-precision form (FP32 inner PCG, FP64 reliable
updates) against the plain FP64 GPU solve of the same exact-kernel system and
the CPU oracle.

Bars: the FP64 true residual |b - A x| <= tol |b| (checked independently
with the FP64 operator), and solution / map within 1e-6 relative of the FP64
oracle (the FP32 operator's ~1e-6 error is removed by the FP64 residual; the
map is evaluated in FP32 with FP64 accumulation).
"""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (MapGrid, MixedParams, PCGParams, SignalCovarParams, WFVectorSN,
                             WFVectorW, pixel_to_npixel, pixel_to_wpixel, synth)

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA
EXACT = SignalCovarParams(VS, LP, LQ, eval="exact")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def make(ctx, form, pix):
    if form == "sn":
        rec = pixel_to_npixel(pix)
        return WFVectorSN(ctx, rec, EXACT), rec
    rec = pixel_to_wpixel(pix)
    return WFVectorW(ctx, rec, EXACT), rec


def true_residual(op, rec, form, x):
    y = x / rec[:, 3] if form == "w" else x
    r = op.A_residual(y)
    return np.linalg.norm(r) / np.linalg.norm(rec[:, 4])


@pytest.mark.parametrize("form", ["w", "sn"])
def test_mixed_matches_fp64_and_oracle(ctx, form):
    w = synth.small(24, 48, 14.0, seed=21)
    op, rec = make(ctx, form, w.pixels)
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    assert res.success and res.n_outer >= 1
    assert true_residual(op, rec, form, x) <= 1e-8 * (1 + 1e-6)
    xp, resp = op.solve_pcg(PCGParams(2000, 50, 1e-10))
    assert resp.success
    assert rel(x, xp) < 1e-6
    xo, ok, _, _ = oracle.solve_pcg(form, rec, VS, LP, LQ, 2000, 50, 1e-10, exact=True)
    assert ok and rel(x, xo) < 1e-6


def test_mixed_iteration_count_close_to_fp64(ctx):
    w = synth.small(32, 64, 16.0, seed=4)
    op, rec = make(ctx, "w", w.pixels)
    _, res = op.solve_mixed(MixedParams(tol=1e-8))
    _, resp = op.solve_pcg(PCGParams(3000, 50, 1e-8))
    assert res.success and resp.success
    # FP32 inner iterations stay within 25% of the FP64 count.
    assert res.num_iters <= 1.25 * resp.num_iters + 5
    assert 1 <= res.n_outer <= 6


def test_mixed_initial_guess_and_cap(ctx):
    w = synth.small(16, 32, 12.0, seed=8)
    op, rec = make(ctx, "w", w.pixels)
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    # restart from the solution (the initial guess is in the operator's
    # unscaled variable, x / w): converges with no iteration
    x2, res2 = op.solve_mixed(MixedParams(tol=1e-6), x / rec[:, 3])
    assert res2.success and res2.num_iters == 0
    assert rel(x2, x) < 1e-12
    # an iteration cap ends with an FP64 update and success = False
    _, res3 = op.solve_mixed(MixedParams(max_iter=5, tol=1e-12))
    assert not res3.success and res3.num_iters == 5 and res3.n_outer >= 1


def test_map_f32_vs_fp64(ctx):
    w = synth.small(24, 48, 14.0, seed=13)
    op, rec = make(ctx, "w", w.pixels)
    x, _ = op.solve_mixed(MixedParams(tol=1e-8))
    pts = synth.uniform_map_coords(14.0, 14.0, 96.0, 14, 14, 96)
    grid = MapGrid(ctx, pts)
    m64 = grid.product(op, x)
    m32 = grid.product_f32(op, x)
    assert rel(m32, m64) < 1e-6
    mo = oracle.smp_product(w.pixels[:, :3], pts, x, VS, LP, LQ, exact=True)
    assert rel(m64, mo) < 1e-12
    assert rel(m32, mo) < 1e-6


def test_table_operator_rejected_by_mixed(ctx):
    w = synth.small(4, 8, 6.0, seed=1)
    op = WFVectorW(ctx, pixel_to_wpixel(w.pixels), SignalCovarParams(VS, LP, LQ))
    from dachshund_gb300 import DsError

    with pytest.raises(DsError):
        op.solve_mixed(MixedParams())


@pytest.mark.parametrize("form", ["w", "sn"])
def test_ff_residual_matches_fp64(ctx, form):
    """The float-float outer residual against the FP64 one: within 1e-12 of
    the largest |r| for a random x (about 1e-14 of the summed |S_ij x_j|) and
    within 1e-12 |b| at a converged solution (where |r| ~ 1e-8 |b|)."""
    w = synth.small(24, 48, 14.0, seed=33)
    op, rec = make(ctx, form, w.pixels)
    nb = np.linalg.norm(rec[:, 4])
    x = np.random.default_rng(3).standard_normal(op.n)
    r64 = op.A_residual(x)
    rff = op.A_residual_ff(x)
    assert np.max(np.abs(rff - r64)) <= 1e-12 * np.max(np.abs(r64))
    xs, res = op.solve_mixed(MixedParams(tol=1e-8))
    y = xs / rec[:, 3] if form == "w" else xs
    r64 = op.A_residual(y)
    rff = op.A_residual_ff(y)
    assert np.linalg.norm(rff - r64) <= 1e-12 * nb
    assert np.linalg.norm(r64) <= 1e-8 * nb * (1 + 1e-6)
