"""GPU tests of the tensor-core inner matvec of the mixed-precision form
(pair exponents by tcgen05 TF32 MMAs, pair_tc.cu) against the CUDA-core
inner matvec (pair_f32.cu), the plain FP64 GPU solve and the CPU oracle.

Both inner kernels only steer the FP32 iterations: the stopping test is the
FP64-accurate true residual, so both must reach |b - A x| <= tol |b| and agree
with the FP64 solution to 1e-6 relative; the tensor-core operator's exponent
error (~1e-6 near the diagonal, 3xTF32 products) may cost a few iterations,
bounded here at 10% + 5 over the CUDA-core count.
"""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (MixedParams, PCGParams, SignalCovarParams, WFVectorSN, WFVectorW,
                             pixel_to_npixel, pixel_to_wpixel, synth)

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
    return np.linalg.norm(op.A_residual(y)) / np.linalg.norm(rec[:, 4])


def both(op):
    op.set_inner_matvec("cuda_core")
    xc, rc = op.solve_mixed(MixedParams(tol=1e-8))
    op.set_inner_matvec("tensor")
    xt, rt = op.solve_mixed(MixedParams(tol=1e-8))
    op.set_inner_matvec("auto")
    return (xc, rc), (xt, rt)


@pytest.mark.parametrize("form", ["w", "sn"])
def test_tensor_inner_matches_oracle(ctx, form):
    w = synth.small(24, 48, 14.0, seed=21)
    op, rec = make(ctx, form, w.pixels)
    (xc, rc), (xt, rt) = both(op)
    assert rc.success and rt.success
    assert true_residual(op, rec, form, xt) <= 1e-8 * (1 + 1e-6)
    xo, ok, _, _ = oracle.solve_pcg(form, rec, VS, LP, LQ, 2000, 50, 1e-10, exact=True)
    assert ok and rel(xt, xo) < 1e-6 and rel(xc, xo) < 1e-6
    assert rt.num_iters <= 1.1 * rc.num_iters + 5


def test_tensor_inner_many_row_tiles(ctx):
    # 24,576 pixels: 192 row tiles, more than one per CTA of the persistent grid
    w = synth.small(96, 256, 24.0, seed=7)
    op, rec = make(ctx, "w", w.pixels)
    (xc, rc), (xt, rt) = both(op)
    assert rc.success and rt.success
    assert true_residual(op, rec, "w", xt) <= 1e-8 * (1 + 1e-6)
    xp, rp = op.solve_pcg(PCGParams(3000, 50, 1e-10))
    assert rp.success
    assert rel(xt, xp) < 1e-6 and rel(xc, xp) < 1e-6
    assert rt.num_iters <= 1.1 * rc.num_iters + 5


def test_tensor_inner_initial_guess_and_cap(ctx):
    w = synth.small(32, 64, 16.0, seed=4)
    op, rec = make(ctx, "w", w.pixels)
    op.set_inner_matvec("tensor")
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    assert res.success
    x2, res2 = op.solve_mixed(MixedParams(tol=1e-6), x / rec[:, 3])
    assert res2.success and res2.num_iters <= 2
    _, res3 = op.solve_mixed(MixedParams(max_iter=5, tol=1e-12))
    assert not res3.success and res3.num_iters == 5
    op.set_inner_matvec("auto")


def test_inner_variant_rejects_bad_value(ctx):
    w = synth.small(8, 32, 8.0, seed=1)
    op, _ = make(ctx, "w", w.pixels)
    assert op._lib.ds_operator_set_inner_matvec(op.handle, 7) != 0
