"""GPU tests of the cluster preconditioner of the mixed-precision solve (an
FSAI factor M^-1 = G G^T over clusters of neighbouring skewers; no reference
counterpart, the reference's PCG is Jacobi, lib/wf_vector.cc:42-49,185-194).

* Both forms: the preconditioned solve stops on the FP64 true residual
  |b - A x| <= tol |b| and its solution is within 1e-6 of the FP64 oracle's
  (lib/pcg.h:27-160 with the exact kernel); removing the preconditioner
  gives back the Jacobi iteration count and solution.
* With the full pattern (band >= cluster size - 1) G G^T is the exact
  inverse of each cluster's block, so on clusters that do not couple to each
  other (pairs of skewers 100 Mpc/h apart) the solve needs a few iterations
  only (FP32 factor, FP64 reliable updates).
* Ragged clusters: skewer counts that are not a multiple of the cluster size
  leave padding slots in the last block.
* At the 262,144-pixel workload's skewer density (48 skewers x 256 pixels
  in [0, 17.3)^2 Mpc/h) the cluster factor saves at least 40% of the Jacobi
  iterations (the exact inverse of each skewer's own block saves 23% there).
"""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (MixedParams, SignalCovarParams, WFVectorSN, WFVectorW,
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


@pytest.mark.parametrize("form", ["w", "sn"])
def test_cluster_solve_matches_oracle(ctx, form):
    n_sk, n_per = 16, 64
    w = synth.small(n_sk, n_per, 8.0, seed=21)
    op, rec = make(ctx, form, w.pixels)
    mp = MixedParams(tol=1e-8)
    xj, rj = op.solve_mixed(mp)
    assert op.set_cluster_preconditioner(n_sk, n_per, cluster=4, band=16) == 0
    x, res = op.solve_mixed(mp)
    assert res.success and rj.success
    assert true_residual(op, rec, form, x) <= 1e-8 * (1 + 1e-6)
    xo, ok, _, _ = oracle.solve_pcg(form, rec, VS, LP, LQ, 3000, 50, 1e-10, exact=True)
    assert ok and rel(x, xo) < 1e-6
    assert res.num_iters < rj.num_iters
    op.set_cluster_preconditioner(n_sk, n_per, cluster=0)
    x2, r2 = op.solve_mixed(mp)
    assert r2.num_iters == rj.num_iters and rel(x2, xj) < 1e-12
    op.close()


def test_full_pattern_is_exact_block_inverse(ctx):
    """Two pairs of skewers 100 Mpc/h apart (no coupling between the pairs),
    12 pixels each: clusters of 2 with band 23 >= 24 - 1 slots."""
    rng = np.random.default_rng(5)
    n_per = 12
    xy = np.array([[0.0, 0.0], [1.5, 0.5], [100.0, 100.0], [101.0, 99.2]])
    pix = np.empty((4 * n_per, 5))
    pix[:, 0] = np.repeat(xy[:, 0], n_per)
    pix[:, 1] = np.repeat(xy[:, 1], n_per)
    pix[:, 2] = np.tile((np.arange(n_per) + 0.5) * synth.DZ, 4)
    pix[:, 3] = rng.uniform(0.05, 0.3, 4 * n_per)
    pix[:, 4] = rng.standard_normal(4 * n_per) * 0.3
    op, rec = make(ctx, "w", pix)
    _, rj = op.solve_mixed(MixedParams(tol=1e-8))
    assert op.set_cluster_preconditioner(4, n_per, cluster=2, band=23) == 0
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    assert res.success and true_residual(op, rec, "w", x) <= 1e-8 * (1 + 1e-6)
    assert res.num_iters <= 3 < rj.num_iters, (res.num_iters, rj.num_iters)
    op.close()


def test_ragged_last_cluster(ctx):
    n_sk, n_per = 11, 40
    w = synth.small(n_sk, n_per, 7.0, seed=3)
    op, rec = make(ctx, "w", w.pixels)
    assert op.set_cluster_preconditioner(n_sk, n_per, cluster=4, band=12) == 0
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    assert res.success and true_residual(op, rec, "w", x) <= 1e-8 * (1 + 1e-6)
    xo, ok, _, _ = oracle.solve_pcg("w", rec, VS, LP, LQ, 3000, 50, 1e-10, exact=True)
    assert ok and rel(x, xo) < 1e-6
    op.close()


def test_bad_arguments(ctx):
    from dachshund_gb300._lib import DsError

    w = synth.small(8, 32, 6.0, seed=1)
    op, _ = make(ctx, "w", w.pixels)
    for args in [(7, 32, 4, 16), (8, 32, 40, 16), (8, 32, 4, 25), (8, 32, 4, -1)]:
        with pytest.raises(DsError):
            op.set_cluster_preconditioner(*args)
    op.close()


def test_iteration_saving_at_workload_density(ctx):
    n_sk, n_per = 48, 256
    box = 80.0 * np.sqrt(n_sk / 1024)
    w = synth.grf_workload("t", n_sk, n_per, box, 3, (8, 8, 64), 1e-8)
    op, rec = make(ctx, "w", w.pixels)
    _, rj = op.solve_mixed(MixedParams(tol=1e-8))
    op.set_cluster_preconditioner(n_sk, n_per, cluster=4, band=16)
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    assert res.success and true_residual(op, rec, "w", x) <= 1e-8 * (1 + 1e-6)
    assert res.num_iters <= 0.6 * rj.num_iters, (res.num_iters, rj.num_iters)
    op.close()
