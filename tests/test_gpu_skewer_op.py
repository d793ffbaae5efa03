"""GPU tests of the structured FP64 operator for skewers on a shared uniform
z grid (ds_operator_set_skewer_grid; no reference counterpart for the
evaluation order, the operator is lib/wf_vector.cc:196-251 with the exact
kernel of lib/signal_covar.h:79-86).

* A v and b - A v agree with the oracle's FP64 products to 1e-12 of A|v| (the
  W form's A has no negative entry, so A|v| bounds the round-off of every
  sum) and with the pair-kernel FP64 product, in both forms.
* Records that are not skewers on one uniform grid, and the table kernel,
  are refused with DS_ERR_ARG.
* The mixed-precision solve with the structured FP32 inner product and FP64
  outer residual stops on the FP64 true residual <= tol |b| (checked with
  the pair-kernel operator) and its solution is within 1e-6 of the FP64
  oracle's and of the pair-kernel solve's.
"""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (MixedParams, SignalCovarParams, WFVectorSN, WFVectorW,
                             pixel_to_npixel, pixel_to_wpixel, synth)
from dachshund_gb300._lib import DS_ERR_ARG, DsError

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA
EXACT = SignalCovarParams(VS, LP, LQ, eval="exact")


def make(ctx, form, pix, sp=EXACT):
    if form == "sn":
        rec = pixel_to_npixel(pix)
        return WFVectorSN(ctx, rec, sp), rec
    rec = pixel_to_wpixel(pix)
    return WFVectorW(ctx, rec, sp), rec


@pytest.mark.parametrize("form", ["w", "sn"])
def test_products_match_oracle(ctx, form):
    n_sk, n_per = 24, 48
    w = synth.small(n_sk, n_per, 9.0, seed=31)
    op, rec = make(ctx, form, w.pixels)
    op.set_skewer_grid(n_sk, n_per)
    v = np.random.default_rng(4).standard_normal(rec.shape[0])
    q = op.skewer_product(v)
    qo = oracle.A_product(form, rec, v, VS, LP, LQ, exact=True)
    bound = oracle.A_product(form, rec, np.abs(v), VS, LP, LQ, exact=True)
    assert np.max(np.abs(q - qo) / bound) < 1e-12
    assert np.max(np.abs(q - op.A_product(v)) / bound) < 1e-13
    r = op.skewer_product(v, residual=True)
    assert np.max(np.abs(r - (rec[:, 4] - qo)) / (bound + np.abs(rec[:, 4]))) < 1e-12
    op.close()


def test_refused_without_grid_structure(ctx):
    n_sk, n_per = 8, 32
    w = synth.small(n_sk, n_per, 6.0, seed=2)
    pix = w.pixels.copy()
    pix[5, 2] += 1e-3  # one pixel off the shared z grid
    op, _ = make(ctx, "w", pix)
    with pytest.raises(DsError) as ei:
        op.set_skewer_grid(n_sk, n_per)
    assert ei.value.code == DS_ERR_ARG
    op.close()
    pix = w.pixels.copy()
    pix[n_per + 3, 0] += 1e-3  # one pixel off its skewer's (x, y)
    op, _ = make(ctx, "w", pix)
    with pytest.raises(DsError):
        op.set_skewer_grid(n_sk, n_per)
    with pytest.raises(DsError):
        op.set_skewer_grid(n_sk - 1, n_per)
    op.close()
    op, _ = make(ctx, "w", w.pixels, SignalCovarParams(VS, LP, LQ))  # table kernel
    with pytest.raises(DsError):
        op.set_skewer_grid(n_sk, n_per)
    op.close()


@pytest.mark.parametrize("form", ["w", "sn"])
@pytest.mark.parametrize("n_sk,n_per,cluster", [(32, 64, 4), (10, 50, 0)])
def test_mixed_solve_structured(ctx, form, n_sk, n_per, cluster):
    """The structured FP32 inner product and FP64 outer residual (with the
    cluster preconditioner, and with Jacobi on a record count that leaves
    padding in the last tile): FP64 true residual <= tol |b|, solution within
    1e-6 of the oracle's, and within 1e-6 of the pair-kernel solve."""
    w = synth.small(n_sk, n_per, 12.0 * np.sqrt(n_sk / 32), seed=17)
    op, rec = make(ctx, form, w.pixels)
    mp = MixedParams(tol=1e-8)
    if cluster:
        op.set_cluster_preconditioner(n_sk, n_per, cluster=cluster, band=16)
    x0, r0 = op.solve_mixed(mp)
    op.set_skewer_grid(n_sk, n_per)
    x, res = op.solve_mixed(mp)
    assert res.success and r0.success and res.n_outer >= 1
    y = x / rec[:, 3] if form == "w" else x
    assert np.linalg.norm(op.A_residual(y)) <= 1e-8 * (1 + 1e-6) * np.linalg.norm(rec[:, 4])
    xo, ok, _, _ = oracle.solve_pcg(form, rec, VS, LP, LQ, 3000, 50, 1e-10, exact=True)
    assert ok
    assert np.max(np.abs(x - xo)) / np.max(np.abs(xo)) < 1e-6
    assert np.max(np.abs(x - x0)) / np.max(np.abs(x0)) < 1e-6
    assert abs(res.num_iters - r0.num_iters) <= max(3, r0.num_iters // 10)
    # the pair kernel as inner matvec, structured outer residual
    op.set_inner_matvec("cuda_core")
    x1, r1 = op.solve_mixed(mp)
    assert r1.success and np.max(np.abs(x1 - xo)) / np.max(np.abs(xo)) < 1e-6
    op.set_inner_matvec("auto")
    op.set_skewer_grid(0, 0)
    op.close()


def test_structured_map_matches_oracle(ctx):
    """The structured FP64 map (column grid x skewer grid) against the
    oracle's FP64 smp_product with the exact kernel (lib/map.cc:20-43) and
    the pair-kernel FP64 map: within 1e-12 of the largest |m| (the cutoff at
    exponent 30 drops terms below 1e-13 of var_s |x_j|)."""
    from dachshund_gb300 import MapGrid

    n_sk, n_per = 20, 40
    w = synth.small(n_sk, n_per, 8.0, seed=11)
    op, rec = make(ctx, "sn", w.pixels)
    op.set_skewer_grid(n_sk, n_per)
    nx, ny, nz = 6, 5, 2 * n_per  # map z every 1 Mpc/h, pixels every 2
    pts = synth.uniform_map_coords(8.0, 8.0, n_per * synth.DZ, nx, ny, nz)
    grid = MapGrid(ctx, pts)
    x = np.random.default_rng(3).standard_normal(rec.shape[0])
    m_pair = grid.product_f32(op, x)  # no column grid yet: the FP32 pair kernel
    grid.set_column_grid(nx * ny, nz)
    m = grid.product_f32(op, x)
    mo = oracle.smp_product(w.pixels[:, :3], pts, x, VS, LP, LQ, exact=True)
    scale = np.max(np.abs(mo))
    assert np.max(np.abs(m - mo)) / scale < 1e-12
    assert np.max(np.abs(m - grid.product(op, x))) / scale < 1e-12
    assert np.max(np.abs(m_pair - mo)) / scale < 1e-6
    # repeated products reuse the lists; removing the grid returns to the pair kernel
    assert np.array_equal(grid.product_f32(op, x), m)
    grid.set_column_grid(0, 0)
    assert np.max(np.abs(grid.product_f32(op, x) - mo)) / scale < 1e-6
    grid.close()
    op.close()


def test_column_grid_refused_for_other_layouts(ctx):
    from dachshund_gb300 import MapGrid

    pts = synth.uniform_map_coords(8.0, 8.0, 40.0, 4, 4, 10)
    grid = MapGrid(ctx, pts[np.random.default_rng(1).permutation(pts.shape[0])])
    with pytest.raises(DsError):
        grid.set_column_grid(16, 10)
    grid.close()
    grid = MapGrid(ctx, pts)
    with pytest.raises(DsError):
        grid.set_column_grid(15, 10)
    grid.set_column_grid(16, 10)
    grid.close()
    for v in (np.inf, np.nan):  # map points are checked when the map is created
        bad = pts.copy()
        bad[5, 2] = v
        with pytest.raises(DsError):
            MapGrid(ctx, bad)


def test_map_points_tiled_on_first_pair_product(ctx):
    """A column-grid map against a skewer grid reads its points as given;
    their sorted, tiled copy is built by the first product that needs it
    (here the pair-kernel maps after the column grid is removed), with the
    same results as on a map tiled from the start."""
    from dachshund_gb300 import MapGrid

    n_sk, n_per = 20, 40
    w = synth.small(n_sk, n_per, 8.0, seed=11)
    op, rec = make(ctx, "sn", w.pixels)
    op.set_skewer_grid(n_sk, n_per)
    nx, ny, nz = 6, 5, 2 * n_per
    pts = synth.uniform_map_coords(8.0, 8.0, n_per * synth.DZ, nx, ny, nz)
    x = np.random.default_rng(3).standard_normal(rec.shape[0])
    grid = MapGrid(ctx, pts)
    grid.set_column_grid(nx * ny, nz)
    m_col = grid.product_f32(op, x)
    grid.set_column_grid(0, 0)
    m32_late = grid.product_f32(op, x)
    m64_late = grid.product(op, x)
    grid.close()
    grid = MapGrid(ctx, pts)
    m32_first = grid.product_f32(op, x)
    m64_first = grid.product(op, x)
    grid.close()
    scale = np.max(np.abs(m_col))
    assert np.max(np.abs(m32_late - m32_first)) / scale < 1e-12
    assert np.max(np.abs(m64_late - m64_first)) / scale < 1e-12
    assert np.max(np.abs(m64_late - m_col)) / scale < 1e-12
    op.close()


@pytest.mark.parametrize("form", ["w", "sn"])
@pytest.mark.parametrize("n_sk,n_per,cluster", [(64, 96, 4), (10, 50, 4), (24, 40, 8),
                                               (12, 64, 1), (30, 64, 4), (30, 32, 3),
                                               (16, 128, 2)])
def test_persistent_solve_matches_graph(ctx, form, n_sk, n_per, cluster):
    """The structured mixed solve with the cluster preconditioner as one
    cooperative launch (ds_operator_set_iteration_form AUTO) against the same
    recurrence as a replayed graph of per-phase kernels (GRAPH) -- the
    resident form where the pixels per skewer divide the CTA and clusters
    have at most 4 skewers (ragged last clusters included), the general form
    otherwise: both stop on
    the FP64 true residual <= tol |b|, their solutions agree with the oracle's
    to 1e-6, their iteration counts to rounding, and the persistent solve's
    launches do not grow with its iterations."""
    w = synth.small(n_sk, n_per, 12.0 * np.sqrt(n_sk / 32), seed=23)
    op, rec = make(ctx, form, w.pixels)
    op.set_cluster_preconditioner(n_sk, n_per, cluster=cluster, band=16)
    op.set_skewer_grid(n_sk, n_per)
    mp = MixedParams(tol=1e-8)
    op.set_iteration_form("graph")
    xg, rg = op.solve_mixed(mp)
    op.set_iteration_form("auto")
    l0 = ctx.profile()["kernel_launches"]
    xp, rp = op.solve_mixed(mp)
    launches = ctx.profile()["kernel_launches"] - l0
    assert rg.success and rp.success and rp.n_outer >= 1
    assert launches < 40, (launches, rp.num_iters)
    y = xp / rec[:, 3] if form == "w" else xp
    assert np.linalg.norm(op.A_residual(y)) <= 1e-8 * (1 + 1e-6) * np.linalg.norm(rec[:, 4])
    xo, ok, _, _ = oracle.solve_pcg(form, rec, VS, LP, LQ, 3000, 50, 1e-10, exact=True)
    assert ok
    scale = np.max(np.abs(xo))
    assert np.max(np.abs(xp - xo)) / scale < 1e-6
    assert np.max(np.abs(xp - xg)) / scale < 1e-6
    assert abs(rp.num_iters - rg.num_iters) <= max(3, rg.num_iters // 10)
    assert rp.residual_norms[0] == pytest.approx(rg.residual_norms[0], rel=1e-12)
    # a second solve on the same operator (barrier words reused)
    xp2, rp2 = op.solve_mixed(mp)
    assert rp2.success and rp2.num_iters == rp.num_iters and np.array_equal(xp2, xp)
    op.close()


def test_persistent_barrier_timeout_is_reported_and_recoverable(ctx):
    """The persistent solve's grid barriers are bounded: with a bound of one
    SM clock cycle every CTA but the last to arrive gives up at the first
    barrier, records the phase, and the launch ends; the solve raises
    DS_ERR_TIMEOUT.  With the default bound the same operator then solves to
    tolerance, so the failed launch left the context and buffers usable."""
    from dachshund_gb300 import _lib

    n_sk, n_per = 32, 64
    w = synth.small(n_sk, n_per, 12.0, seed=29)
    op, rec = make(ctx, "w", w.pixels)
    op.set_cluster_preconditioner(n_sk, n_per, cluster=4, band=16)
    op.set_skewer_grid(n_sk, n_per)
    mp = MixedParams(tol=1e-8)
    try:
        ctx.set_wait_limit(1)
        with pytest.raises(DsError) as ei:
            op.solve_mixed(mp)
        assert ei.value.code == _lib.DS_ERR_TIMEOUT
    finally:
        ctx.set_wait_limit(0)
    x, res = op.solve_mixed(mp)
    assert res.success
    y = x / rec[:, 3]
    assert np.linalg.norm(op.A_residual(y)) <= 1e-8 * (1 + 1e-6) * np.linalg.norm(rec[:, 4])
    op.close()


def test_persistent_profile_counts_phases(ctx):
    """The persistent launches' phase timers: one launch per solve, one
    product and one step phase per iteration, one FP64 update phase per
    reliable update, positive times, and the slowest CTA's work at least the
    mean; the reset clears them."""
    n_sk, n_per = 32, 64
    w = synth.small(n_sk, n_per, 12.0, seed=41)
    op, _ = make(ctx, "w", w.pixels)
    op.set_cluster_preconditioner(n_sk, n_per, cluster=4, band=16)
    op.set_skewer_grid(n_sk, n_per)
    assert op.persistent_profile() is None
    _, res = op.solve_mixed(MixedParams(tol=1e-8))
    prof = op.persistent_profile(reset=True)
    assert prof["launches"] == 1 and prof["ctas"] >= 1 and prof["kernel_ms"] > 0
    assert prof["barrier_us"] > 0
    assert prof["product"]["visits"] == res.num_iters
    assert prof["step"]["visits"] == res.num_iters
    assert prof["update"]["visits"] == res.n_outer
    for ph in ("product", "step"):
        assert prof[ph]["us_per_visit"] > 0
        assert prof[ph]["cta_max_us"] >= prof[ph]["cta_mean_us"] > 0
    # the resident form (64 pixels per skewer divide the CTA, clusters of 4):
    # each distinct (neighbour, level) row of a cluster loaded once
    assert prof["product_rows"] > 0 and prof["product_loads"] == prof["product_rows"] * n_per
    again = op.persistent_profile()
    assert again["launches"] == 0 and again["product"]["visits"] == 0
    op.close()
