"""GPU tests of the dense paths: the dense operator in HBM (same matvec and
PCG as the matrix-free kernels), the closed-form solve (GPU Cholesky vs the
oracle's LDL^T), and MapCovarDiag against the reference's golden output."""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (PCGParams, SignalCovarParams, WFVectorSN, WFVectorW,
                             map_covar_diag, pixel_to_npixel, pixel_to_wpixel, solve_cf, synth)

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("form", ["w", "sn"])
@pytest.mark.parametrize("ev", ["table", "exact"])
def test_dense_operator_matches_matrix_free(ctx, form, ev):
    w = synth.small(20, 40, 14.0, seed=17)
    sp = SignalCovarParams(VS, LP, LQ, eval=ev)
    rec = pixel_to_wpixel(w.pixels) if form == "w" else pixel_to_npixel(w.pixels)
    cls = WFVectorW if form == "w" else WFVectorSN
    mf, dn = cls(ctx, rec, sp), cls(ctx, rec, sp)
    dn.set_dense(True)
    a = np.random.default_rng(3).standard_normal(w.n)
    assert rel(dn.A_product(a), mf.A_product(a)) < 1e-12
    assert rel(dn.A_residual(a), mf.A_residual(a)) < 1e-12
    x1, r1 = mf.solve_pcg(PCGParams(1000, 50, 1e-8))
    x2, r2 = dn.solve_pcg(PCGParams(1000, 50, 1e-8))
    assert r1.success and r2.success and abs(r1.num_iters - r2.num_iters) <= 2
    assert rel(x2, x1) < 1e-6
    xf1, _ = mf.solve_pcg(PCGParams(r1.num_iters + 1, 50, 0.0))
    xf2, _ = dn.solve_pcg(PCGParams(r1.num_iters + 1, 50, 0.0))
    assert rel(xf2, xf1) < 1e-8
    dn.set_dense(False)
    assert rel(dn.A_product(a), mf.A_product(a)) < 1e-12


@pytest.mark.parametrize("form", ["w", "sn"])
@pytest.mark.parametrize("exact", [False, True])
def test_solve_cf_matches_oracle(ctx, form, exact):
    w = synth.small(9, 40, 10.0, seed=23)  # 360 pixels, not a multiple of the panel
    rec = pixel_to_wpixel(w.pixels) if form == "w" else pixel_to_npixel(w.pixels)
    sp = SignalCovarParams(VS, LP, LQ, eval="exact" if exact else "table")
    x = solve_cf(ctx, form, rec, sp)
    xo = oracle.solve_cf(form, rec, VS, LP, LQ, exact=exact)
    assert rel(x, xo) < 1e-10


def test_solve_cf_matches_pcg(ctx, golden):
    g = golden["small"]
    rec = pixel_to_wpixel(g["pixels"])
    x = solve_cf(ctx, "w", rec, SignalCovarParams(VS, LP, LQ))
    assert rel(x, g["x_w"]) < 1e-6  # the golden PCG stopped at |r| <= 1e-8 |b|


def test_map_covar_diag_golden(ctx, golden):
    g = golden["small"]
    nrec = pixel_to_npixel(g["pixels"])
    s, iters, ok = map_covar_diag(ctx, nrec, g["cov_pts"], SignalCovarParams(VS, LP, LQ),
                                  PCGParams(1000, 50, 1e-6))
    assert ok.all() == g["cov_success"].all()
    assert np.all(np.abs(iters - g["cov_iters"]) <= 2)
    # Both stopped at |r| <= 1e-6 |b|; sigma = b . x agrees to ~tol * cond.
    assert rel(s, g["cov"]) < 1e-5


def test_map_covar_diag_exact_batched(ctx):
    """Exact-kernel MapCovarDiag runs groups of 64 map points as the
    right-hand sides of one batched mixed-precision solve; against the
    oracle's per-point FP64 Jacobi-PCG (both to |r| <= 1e-8 |b|): sigma within
    1e-6 relative, all solves successful, iteration counts close."""
    w = synth.small(16, 64, 12.0, seed=5)
    nrec = pixel_to_npixel(w.pixels)
    rng = np.random.default_rng(2)
    pts = np.column_stack([rng.uniform(0, 12.0, 100), rng.uniform(0, 12.0, 100),
                           rng.uniform(0, 64 * synth.DZ, 100)])
    sp = SignalCovarParams(VS, LP, LQ, eval="exact")
    s, iters, ok = map_covar_diag(ctx, nrec, pts, sp, PCGParams(1000, 50, 1e-8))
    so, io, oko = oracle.map_covar_diag(nrec, pts, VS, LP, LQ, 1000, 50, 1e-8, exact=True)
    assert ok.all() and oko.all()
    assert rel(s, so) < 1e-6
    assert np.all(np.abs(iters - io) <= 0.25 * io + 5)


def test_dense_signed_entries(ctx):
    """W-form records with some negative weights give negative entries: the
    float-pair matvec carries the signs (matrix-free FP64 as the yardstick)."""
    w = synth.small(12, 40, 10.0, seed=29)
    rec = pixel_to_wpixel(w.pixels)
    rec[::3, 3] *= -1.0
    rec[::3, 4] *= -1.0
    sp = SignalCovarParams(VS, LP, LQ, eval="exact")
    mf, dn = WFVectorW(ctx, rec, sp), WFVectorW(ctx, rec, sp)
    dn.set_dense(True)
    assert dn.dense_arith() == "float_pair"
    a = np.random.default_rng(4).standard_normal(w.n)
    scale = np.max(np.abs(mf.A_product(np.abs(a))))
    assert np.max(np.abs(dn.A_product(a) - mf.A_product(a))) <= 1e-12 * scale
    dn.close()
    mf.close()


def test_dense_out_of_range_entries_use_fp64(ctx):
    """Entries below 2^-100 (var_s = 1e-40) cannot be split into float pairs;
    the dense operator then multiplies in FP64."""
    w = synth.small(8, 40, 8.0, seed=30)
    rec = pixel_to_npixel(w.pixels)
    sp = SignalCovarParams(1e-40, LP, LQ, eval="exact")
    mf, dn = WFVectorSN(ctx, rec, sp), WFVectorSN(ctx, rec, sp)
    dn.set_dense(True)
    assert dn.dense_arith() == "fp64"
    a = np.random.default_rng(5).standard_normal(w.n)
    assert rel(dn.A_product(a), mf.A_product(a)) < 1e-12
    dn.close()
    mf.close()


@pytest.mark.parametrize("n_pts", [37, 300])
def test_map_covar_diag_table_multi_rhs(ctx, n_pts):
    """The table kernel's MapCovarDiag solves up to 256 map points per
    multi-RHS FP64 PCG (the smallest power of two from 16 covering them);
    against the oracle's per-point solves (lib/map_covar.cc:73-113): the same
    success flags (points far from every pixel have |b| = 0 and fail as the
    reference's early return), iteration counts within 2, sigma within 1e-6
    relative.  37 points: one ragged solve of 64; 300 points: a full solve of
    256 (more right-hand sides than a vector-kernel block has threads) and a
    ragged one."""
    w = synth.small(12, 48, 10.0, seed=13)
    nrec = pixel_to_npixel(w.pixels)
    rng = np.random.default_rng(9)
    pts = np.column_stack([rng.uniform(0, 10.0, n_pts), rng.uniform(0, 10.0, n_pts),
                           rng.uniform(0, 48 * synth.DZ, n_pts)])
    far = [3, 20, n_pts - 1]
    pts[far] = [500.0, 500.0, 5.0]  # no pixel within the table's cutoff
    sp = SignalCovarParams(VS, LP, LQ)
    s, iters, ok = map_covar_diag(ctx, nrec, pts, sp, PCGParams(1000, 50, 1e-8))
    so, io, oko = oracle.map_covar_diag(nrec, pts, VS, LP, LQ, 1000, 50, 1e-8, exact=False)
    assert np.array_equal(ok.astype(bool), np.asarray(oko).astype(bool))
    assert not ok[far].any() and np.all(s[far] == 0.0)
    good = np.asarray(oko).astype(bool)
    assert good.sum() == n_pts - 3
    assert np.all(np.abs(iters[good] - np.asarray(io)[good]) <= 2)
    assert rel(s[good], np.asarray(so)[good]) < 1e-6
