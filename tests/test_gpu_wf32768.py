"""The 32,768-pixel workload (256 skewers x 128 pixels in [0,40)^2 x [0,256)
Mpc/h, GRF data, tol 1e-8, W form), dense and matrix-free.

* The dense operator in HBM (32,768^2 FP64 = 8.6 GB, float-pair matvec) and
  the matrix-free FP64 kernel give the same product to 1e-12 of A|a|, for the
  exact and the table kernel; the FP64-FMA dense matvec agrees with the
  float-pair one to 1e-13 of A|a|.  A = I + w S w has no negative entry in
  the W form, so A|a| bounds the round-off of every sum.
* 64 rows of the dense product (both ends of the record order) match the
  oracle's rows (lib/wf_vector.cc:196-220, exact kernel) to 1e-11 of A|a|.
* The dense PCG (lib/pcg.h:27-160) reaches |b - A x| <= 1e-8 |b| checked by
  the matrix-free operator, within 2 iterations of the matrix-free PCG, and
  at a forced equal iteration count the two solutions agree to 1e-8.
* The mixed-precision solve reaches the same FP64 residual."""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (MixedParams, PCGParams, SignalCovarParams, WFVectorW,
                             pixel_to_wpixel, synth)

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA


@pytest.fixture(scope="module")
def wl():
    w = synth.wf32768(0)
    assert w.n == 32_768
    return w, pixel_to_wpixel(w.pixels)


@pytest.fixture(scope="module")
def exact_ops(ctx, wl):
    """Matrix-free and dense operators of the exact kernel (W form)."""
    _, rec = wl
    sp = SignalCovarParams(VS, LP, LQ, eval="exact")
    mf, dn = WFVectorW(ctx, rec, sp), WFVectorW(ctx, rec, sp)
    dn.set_dense(True)
    yield mf, dn
    dn.close()
    mf.close()


def test_dense_matches_matrix_free_exact(exact_ops, wl):
    mf, dn = exact_ops
    _, rec = wl
    assert dn.dense_arith() == "float_pair"
    a = np.random.default_rng(31).standard_normal(rec.shape[0])
    bound = mf.A_product(np.abs(a))
    assert np.all(np.abs(dn.A_product(a) - mf.A_product(a)) <= 1e-12 * bound)
    x = np.random.default_rng(32).standard_normal(rec.shape[0])
    assert np.all(np.abs(dn.A_residual(x) - mf.A_residual(x))
                  <= 1e-12 * (mf.A_product(np.abs(x)) + np.abs(rec[:, 4])))


def test_dense_fp64_arith_agrees(exact_ops, wl):
    _, dn = exact_ops
    _, rec = wl
    a = np.random.default_rng(33).standard_normal(rec.shape[0])
    b_ff = dn.A_product(a)
    dn.set_dense_arith("fp64")
    try:
        assert dn.dense_arith() == "fp64"
        b64 = dn.A_product(a)
        bound = dn.A_product(np.abs(a))
    finally:
        dn.set_dense_arith("auto")
    assert np.all(np.abs(b_ff - b64) <= 1e-13 * bound)


def test_dense_rows_match_oracle(exact_ops, wl):
    _, dn = exact_ops
    _, rec = wl
    n = rec.shape[0]
    a = np.random.default_rng(34).standard_normal(n)
    b = dn.A_product(a)
    bound = dn.A_product(np.abs(a))
    for r0, r1 in ((0, 32), (n - 32, n)):
        ref = oracle.A_product_rows("w", rec, a, r0, r1, VS, LP, LQ, exact=True)
        assert np.all(np.abs(b[r0:r1] - ref) <= 1e-11 * bound[r0:r1])


def test_dense_pcg_matches_matrix_free(exact_ops, wl):
    mf, dn = exact_ops
    w, rec = wl
    pp = PCGParams(1000, w.pcg_step_r, w.pcg_tol)
    xd, rd = dn.solve_pcg(pp)
    xm, rm = mf.solve_pcg(pp)
    assert rd.success and rm.success
    assert abs(rd.num_iters - rm.num_iters) <= 2
    y = xd / rec[:, 3]  # the W form returns x = w y
    r = mf.A_residual(y)
    assert np.linalg.norm(r) <= 1e-8 * (1 + 1e-6) * np.linalg.norm(rec[:, 4])
    k = min(rd.num_iters, rm.num_iters) + 1
    xd2, _ = dn.solve_pcg(PCGParams(k, w.pcg_step_r, 0.0))
    xm2, _ = mf.solve_pcg(PCGParams(k, w.pcg_step_r, 0.0))
    assert np.max(np.abs(xd2 - xm2)) <= 1e-8 * np.max(np.abs(xm2))


def test_mixed_solve_residual(exact_ops, wl):
    mf, _ = exact_ops
    _, rec = wl
    x, res = mf.solve_mixed(MixedParams(tol=1e-8))
    assert res.success and res.n_outer >= 1
    r = mf.A_residual(x / rec[:, 3])
    assert np.linalg.norm(r) <= 1e-8 * (1 + 1e-6) * np.linalg.norm(rec[:, 4])


def test_dense_matches_matrix_free_table(ctx, wl):
    _, rec = wl
    sp = SignalCovarParams(VS, LP, LQ, eval="table")
    mf, dn = WFVectorW(ctx, rec, sp), WFVectorW(ctx, rec, sp)
    try:
        dn.set_dense(True)
        a = np.random.default_rng(35).standard_normal(rec.shape[0])
        bound = mf.A_product(np.abs(a))
        assert np.all(np.abs(dn.A_product(a) - mf.A_product(a)) <= 1e-12 * bound)
    finally:
        dn.close()
        mf.close()
