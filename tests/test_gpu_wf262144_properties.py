"""Size-independent checks at the full 262,144-pixel workload (1,024 skewers
x 256 pixels in [0,80)^2 x [0,512) Mpc/h, GRF data, exact kernel, W form),
where the oracle cannot solve the whole system in seconds.

* The FP64 operator is symmetric and linear: u.(A v) = v.(A u) and
  A(2u - v/2) = 2 A u - A v / 2, to round-off.  A = I + w S w has no negative
  entry in the W form, so A|v| bounds the round-off of every sum.
* Rows of A a at both ends of the record order match the oracle's rows
  (lib/wf_vector.cc:196-220 with the exact kernel) to 1e-11 of A|a|.
* The mixed-precision solve stops on |b - A x| <= 1e-8 |b|, and the FP64
  operator agrees (lib/pcg.h:27-160 stopping rule).
* The FP32 map (80 x 80 x 512 grid) of that solution matches the oracle's
  FP64 map rows (lib/map.cc:20-43, exact kernel) on 4,096 grid points (a
  corner slab and a slab at the box centre) to 1e-6 of max |m|."""
import numpy as np
import pytest

import oracle
from dachshund_gb300 import (MapGrid, MixedParams, SignalCovarParams, WFVectorW,
                             pixel_to_wpixel, synth)

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA


@pytest.fixture(scope="module")
def workload():
    return synth.wf262144(0)


@pytest.fixture(scope="module")
def system(ctx, workload):
    rec = pixel_to_wpixel(workload.pixels)
    op = WFVectorW(ctx, rec, SignalCovarParams(VS, LP, LQ, eval="exact"))
    yield rec, op
    op.close()


def test_operator_symmetric_and_linear(system):
    rec, op = system
    n = rec.shape[0]
    assert n == 262_144
    rng = np.random.default_rng(11)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    au, av = op.A_product(u), op.A_product(v)
    a_abs_v = op.A_product(np.abs(v))
    scale = float(np.abs(u) @ a_abs_v)
    assert abs(float(u @ av) - float(v @ au)) <= 1e-11 * scale
    lhs = op.A_product(2.0 * u - 0.5 * v)
    bound = op.A_product(2.0 * np.abs(u) + 0.5 * np.abs(v))
    assert np.all(np.abs(lhs - (2.0 * au - 0.5 * av)) <= 1e-11 * bound)


def test_rows_match_oracle(system):
    rec, op = system
    n = rec.shape[0]
    a = np.random.default_rng(12).standard_normal(n)
    b = op.A_product(a)
    bound = op.A_product(np.abs(a))
    for r0, r1 in ((0, 32), (n - 32, n)):
        ref = oracle.A_product_rows("w", rec, a, r0, r1, VS, LP, LQ, exact=True)
        assert np.all(np.abs(b[r0:r1] - ref) <= 1e-11 * bound[r0:r1])


def test_mixed_solve_residual(system):
    rec, op = system
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    assert res.success and res.n_outer >= 1
    y = x / rec[:, 3]  # the W form returns x = w y
    r = op.A_residual(y)
    assert np.linalg.norm(r) <= 1e-8 * (1 + 1e-6) * np.linalg.norm(rec[:, 4])


def test_fp32_map_matches_oracle_rows(ctx, system, workload):
    rec, op = system
    w = workload
    x, res = op.solve_mixed(MixedParams(tol=1e-8))
    assert res.success
    pts = synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny, w.map_nz)
    grid = MapGrid(ctx, pts)
    m = grid.product_f32(op, x)
    grid.close()
    mid = (w.n_map // 2) - 1024
    for r0 in (0, mid):
        ref = oracle.smp_product_rows(w.pixels[:, :3], pts, x, r0, r0 + 2048, VS, LP, LQ,
                                      exact=True)
        err = np.max(np.abs(m[r0:r0 + 2048] - ref)) / np.max(np.abs(ref))
        assert err <= 1e-6, (r0, err)
