"""CPU checks of the Gaussian-random-field data generator (dachshund_gb300/synth.py)
that feeds the GRF workloads.

The field is drawn with the kernel's own power spectrum, so its covariance
is the kernel: xi(r) = var_s exp(-r_perp^2 / (2 l_perp^2) - r_para^2 /
(2 l_para^2)).  Checked on a periodic grid against that closed form:
* the sample variance, and the covariance at lags of 1-3 cells along x, y
  and z, within a few standard errors of the estimate;
* trilinear interpolation: exact at cell centres, and at random points the
  mean square matches the interpolation weights applied to xi (the
  smoothing it introduces);
* the workload's d = signal + n N(0, 1) has the variance of the two parts.
"""
import numpy as np

from dachshund_gb300 import synth

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA


def xi(dx, dy, dz):
    return VS * np.exp(-(dx * dx + dy * dy) / (2 * LP**2) - dz * dz / (2 * LQ**2))


def fields(n_fields=4, shape=(64, 64, 96)):
    return [synth.grf_field(np.random.default_rng(100 + s), shape) for s in range(n_fields)]


def test_grf_variance_and_covariance():
    fs = fields()
    var = np.mean([np.mean(f * f) for f in fs])
    # ~4 x 393k cells with a correlation volume of ~200 cells: the variance
    # estimate has a relative standard error near 1.1%
    assert abs(var / VS - 1.0) < 0.05, var
    for lag in (1, 2, 3):
        for axis, expect in ((0, xi(lag, 0, 0)), (1, xi(0, lag, 0)), (2, xi(0, 0, lag))):
            cov = np.mean([np.mean(f * np.roll(f, lag, axis=axis)) for f in fs])
            assert abs(cov - expect) < 0.05 * VS, (lag, axis, cov, expect)
    # the field has zero mean (the k = 0 mode carries P(0) / V of variance)
    assert abs(np.mean([f.mean() for f in fs])) < 0.05 * np.sqrt(VS)


def test_trilinear_exact_at_cell_centres():
    f = synth.grf_field(np.random.default_rng(7), (16, 16, 32))
    ix, iy, iz = np.meshgrid(np.arange(16), np.arange(16), np.arange(32), indexing="ij")
    pts = np.column_stack([ix.ravel() + 0.5, iy.ravel() + 0.5, iz.ravel() + 0.5])
    np.testing.assert_allclose(synth.trilinear(f, pts), f.ravel(), rtol=0, atol=1e-15)


def test_trilinear_smoothing_matches_weights():
    """E[d(x)^2] for d the trilinear interpolation of the field equals
    sum_ab w_a w_b xi(r_ab) over the 8 surrounding cell centres."""
    rng = np.random.default_rng(3)
    shape = (64, 64, 96)
    pts = rng.uniform(0, 1, size=(20000, 3)) * np.array(shape)
    sq = np.mean([np.mean(synth.trilinear(f, pts) ** 2) for f in fields(shape=shape)])
    g = pts - 0.5
    frac = g - np.floor(g)
    corners = [(a, b, c) for a in (0, 1) for b in (0, 1) for c in (0, 1)]
    w = np.stack([np.where(a, frac[:, 0], 1 - frac[:, 0]) * np.where(b, frac[:, 1], 1 - frac[:, 1])
                  * np.where(c, frac[:, 2], 1 - frac[:, 2]) for a, b, c in corners], axis=1)
    expect = 0.0
    for i, (a1, b1, c1) in enumerate(corners):
        for j, (a2, b2, c2) in enumerate(corners):
            expect = expect + w[:, i] * w[:, j] * xi(a1 - a2, b1 - b2, c1 - c2)
    expect = float(np.mean(expect))
    assert expect < 0.95 * VS  # interpolation smooths the field measurably (~0.91 var_s)
    assert abs(sq / expect - 1.0) < 0.05, (sq, expect)


def test_grf_workload_data_variance():
    w = synth.small(24, 64, 16.0, seed=11)
    d, noise = w.pixels[:, 4], w.pixels[:, 3]
    assert np.all((noise >= 0.05) & (noise <= 0.3))
    # signal variance (trilinear-smoothed, ~0.91 var_s) plus mean(n^2)
    var_expect = 0.91 * VS + np.mean(noise**2)
    assert 0.7 * var_expect < np.var(d) < 1.3 * var_expect
