"""CPU tests: the oracle restatement against the reference's golden vectors,
and against the reference's own known-answer tests.

The golden vectors were produced by the unmodified reference
(tests/golden/make_golden.py).  Where the reference harness is built here
(oracle/_ref), the reference's own test cases (tests/*_tests.cc) are also
replayed on its fixture through both the port and the reference.
"""
import os

import numpy as np
import pytest

import oracle
from dachshund_gb300 import synth

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA
_REF_DIR = oracle.ref_source_dir()
# the reference's own test fixture (tests/small_pixel_data.bin in its tree)
REF_FIXTURE = os.path.join(_REF_DIR, "tests", "small_pixel_data.bin") if _REF_DIR else ""


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_table_matches_reference_ctor():
    # SignalCovarParams ctor, lib/signal_covar.h:19-41
    t, dx_inv, cp, cq = oracle.table(VS, LP, LQ)
    assert t.shape == (200,) and t[0] == 1.0
    assert dx_inv == 24.875
    np.testing.assert_allclose(t, np.exp(-(8.0 / 199) * np.arange(200)), rtol=2e-16, atol=0)
    if oracle.ref_available():
        tr, dxr, cpr, cqr = oracle.table(VS, LP, LQ, impl="ref")
        np.testing.assert_array_equal(t, tr)
        assert (dx_inv, cp, cq) == (dxr, cpr, cqr)


def test_signal_covar_probes(golden):
    e = golden["edge"]
    s = oracle.signal_covar(e["probe_perp2"], e["probe_para2"], VS, LP, LQ)
    np.testing.assert_array_equal(s, e["probe_S"])  # bit-exact, incl. the cutoff
    s = oracle.signal_covar(e["probe_perp2"], e["probe_para2"], VS, LP, LQ, exact=True)
    np.testing.assert_allclose(s, e["probe_S_exact"], rtol=1e-15)


@pytest.mark.parametrize("form", ["sn", "w"])
def test_operator_golden(golden, form):
    g = golden["small"]
    pix = g["pixels"]
    rec = oracle.pixel_to_npixel(pix) if form == "sn" else oracle.pixel_to_wpixel(pix)
    # Same loops in the same order as the reference: bit-exact.
    np.testing.assert_array_equal(oracle.A_product(form, rec, g["a"], VS, LP, LQ), g[f"Aa_{form}"])
    np.testing.assert_array_equal(oracle.A_residual(form, rec, g["a"], VS, LP, LQ), g[f"r_{form}"])


@pytest.mark.parametrize("form", ["sn", "w"])
def test_pcg_golden(golden, form):
    g = golden["small"]
    pix = g["pixels"]
    rec = oracle.pixel_to_npixel(pix) if form == "sn" else oracle.pixel_to_wpixel(pix)
    x, ok, it, hist = oracle.solve_pcg(form, rec, VS, LP, LQ, 1000, 50, 1e-8)
    assert ok and it == int(g[f"iters_{form}"])
    np.testing.assert_array_equal(x, g[f"x_{form}"])
    np.testing.assert_array_equal(hist, g[f"hist_{form}"])


def test_map_products_golden(golden):
    g = golden["small"]
    pix = g["pixels"]
    m = oracle.smp_product(pix[:, :3], g["map_pts"], g["x_w"], VS, LP, LQ)
    np.testing.assert_array_equal(m, g["map"])
    s = oracle.sigma_m_noise_dom(oracle.pixel_to_npixel(pix), g["map_pts"], VS, LP, LQ)
    np.testing.assert_array_equal(s, g["sigma_nd"])


def test_map_covar_diag_golden(golden):
    g = golden["small"]
    s, iters, ok = oracle.map_covar_diag(oracle.pixel_to_npixel(g["pixels"]), g["cov_pts"], VS, LP,
                                         LQ, 1000, 50, 1e-6)
    np.testing.assert_array_equal(iters, g["cov_iters"])
    np.testing.assert_array_equal(s, g["cov"])


@pytest.mark.parametrize("case", ["n1", "n7", "coinc"])
@pytest.mark.parametrize("form", ["sn", "w"])
def test_edge_golden(golden, case, form):
    e = golden["edge"]
    pix = e[f"{case}_pixels"]
    rec = oracle.pixel_to_npixel(pix) if form == "sn" else oracle.pixel_to_wpixel(pix)
    np.testing.assert_array_equal(oracle.A_product(form, rec, e[f"{case}_a"], VS, LP, LQ),
                                  e[f"{case}_Aa_{form}"])
    x, ok, it, _ = oracle.solve_pcg(form, rec, VS, LP, LQ, 100, 50, 1e-10)
    assert it == int(e[f"{case}_iters_{form}"]) and int(ok) == int(e[f"{case}_ok_{form}"])
    np.testing.assert_array_equal(x, e[f"{case}_x_{form}"])


def test_wf4096_app_golden(golden):
    """The reference app's map on the 4,096-pixel workload: W-form PCG
    (tol 1e-5) then smp_product, restated by the port."""
    g = golden["wf4096"]
    pix = g["pixels"]
    lx, ly, lz, nx, ny, nz, tol, max_iter, step_r = g["params"]
    wrec = oracle.pixel_to_wpixel(pix)
    x, ok, it, hist = oracle.solve_pcg("w", wrec, VS, LP, LQ, int(max_iter), int(step_r), tol)
    assert ok and it == int(g["num_iters"])
    np.testing.assert_array_equal(x, g["x"])
    mp = oracle.uniform_map_coords(lx, ly, lz, int(nx), int(ny), int(nz))
    m = oracle.smp_product(pix[:, :3], mp, x, VS, LP, LQ)
    assert rel(m, g["map"]) < 1e-13


def test_cf_matches_pcg_port():
    w = synth.small(6, 16, 8.0, seed=1)
    rec = oracle.pixel_to_wpixel(w.pixels)
    xcf = oracle.solve_cf("w", rec, VS, LP, LQ)
    xpcg, ok, _, _ = oracle.solve_pcg("w", rec, VS, LP, LQ, 500, 50, 1e-12)
    assert ok and rel(xpcg, xcf) < 1e-9


# ---- the reference's own known-answer tests, replayed on its fixture -------

needs_ref = pytest.mark.skipif(not (oracle.ref_available() and os.path.exists(REF_FIXTURE)),
                               reason="reference sources/harness not available")


@needs_ref
def test_ref_fixture_operator_and_pcg_port_vs_reference():
    pix = np.fromfile(REF_FIXTURE).reshape(-1, 5)
    a = np.random.default_rng(0).standard_normal(pix.shape[0])
    for form, rec in (("sn", oracle.pixel_to_npixel(pix)), ("w", oracle.pixel_to_wpixel(pix))):
        # wfx_tests.cc:123-151 settings (var_s 0.05, l 1, tol 1e-4, step_r 10)
        np.testing.assert_array_equal(oracle.A_product(form, rec, a, 0.05, 1.0, 1.0),
                                      oracle.A_product(form, rec, a, 0.05, 1.0, 1.0, impl="ref"))
        p = oracle.solve_pcg(form, rec, 0.05, 1.0, 1.0, 1000, 10, 1e-4)
        r = oracle.solve_pcg(form, rec, 0.05, 1.0, 1.0, 1000, 10, 1e-4, impl="ref")
        assert p[2] == r[2]
        np.testing.assert_array_equal(p[0], r[0])


@needs_ref
def test_ref_known_answers_on_port():
    """tests/signal_covar_tests.cc and tests/wfx_tests.cc assertions, on the port."""
    # S_lookup_vs_exact_1d (signal_covar_tests.cc:12-29): table within 1e-3.
    l = 0.5
    x = np.arange(0.0, 4.0 * l, 0.03 * l)
    sf = oracle.signal_covar(x * x, np.zeros_like(x), 1.0, l, l)
    se = np.exp(-(x * x) / 2.0 / (l * l))
    assert np.all(np.abs(se - sf) <= 1e-3 * np.abs(se))
    # S_lookup_table_cutoff (signal_covar_tests.cc:65-80)
    for l in (0.3, 0.77, 1.9):
        assert oracle.signal_covar([(3.99 * l) ** 2], [0.0], 1.0, l, l)[0] > 0.0
        assert oracle.signal_covar([(4.01 * l) ** 2], [0.0], 1.0, l, l)[0] == 0.0
    pix = np.fromfile(REF_FIXTURE).reshape(-1, 5)
    nrec, wrec = oracle.pixel_to_npixel(pix), oracle.pixel_to_wpixel(pix)
    # different_x_expressions (wfx_tests.cc:49-64): SN vs W closed form, exact S.
    xsn = oracle.solve_cf("sn", nrec, 0.05, 1.0, 1.0, exact=True)
    xw = oracle.solve_cf("w", wrec, 0.05, 1.0, 1.0, exact=True)
    assert np.all(np.abs(xsn - xw) <= 1e-8 * np.abs(xsn))
    # PCG_lookup_S_vs_CF_exact_S (wfx_tests.cc:123-151): rms(x_pcg/x_cf - 1) < 0.01
    xcf = oracle.solve_cf("w", wrec, 0.05, 1.0, 1.0)
    xp, _, _, _ = oracle.solve_pcg("w", wrec, 0.05, 1.0, 1.0, 1000, 10, 1e-4)
    assert np.sqrt(np.mean((xp / xcf - 1.0) ** 2)) < 0.01


@needs_ref
def test_golden_fixtures_reproduce_from_their_script(tmp_path):
    """tests/golden/make_golden.py, run again on the reference, writes the
    committed fixtures bit for bit (in a child process: the reference's
    MapCovarDiag prints progress lines from C)."""
    import subprocess
    import sys

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    r = subprocess.run([sys.executable, os.path.join(here, "make_golden.py"), "--out",
                        str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    for name in ("edge", "small", "wf4096"):
        old = np.load(os.path.join(here, name + ".npz"))
        new = np.load(tmp_path / (name + ".npz"))
        assert set(old.files) == set(new.files), name
        for k in old.files:
            np.testing.assert_array_equal(new[k], old[k], err_msg=f"{name}:{k}")
