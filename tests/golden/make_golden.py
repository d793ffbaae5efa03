"""Generates the golden vectors under tests/golden/ by running the UNMODIFIED
reference (oracle/_ref, compiled from the reference's own sources by
``make -C oracle ref``) on seeded synthetic inputs.

The reference commits no golden outputs of its own; these fixtures pin both
the oracle restatement (CPU tests) and the CUDA path (GPU tests).

    python tests/golden/make_golden.py [--out DIR]   (default: this folder)

Outputs (all float64 unless noted):
  wf4096.npz   4,096-pixel workload: pixels, the reference app's map.bin,
                its iteration count (parsed from the app's trace), the W-form
                PCG solution x and residual history from the harness.
  small.npz     512-pixel GRF workload: A_product / A_residual in both forms,
                A(i, j) entries (table and exact), PCG solutions and
                histories (both forms), smp_product on a small grid,
                sigma_m_noise_dom, MapCovarDiag on a few map points.
  edge.npz      tiny and boundary cases: n = 1, n = 7, pixels exactly on the
                table cutoff, coincident pixels.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = HERE  # where the .npz files are written
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from dachshund_gb300 import synth  # noqa: E402

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA


def run_app(w: synth.Workload):
    with tempfile.TemporaryDirectory() as d:
        cfg = w.write(d)
        out = subprocess.run([oracle.REF_EXE, cfg], capture_output=True, text=True, check=True,
                             env=dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count())))
        m = np.fromfile(os.path.join(d, "map.bin"), dtype=np.float64)
    it = re.search(r"iter (\d+) reached", out.stdout)
    return m, (int(it.group(1)) if it else -1)


def make_wf4096():
    w = synth.wf4096()
    m, iters = run_app(w)
    wrec = oracle.pixel_to_wpixel(w.pixels)
    x, ok, it2, hist = oracle.solve_pcg("w", wrec, VS, LP, LQ, w.pcg_max_iter, w.pcg_step_r,
                                        w.pcg_tol, impl="ref")
    assert ok and it2 == iters, (ok, it2, iters)
    np.savez_compressed(os.path.join(OUT, "wf4096.npz"), pixels=w.pixels, map=m,
                        num_iters=iters, x=x, hist=hist,
                        params=np.array([w.lx, w.ly, w.lz, w.map_nx, w.map_ny, w.map_nz,
                                         w.pcg_tol, w.pcg_max_iter, w.pcg_step_r]))


def make_small():
    w = synth.small(16, 32, 12.0, seed=3)
    rng = np.random.default_rng(7)
    pix = w.pixels
    n = w.n
    nrec, wrec = oracle.pixel_to_npixel(pix), oracle.pixel_to_wpixel(pix)
    a = rng.standard_normal(n)
    out = dict(pixels=pix, a=a)
    for form, rec in (("sn", nrec), ("w", wrec)):
        out[f"Aa_{form}"] = oracle.A_product(form, rec, a, VS, LP, LQ, impl="ref")
        out[f"r_{form}"] = oracle.A_residual(form, rec, a, VS, LP, LQ, impl="ref")
        x, ok, it, hist = oracle.solve_pcg(form, rec, VS, LP, LQ, 1000, 50, 1e-8, impl="ref")
        assert ok
        out[f"x_{form}"], out[f"iters_{form}"], out[f"hist_{form}"] = x, it, hist
        x, ok, it, hist = oracle.solve_pcg(form, rec, VS, LP, LQ, 1000, 10, 1e-4, impl="ref")
        out[f"x4_{form}"], out[f"iters4_{form}"], out[f"hist4_{form}"] = x, it, hist
    ii = rng.integers(0, n, 4000).astype(np.int32)
    jj = rng.integers(0, n, 4000).astype(np.int32)
    ii[:64] = jj[:64]  # diagonal entries
    out["ii"], out["jj"] = ii, jj
    for form, rec in (("sn", nrec), ("w", wrec)):
        out[f"Aij_table_{form}"] = oracle.A_entries(form, rec, ii, jj, VS, LP, LQ, exact=False)
        out[f"Aij_exact_{form}"] = oracle.A_entries(form, rec, ii, jj, VS, LP, LQ, exact=True)
    mp = oracle.uniform_map_coords(12.0, 12.0, 64.0, 6, 6, 32, impl="ref")
    out["map_pts"] = mp
    out["map"] = oracle.smp_product(pix[:, :3], mp, out["x_w"], VS, LP, LQ, impl="ref")
    out["sigma_nd"] = oracle.sigma_m_noise_dom(nrec, mp, VS, LP, LQ, impl="ref")
    cov_pts = mp[::397][:6].copy()
    s, iters, succ = oracle.map_covar_diag(nrec, cov_pts, VS, LP, LQ, 1000, 50, 1e-6, impl="ref")
    out["cov_pts"], out["cov"], out["cov_iters"], out["cov_success"] = cov_pts, s, iters, succ
    np.savez_compressed(os.path.join(OUT, "small.npz"), **out)


def make_edge():
    out = {}
    # n = 1
    p1 = np.array([[1.0, 2.0, 3.0, 0.1, 0.5]])
    # n = 7, one skewer with pixels 2 Mpc/h apart: pairs 8 Mpc/h apart sit
    # exactly on the table cutoff (xx = 199.0).
    p7 = np.zeros((7, 5))
    p7[:, 0], p7[:, 1] = 3.0, 4.0
    p7[:, 2] = (np.arange(7) + 0.5) * 2.0
    p7[:, 3] = np.linspace(0.05, 0.3, 7)
    p7[:, 4] = np.linspace(-0.5, 0.7, 7)
    # coincident pixels + a far-away pixel (decoupled)
    pc = np.array([[5.0, 5.0, 5.0, 0.2, 0.3], [5.0, 5.0, 5.0, 0.1, -0.2],
                   [5.5, 5.0, 6.0, 0.15, 0.1], [500.0, 500.0, 500.0, 0.2, 0.4]])
    rng = np.random.default_rng(11)
    for name, pix in (("n1", p1), ("n7", p7), ("coinc", pc)):
        n = pix.shape[0]
        a = rng.standard_normal(n)
        out[f"{name}_pixels"], out[f"{name}_a"] = pix, a
        for form, rec in (("sn", oracle.pixel_to_npixel(pix)), ("w", oracle.pixel_to_wpixel(pix))):
            out[f"{name}_Aa_{form}"] = oracle.A_product(form, rec, a, VS, LP, LQ, impl="ref")
            x, ok, it, hist = oracle.solve_pcg(form, rec, VS, LP, LQ, 100, 50, 1e-10, impl="ref")
            out[f"{name}_x_{form}"], out[f"{name}_iters_{form}"] = x, it
            out[f"{name}_ok_{form}"] = int(ok)
    # cutoff probes for signal_covar: x_para^2 with exact-boundary values
    para2 = np.array([0.0, 4.0, 16.0, 36.0, 63.999999, 64.0, 64.000001, 100.0])
    perp2 = np.zeros_like(para2)
    out["probe_perp2"], out["probe_para2"] = perp2, para2
    out["probe_S"] = oracle.signal_covar(perp2, para2, VS, LP, LQ, exact=False, impl="ref")
    out["probe_S_exact"] = oracle.signal_covar(perp2, para2, VS, LP, LQ, exact=True, impl="ref")
    np.savez_compressed(os.path.join(OUT, "edge.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) == 3 and sys.argv[1] == "--out":
        OUT = sys.argv[2]
    elif len(sys.argv) != 1:
        sys.exit("usage: make_golden.py [--out DIR]")
    oracle.build(oracle.ref_source_dir())
    if not oracle.ref_available():
        sys.exit("reference harness unavailable: build oracle/_ref first "
                 "(make -C oracle ref REF=<reference source tree>)")
    make_edge()
    make_small()
    make_wf4096()
    print("golden vectors written to", OUT)
