"""Drop-in checks of the C++ layer (dachshund_gb300/lib): the reference's own
application and test sources compile and link unchanged against it (CPU,
where the reference sources exist), and a C++ driver of the app path runs on
the GPU against the reference's golden map."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "dachshund_gb300")
import oracle  # noqa: E402  (only for the location of the reference sources)

REF = oracle.ref_source_dir() or ""
CXX = ["g++", "-std=c++11", "-O1", "-I" + os.path.join(LIBDIR, "lib"),
       "-I" + os.path.join(ROOT, "include")]
LINK = ["-L" + LIBDIR, "-ldachshund_gb300", "-ldsgb300", "-Wl,-rpath," + LIBDIR, "-lpthread"]

needs_ref = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "app"))),
                               reason="reference sources not present")


def _build_lib():
    import dachshund_gb300

    dachshund_gb300.build()


@needs_ref
def test_reference_app_builds_unchanged(tmp_path):
    _build_lib()
    out = tmp_path / "dachshund.exe"
    r = subprocess.run(CXX + [os.path.join(REF, "app", "dachshund.cc"), "-o", str(out)] + LINK,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert out.exists()


@needs_ref
def test_reference_test_suite_builds_unchanged(tmp_path):
    _build_lib()
    srcs = sorted(os.path.join(REF, "tests", f) for f in os.listdir(os.path.join(REF, "tests"))
                  if f.endswith(".cc"))
    inc = ["-I" + os.path.join(REF, "ext"), "-I" + os.path.join(REF, "ext", "gtest"),
           "-I" + os.path.join(REF, "ext", "gtest", "include"), "-I" + os.path.join(REF, "tests")]
    out = tmp_path / "run_tests.exe"
    r = subprocess.run(CXX + inc + srcs + ["-o", str(out)] + LINK, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
def test_cxx_app_path_on_gpu(tmp_path, golden):
    """tests/cpp/wf_app.cc through the C++ layer: the 4,096-pixel workload at
    the reference's iteration count, map within 1e-8 of the reference app's
    map.bin; the closed-form solve within 1e-6 of the PCG solution (tol 1e-5)."""
    _build_lib()
    g = golden["wf4096"]
    pix = g["pixels"]
    lx, ly, lz, nx, ny, nz, tol, max_iter, step_r = g["params"]
    exe = tmp_path / "wf_app"
    r = subprocess.run(CXX + [os.path.join(ROOT, "tests", "cpp", "wf_app.cc"), "-o", str(exe)]
                       + LINK, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pix_path = tmp_path / "pixels.bin"
    np.ascontiguousarray(pix).tofile(pix_path)
    prefix = str(tmp_path / "out")
    args = [str(exe), str(pix_path), str(pix.shape[0]), repr(float(lx)), repr(float(ly)),
            repr(float(lz)),
            str(int(nx)), str(int(ny)), str(int(nz)), repr(float(tol)), str(int(max_iter)),
            str(int(step_r)), prefix]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    it = int(r.stdout.split()[1])
    assert it == int(g["num_iters"]) and r.stdout.split()[3] == "1"
    m = np.fromfile(prefix + ".map")
    assert np.max(np.abs(m - g["map"])) / np.max(np.abs(g["map"])) < 1e-8
    x = np.fromfile(prefix + ".x")
    xcf = np.fromfile(prefix + ".xcf")
    # PCG stopped at |r| <= 1e-5 |b|; the closed form is exact.
    assert np.max(np.abs(x - xcf)) / np.max(np.abs(xcf)) < 1e-3
