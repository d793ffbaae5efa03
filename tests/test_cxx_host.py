"""Host-side parts of the C++ layer (dachshund_gb300/lib), run without a GPU:
record reading with its error exits, the in-place record conversions and the
map grid, against the reference's semantics (lib/util.cc:11-46,
lib/pixel.cc:9-71) restated in numpy.  tests/cpp/io_check.cc is the driver."""
import os
import subprocess

import numpy as np
import pytest

from dachshund_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "dachshund_gb300")
CXX = ["g++", "-std=c++11", "-O1", "-I" + os.path.join(LIBDIR, "lib"),
       "-I" + os.path.join(ROOT, "include")]
LINK = ["-L" + LIBDIR, "-ldachshund_gb300", "-ldsgb300", "-Wl,-rpath," + LIBDIR, "-lpthread"]


@pytest.fixture(scope="module")
def io_check(tmp_path_factory):
    import dachshund_gb300

    dachshund_gb300.build()
    exe = tmp_path_factory.mktemp("cxx") / "io_check"
    r = subprocess.run(CXX + [os.path.join(ROOT, "tests", "cpp", "io_check.cc"), "-o", str(exe)]
                       + LINK, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return str(exe)


def _run(exe, path, n, grid=(2, 3, 4)):
    return subprocess.run([exe, str(path), str(n)] + [str(g) for g in grid],
                          capture_output=True, text=True, timeout=60)


def _rows(out, tag):
    return np.array([[float(v) for v in ln.split()[1:]] for ln in out.splitlines()
                     if ln.startswith(tag + " ")])


def test_records_conversions_and_grid(io_check, tmp_path):
    w = synth.small(4, 8, 6.0, seed=3)
    pix = w.pixels
    path = tmp_path / "pixels.bin"
    pix.astype("<f8").tofile(path)
    r = _run(io_check, path, len(pix))
    assert r.returncode == 0, r.stdout[-500:] + r.stderr[-500:]

    np.testing.assert_array_equal(_rows(r.stdout, "P"), pix)
    np.testing.assert_array_equal(_rows(r.stdout, "Q"), pix[:, :3])

    npx = pix.copy()
    npx[:, 3] = pix[:, 3] * pix[:, 3]
    np.testing.assert_array_equal(_rows(r.stdout, "N"), npx)

    # after Pixel -> NPixel -> Pixel, n = sqrt(n * n)
    p1 = npx.copy()
    p1[:, 3] = np.sqrt(npx[:, 3])
    wp = p1.copy()
    wp[:, 3] = 1.0 / p1[:, 3]
    wp[:, 4] = p1[:, 4] / p1[:, 3]
    np.testing.assert_array_equal(_rows(r.stdout, "W"), wp)

    back = wp.copy()
    back[:, 3] = 1.0 / wp[:, 3]
    back[:, 4] = wp[:, 4] / wp[:, 3]
    np.testing.assert_array_equal(_rows(r.stdout, "R"), back)
    np.testing.assert_allclose(back, pix, rtol=1e-15)

    nx, ny, nz = 2, 3, 4
    np.testing.assert_array_equal(_rows(r.stdout, "G"),
                                  synth.uniform_map_coords(1.0 * nx, 2.0 * ny, 0.5 * nz,
                                                           nx, ny, nz))


def test_short_file_exits_with_message(io_check, tmp_path):
    pix = synth.small(2, 8, 4.0, seed=1).pixels
    path = tmp_path / "short.bin"
    pix.astype("<f8").tofile(path)
    r = _run(io_check, path, len(pix) + 1)
    assert r.returncode == 1
    assert f"holds {len(pix)} pixel records, expected {len(pix) + 1}" in r.stdout
    assert not any(ln.startswith("P ") for ln in r.stdout.splitlines())


def test_missing_file_exits_with_message(io_check, tmp_path):
    r = _run(io_check, tmp_path / "absent.bin", 4)
    assert r.returncode == 1
    assert "Could not open file" in r.stdout
