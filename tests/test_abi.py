"""CPU tests of the boundary: the C-ABI library builds for sm_103a, loads, and
exports every function that include/*.h declares; host-side helpers mirror
the reference's formats.  No compute call is made (no GPU here)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import dachshund_gb300 as ds
from dachshund_gb300 import _lib, api, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(ds_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    ds.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows every one of them
    assert names <= set(_lib.SIGNATURES), sorted(names - set(_lib.SIGNATURES))


def test_status_strings_and_table_without_gpu():
    lib = _lib.load()
    assert lib.ds_status_string(0) == b"ok"
    assert b"max iteration" in lib.ds_status_string(3)
    t, dx_inv = api.table_init()
    assert dx_inv == 24.875
    np.testing.assert_allclose(t, np.exp(-(8.0 / 199) * np.arange(200)), rtol=2e-16)


def test_context_fails_loudly_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(ds.DsError):
        ds.Context(0)


def test_pixel_conversions_match_reference_semantics():
    # tests/pixel_tests.cc:40-74 on the host-side converters
    rng = np.random.default_rng(0)
    pix = np.zeros((10, 5))
    pix[:, 3] = rng.uniform(0.01, 1, 10)
    pix[:, 4] = rng.standard_normal(10)
    npx = api.pixel_to_npixel(pix)
    np.testing.assert_array_equal(npx[:, 3], pix[:, 3] * pix[:, 3])
    np.testing.assert_array_equal(api.npixel_to_pixel(npx)[:, 3], pix[:, 3])
    wp = api.pixel_to_wpixel(pix)
    np.testing.assert_array_equal(wp[:, 3], 1.0 / pix[:, 3])
    np.testing.assert_array_equal(wp[:, 4], pix[:, 4] / pix[:, 3])
    back = api.wpixel_to_pixel(wp)
    np.testing.assert_allclose(back[:, 3:], pix[:, 3:], rtol=1e-15)


def test_map_coords_and_config_format(tmp_path):
    import oracle

    a = api.init_uniform_map_coords(3.0, 4.0, 5.0, 3, 4, 5)
    b = oracle.uniform_map_coords(3.0, 4.0, 5.0, 3, 4, 5)
    np.testing.assert_array_equal(a, b)
    w = synth.small(4, 8, 6.0, seed=0)
    cfg = w.write(str(tmp_path))
    text = open(cfg).read()
    assert "num_pixels = 32" in text and "corr_l_perp = 2.5" in text
    pix = api.read_pixel_data(str(tmp_path / "pixels.bin"), 32)
    np.testing.assert_array_equal(pix, w.pixels)
    with pytest.raises(ValueError):
        api.read_pixel_data(str(tmp_path / "pixels.bin"), 33)


def test_synth_workloads_deterministic_and_shaped():
    a, b = synth.wf32768(), synth.wf32768()
    np.testing.assert_array_equal(a.pixels, b.pixels)
    assert a.n == 32768 and a.n_map == 40 * 40 * 256
    p = a.pixels
    assert p[:, 3].min() >= 0.05 and p[:, 3].max() <= 0.3
    z = p[:128, 2]
    np.testing.assert_allclose(np.diff(z), 2.0)
    assert abs(np.std(p[:, 4]) - np.sqrt(0.0625 + np.mean(p[:, 3] ** 2))) < 0.05


def test_missing_library_raises_instead_of_falling_back(monkeypatch):
    # No CPU fallback: without the built CUDA library every entry point raises.
    from dachshund_gb300 import _lib as lib_mod

    monkeypatch.setattr(lib_mod, "_lib", None)
    monkeypatch.setattr(lib_mod, "LIB_PATH", os.path.join(ROOT, "no-such-dir", "libdsgb300.so"))
    with pytest.raises(RuntimeError, match="not built"):
        lib_mod.load(build_if_missing=False)
    with pytest.raises(OSError):
        lib_mod.load()  # builds the real library, then fails to open the missing path


def test_argument_checks_need_no_gpu():
    # Calls the ABI rejects before any CUDA call return DS_ERR_ARG, also on a
    # machine without a GPU: null handles, bad forms, sizes out of range.
    from dachshund_gb300 import _lib as L

    lib = L.load()
    vp = ctypes.c_void_p
    out = vp()
    kp = api.SignalCovarParams(0.0625, 2.5, 2.0, eval="exact").as_c()
    rec = np.zeros((8, 5))
    vec = np.zeros(8)
    p = rec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    v = vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert lib.ds_operator_create(None, L.DS_FORM_W, 8, p, ctypes.byref(kp),
                                  ctypes.byref(out)) == L.DS_ERR_ARG
    assert lib.ds_A_product(None, v, v) == L.DS_ERR_ARG
    assert lib.ds_A_residual(None, v, v) == L.DS_ERR_ARG
    assert lib.ds_map_create(None, 8, p, ctypes.byref(out)) == L.DS_ERR_ARG
    assert lib.ds_learned_create(None, ctypes.byref(kp), 128, 2, 0,
                                 ctypes.byref(out)) == L.DS_ERR_ARG
    sizes = (ctypes.c_int * 1)(8)
    assert lib.ds_batch_create(None, L.DS_FORM_W, 1, sizes, p, ctypes.byref(kp), 4, 0.0,
                               ctypes.byref(out)) == L.DS_ERR_ARG

    # The allocation-free PCG checks its arguments and its size limit (32,768
    # pixels, the fixed work space) before it touches the device.
    pp = L.PcgParamsC(100, 50, 1e-8, 0)
    res = L.PcgResultC()
    rp = vp(rec.ctypes.data)
    xp = vp(vec.ctypes.data)

    def noalloc(form, n, records=rp, x=xp, params=pp):
        return lib.ds_solve_pcg_noalloc(form, n, records, ctypes.byref(kp),
                                        ctypes.byref(params) if params is not None else None,
                                        x, ctypes.byref(res), None, None)

    assert noalloc(L.DS_FORM_W, 32769) == L.DS_ERR_ARG
    assert noalloc(L.DS_FORM_W, 0) == L.DS_ERR_ARG
    assert noalloc(7, 8) == L.DS_ERR_ARG
    assert noalloc(L.DS_FORM_W, 8, records=None) == L.DS_ERR_ARG
    assert noalloc(L.DS_FORM_W, 8, x=None) == L.DS_ERR_ARG
    assert noalloc(L.DS_FORM_W, 8, params=None) == L.DS_ERR_ARG
    assert noalloc(L.DS_FORM_W, 8, params=L.PcgParamsC(100, 0, 1e-8, 0)) == L.DS_ERR_ARG
