"""TEST INFRASTRUCTURE -- the CPU oracle for the Wiener-filter path.

Two oracle libraries behind one numpy interface:

* ``impl="port"``: ``oracle/libdsoracle.so``, the C restatement in
  ``oracle/ds_oracle.c`` (built by ``make -C oracle port``; builds on any host);
* ``impl="ref"``: ``oracle/_ref/libdsref.so``, the unmodified reference
  library compiled from its own sources by ``make -C oracle ref`` (only where
  the reference sources are present).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this package.  The product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libdsoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdsref.so")
REF_EXE = os.path.join(HERE, "_ref", "dachshund.exe")

TABLE_N = 200

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class _DsoKernel(C.Structure):
    _fields_ = [
        ("var_s", C.c_double),
        ("c_perp", C.c_double),
        ("c_para", C.c_double),
        ("dx_inv", C.c_double),
        ("table", C.c_double * TABLE_N),
        ("exact", C.c_int),
    ]


def build(ref_dir: str | None = None, quiet: bool = True) -> None:
    """Build the port (always) and, given the reference source tree
    (``ref_dir``, else the REF environment variable), the reference harness."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE, "port"], stdout=out)
    ref_dir = ref_dir or os.environ.get("REF")
    if ref_dir and os.path.isdir(os.path.join(ref_dir, "lib")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF=" + ref_dir], stdout=out)


def ref_source_dir() -> str | None:
    """The reference source tree the harness in oracle/_ref was built from
    (recorded by ``make ref``), or the REF environment variable; None when
    neither names an existing tree."""
    cands = [os.environ.get("REF")]
    try:
        with open(os.path.join(HERE, "_ref", "source_dir")) as f:
            cands.insert(0, f.read().strip())
    except OSError:
        pass
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "lib")):
            return c
    return None


_port = None
_ref = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build()
        lib = C.CDLL(PORT_SO)
        K = C.POINTER(_DsoKernel)
        lib.dso_kernel_init.argtypes = [K, C.c_double, C.c_double, C.c_double, C.c_int]
        lib.dso_signal_covar.argtypes = [K, C.c_double, C.c_double]
        lib.dso_signal_covar.restype = C.c_double
        for name in ("dso_A_product", "dso_A_residual", "dso_precond"):
            getattr(lib, name).argtypes = [K, C.c_int, C.c_int, _dp, _dp, _dp]
        lib.dso_A_product_rows.argtypes = [K, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int, C.c_int]
        lib.dso_smp_product_rows.argtypes = [K, C.c_int, _dp, _dp, _dp, _dp, C.c_int, C.c_int]
        lib.dso_norm_b.argtypes = [C.c_int, C.c_int, _dp]
        lib.dso_norm_b.restype = C.c_double
        lib.dso_solve_pcg.argtypes = [K, C.c_int, C.c_int, _dp, C.c_int, C.c_int,
                                      C.c_double, _dp, C.POINTER(C.c_int), _dp,
                                      C.c_int, C.POINTER(C.c_int)]
        lib.dso_solve_pcg.restype = C.c_int
        lib.dso_solve_cf.argtypes = [K, C.c_int, C.c_int, _dp, _dp]
        lib.dso_solve_cf.restype = C.c_int
        lib.dso_smp_product.argtypes = [K, C.c_int, _dp, C.c_int, _dp, _dp, _dp]
        lib.dso_sigma_m_noise_dom.argtypes = [K, C.c_int, _dp, C.c_int, _dp, _dp]
        lib.dso_map_covar_diag.argtypes = [K, C.c_int, _dp, C.c_int, _dp, C.c_int,
                                           C.c_int, C.c_double, _dp, _ip, _ip]
        lib.dso_init_uniform_map_coords.argtypes = [C.c_double] * 3 + [C.c_int] * 3 + [_dp]
        lib.dso_pixel_to_wpixel.argtypes = [C.c_int, _dp]
        lib.dso_pixel_to_npixel.argtypes = [C.c_int, _dp]
        _port = lib
    return _port


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference harness not built (make -C oracle ref)")
        lib = C.CDLL(REF_SO)
        d, i = C.c_double, C.c_int
        lib.dsref_table.argtypes = [d, d, d, _dp, C.POINTER(d), C.POINTER(d), C.POINTER(d)]
        lib.dsref_signal_covar.argtypes = [d, d, d, i, _dp, _dp, i, _dp]
        lib.dsref_A_product.argtypes = [i, i, _dp, d, d, d, _dp, _dp]
        lib.dsref_A_residual.argtypes = [i, i, _dp, d, d, d, _dp, _dp]
        lib.dsref_A_entries.argtypes = [i, i, _dp, d, d, d, i, i, _ip, _ip, _dp]
        lib.dsref_solve_pcg.argtypes = [i, i, _dp, d, d, d, i, i, d, _dp,
                                        C.POINTER(i), _dp, i, C.POINTER(i)]
        lib.dsref_solve_pcg.restype = i
        lib.dsref_solve_cf.argtypes = [i, i, _dp, d, d, d, i, _dp]
        lib.dsref_smp_product.argtypes = [i, _dp, i, _dp, d, d, d, _dp, _dp]
        lib.dsref_sigma_m_noise_dom.argtypes = [i, _dp, i, _dp, d, d, d, _dp]
        lib.dsref_map_covar_diag.argtypes = [i, _dp, i, _dp, d, d, d, i, i, d,
                                             _dp, _ip, _ip]
        lib.dsref_init_uniform_map_coords.argtypes = [d, d, d, i, i, i, _dp]
        _ref = lib
    return _ref


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _kernel(var_s, l_perp, l_para, exact):
    k = _DsoKernel()
    port_lib().dso_kernel_init(C.byref(k), var_s, l_perp, l_para, int(bool(exact)))
    return k


FORMS = {"sn": 0, "w": 1}


def _form(form):
    return FORMS[form] if isinstance(form, str) else int(form)


# --------------------------------------------------------------------------
# numpy-facing oracle calls.  ``rec`` is an (n, 5) float64 array of NPixel
# (form "sn") or WPixel (form "w") records; ``pts`` is (m, 3).
# --------------------------------------------------------------------------

def table(var_s, l_perp, l_para, impl="port"):
    if impl == "ref":
        t = np.zeros(TABLE_N)
        dx_inv, cp, cq = C.c_double(), C.c_double(), C.c_double()
        ref_lib().dsref_table(var_s, l_perp, l_para, t, C.byref(dx_inv), C.byref(cp), C.byref(cq))
        return t, dx_inv.value, cp.value, cq.value
    k = _kernel(var_s, l_perp, l_para, False)
    return np.array(k.table[:]), k.dx_inv, k.c_perp, k.c_para


def signal_covar(perp2, para2, var_s, l_perp, l_para, exact=False, impl="port"):
    perp2 = _c(perp2).ravel()
    para2 = _c(para2).ravel()
    out = np.empty_like(perp2)
    if impl == "ref":
        ref_lib().dsref_signal_covar(var_s, l_perp, l_para, perp2.size, perp2, para2,
                                     int(bool(exact)), out)
        return out
    k = _kernel(var_s, l_perp, l_para, exact)
    lib = port_lib()
    for i in range(perp2.size):
        out[i] = lib.dso_signal_covar(C.byref(k), perp2[i], para2[i])
    return out


def A_product(form, rec, a, var_s, l_perp, l_para, exact=False, impl="port"):
    rec, a = _c(rec), _c(a)
    n = rec.shape[0]
    b = np.empty(n)
    if impl == "ref":
        assert not exact, "the reference operator is table-only"
        ref_lib().dsref_A_product(_form(form), n, rec, var_s, l_perp, l_para, a, b)
    else:
        k = _kernel(var_s, l_perp, l_para, exact)
        port_lib().dso_A_product(C.byref(k), _form(form), n, rec, a, b)
    return b


def A_product_rows(form, rec, a, row0, row1, var_s, l_perp, l_para, exact=False):
    """Rows [row0, row1) of A a (the port), for bounded CPU-baseline samples."""
    rec, a = _c(rec), _c(a)
    b = np.empty(row1 - row0)
    k = _kernel(var_s, l_perp, l_para, exact)
    port_lib().dso_A_product_rows(C.byref(k), _form(form), rec.shape[0], rec, a, b, row0, row1)
    return b


def smp_product_rows(pix_pts, map_pts, x, row0, row1, var_s, l_perp, l_para, exact=False):
    pix_pts, map_pts, x = _c(pix_pts), _c(map_pts), _c(x)
    m = np.empty(row1 - row0)
    k = _kernel(var_s, l_perp, l_para, exact)
    port_lib().dso_smp_product_rows(C.byref(k), pix_pts.shape[0], pix_pts, map_pts, x, m,
                                    row0, row1)
    return m


def A_residual(form, rec, x, var_s, l_perp, l_para, exact=False, impl="port"):
    rec, x = _c(rec), _c(x)
    n = rec.shape[0]
    r = np.empty(n)
    if impl == "ref":
        assert not exact, "the reference operator is table-only"
        ref_lib().dsref_A_residual(_form(form), n, rec, var_s, l_perp, l_para, x, r)
    else:
        k = _kernel(var_s, l_perp, l_para, exact)
        port_lib().dso_A_residual(C.byref(k), _form(form), n, rec, x, r)
    return r


def A_entries(form, rec, ii, jj, var_s, l_perp, l_para, exact=False):
    rec = _c(rec)
    ii, jj = _c(ii, np.int32), _c(jj, np.int32)
    out = np.empty(ii.size)
    ref_lib().dsref_A_entries(_form(form), rec.shape[0], rec, var_s, l_perp, l_para,
                              int(bool(exact)), ii.size, ii, jj, out)
    return out


def solve_pcg(form, rec, var_s, l_perp, l_para, max_iter, step_r, tol, x0=None,
              exact=False, impl="port"):
    """Returns (x, success, num_iters, residual_norms)."""
    rec = _c(rec)
    n = rec.shape[0]
    x = np.zeros(n) if x0 is None else _c(x0).copy()
    hist = np.zeros(max(max_iter, 1) + 1)
    it, nh = C.c_int(0), C.c_int(0)
    if impl == "ref":
        assert not exact
        ok = ref_lib().dsref_solve_pcg(_form(form), n, rec, var_s, l_perp, l_para, max_iter,
                                       step_r, tol, x, C.byref(it), hist, hist.size, C.byref(nh))
    else:
        k = _kernel(var_s, l_perp, l_para, exact)
        ok = port_lib().dso_solve_pcg(C.byref(k), _form(form), n, rec, max_iter, step_r, tol,
                                      x, C.byref(it), hist, hist.size, C.byref(nh))
    return x, bool(ok), it.value, hist[: nh.value].copy()


def solve_cf(form, rec, var_s, l_perp, l_para, exact=False, impl="port"):
    rec = _c(rec)
    n = rec.shape[0]
    x = np.zeros(n)
    if impl == "ref":
        ref_lib().dsref_solve_cf(_form(form), n, rec, var_s, l_perp, l_para, int(bool(exact)), x)
    else:
        k = _kernel(var_s, l_perp, l_para, exact)
        if not port_lib().dso_solve_cf(C.byref(k), _form(form), n, rec, x):
            raise RuntimeError("LDL^T breakdown: matrix not positive definite")
    return x


def smp_product(pix_pts, map_pts, x, var_s, l_perp, l_para, exact=False, impl="port"):
    pix_pts, map_pts, x = _c(pix_pts), _c(map_pts), _c(x)
    m = np.empty(map_pts.shape[0])
    if impl == "ref":
        assert not exact
        ref_lib().dsref_smp_product(pix_pts.shape[0], pix_pts, map_pts.shape[0], map_pts,
                                    var_s, l_perp, l_para, x, m)
    else:
        k = _kernel(var_s, l_perp, l_para, exact)
        port_lib().dso_smp_product(C.byref(k), pix_pts.shape[0], pix_pts, map_pts.shape[0],
                                   map_pts, x, m)
    return m


def sigma_m_noise_dom(nrec, map_pts, var_s, l_perp, l_para, exact=False, impl="port"):
    nrec, map_pts = _c(nrec), _c(map_pts)
    out = np.empty(map_pts.shape[0])
    if impl == "ref":
        ref_lib().dsref_sigma_m_noise_dom(nrec.shape[0], nrec, map_pts.shape[0], map_pts,
                                          var_s, l_perp, l_para, out)
    else:
        k = _kernel(var_s, l_perp, l_para, exact)
        port_lib().dso_sigma_m_noise_dom(C.byref(k), nrec.shape[0], nrec, map_pts.shape[0],
                                         map_pts, out)
    return out


def map_covar_diag(nrec, map_pts, var_s, l_perp, l_para, max_iter, step_r, tol,
                   exact=False, impl="port"):
    """Returns (sigma_m, iters, success)."""
    nrec, map_pts = _c(nrec), _c(map_pts)
    m = map_pts.shape[0]
    out = np.zeros(m)
    iters = np.zeros(m, np.int32)
    succ = np.zeros(m, np.int32)
    if impl == "ref":
        ref_lib().dsref_map_covar_diag(nrec.shape[0], nrec, m, map_pts, var_s, l_perp, l_para,
                                       max_iter, step_r, tol, out, iters, succ)
    else:
        k = _kernel(var_s, l_perp, l_para, exact)
        port_lib().dso_map_covar_diag(C.byref(k), nrec.shape[0], nrec, m, map_pts, max_iter,
                                      step_r, tol, out, iters, succ)
    return out, iters, succ.astype(bool)


def uniform_map_coords(lx, ly, lz, nx, ny, nz, impl="port"):
    out = np.empty((nx * ny * nz, 3))
    if impl == "ref":
        ref_lib().dsref_init_uniform_map_coords(lx, ly, lz, nx, ny, nz, out)
    else:
        port_lib().dso_init_uniform_map_coords(lx, ly, lz, nx, ny, nz, out)
    return out


def pixel_to_wpixel(pix):
    rec = _c(pix).copy()
    port_lib().dso_pixel_to_wpixel(rec.shape[0], rec)
    return rec


def pixel_to_npixel(pix):
    rec = _c(pix).copy()
    port_lib().dso_pixel_to_npixel(rec.shape[0], rec)
    return rec
