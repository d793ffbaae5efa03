"""Python face of the C ABI, mirroring the reference library's interface.

Names follow the reference (lib/*.h): ``SignalCovarParams``, ``PCGParams``,
``PCGResult``, ``WFVectorSN`` / ``WFVectorW`` with ``A``, ``A_product``,
``A_residual``, ``preconditioner_solve``, ``norm_b`` and ``solve_pcg``, plus
``smp_product`` and ``sigma_m_noise_dom``.  Arrays are numpy float64 (host) or
CUDA float64 torch tensors for the ``*_dev`` calls.  Every call runs on the
GPU through ``libdsgb300.so``; errors raise :class:`DsError`.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import weakref

import numpy as np

from . import _lib
from ._lib import DsError

FORMS = {"sn": _lib.DS_FORM_SN, "w": _lib.DS_FORM_W}
EVALS = {"table": _lib.DS_EVAL_TABLE, "exact": _lib.DS_EVAL_EXACT}


def _f64(a, n=None, name="array"):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"{name} has {a.size} elements, expected {n}")
    return a


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _dev_ptr(t, n=None):
    """A CUDA float64 tensor's device pointer (contiguous)."""
    import torch  # device buffers only

    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64
            and t.is_contiguous()):
        raise TypeError("expected a contiguous CUDA float64 tensor")
    if n is not None and t.numel() != n:
        raise ValueError(f"tensor has {t.numel()} elements, expected {n}")
    return C.c_void_p(t.data_ptr())


def _torch_done():
    """Finish torch's pending GPU work before the library reads tensors on its
    own stream (the *_dev calls take tensors written on torch's stream)."""
    import torch

    torch.cuda.current_stream().synchronize()


def table_init():
    """SignalCovarParams' 200-knot table and its index scale 1/dx."""
    t = np.zeros(_lib.DS_TABLE_N)
    dx_inv = C.c_double()
    _lib.load().ds_table_init(_ptr(t), C.byref(dx_inv))
    return t, dx_inv.value


@dataclasses.dataclass
class SignalCovarParams:
    """lib/signal_covar.h:10-46, plus the evaluation mode."""

    var_s: float
    l_perp: float
    l_para: float
    eval: str = "table"            # "table" (reference default) or "exact"
    exact_cutoff: float = 0.0      # <= 0: library default (40)
    table: np.ndarray | None = None

    def as_c(self):
        kp = _lib.KernelParamsC()
        kp.var_s = self.var_s
        kp.l_perp = self.l_perp
        kp.l_para = self.l_para
        kp.eval = EVALS[self.eval]
        kp.exact_cutoff = self.exact_cutoff
        if self.table is not None:
            self._table_c = _f64(self.table, _lib.DS_TABLE_N, "table")
            kp.table = _ptr(self._table_c)
        else:
            kp.table = None
        return kp


@dataclasses.dataclass
class PCGParams:
    """lib/pcg.h:13-19 (n is implied by the operator)."""

    max_iter: int
    step_r: int
    tol: float
    verbose: bool = False


@dataclasses.dataclass
class MixedParams:
    """Mixed-precision solve: FP32 PCG inside FP64 reliable updates."""

    max_iter: int = 2000
    tol: float = 1e-8
    reliable_delta: float = 0.0   # <= 0: 1e-4
    inner_cutoff: float = 0.0     # <= 0: the library default (12)
    verbose: bool = False

    def as_c(self):
        return _lib.MixedParamsC(self.max_iter, self.tol, self.reliable_delta, self.inner_cutoff,
                                 int(bool(self.verbose)))


@dataclasses.dataclass
class PCGResult:
    """lib/pcg.h:21-25, plus device timing and mixed-precision counters."""

    success: bool
    num_iters: int
    residual_norms: np.ndarray
    norm_b: float
    final_norm: float
    status: int
    seconds: float
    n_outer: int = 0
    n_inner: int = 0


def signal_covar(perp2, para2, params: SignalCovarParams):
    """signal_covar / signal_covar_exact (lib/signal_covar.h:67-86) on the GPU."""
    perp2 = _f64(perp2).ravel()
    para2 = _f64(para2, perp2.size, "para2").ravel()
    out = np.empty_like(perp2)
    kp = params.as_c()
    rc = _lib.load().ds_signal_covar(C.byref(kp), perp2.size, _ptr(perp2), _ptr(para2), _ptr(out))
    if rc != _lib.DS_OK:
        raise DsError(rc, _lib.status_string(rc))
    return out


class Context:
    """One device + one CUDA stream."""

    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = C.c_void_p()
        rc = self._lib.ds_context_create(device, C.byref(h))
        if rc != _lib.DS_OK:
            raise DsError(rc, "ds_context_create: " + _lib.status_string(rc))
        self.handle = h
        self.device = device
        self._children = weakref.WeakSet()

    def _adopt(self, child):
        self._children.add(child)

    def check(self, rc, what):
        if rc not in (_lib.DS_OK,):
            msg = self._lib.ds_context_last_error(self.handle).decode()
            raise DsError(rc, f"{what}: {_lib.status_string(rc)}: {msg}")

    @property
    def stream(self) -> int:
        return self._lib.ds_context_stream(self.handle) or 0

    def synchronize(self):
        self.check(self._lib.ds_context_synchronize(self.handle), "synchronize")

    def set_profiling(self, enable: bool):
        """Time every pair-kernel launch with CUDA events on this context's stream."""
        self.check(self._lib.ds_context_set_profiling(self.handle, int(bool(enable))), "profiling")

    def set_wait_limit(self, cycles: int = 0):
        """Bound (SM clock cycles) of the device-side waits: the batched
        tensor-core kernel's mbarrier waits and the persistent mixed solve's
        grid barriers; 0 restores the default (4e9 cycles).  A wait that runs
        out makes the call raise DsError with code DS_ERR_TIMEOUT."""
        self.check(self._lib.ds_context_set_wait_limit(self.handle, int(cycles)), "wait limit")

    def profile(self) -> dict:
        p = _lib.ProfileC()
        self.check(self._lib.ds_context_get_profile(self.handle, C.byref(p)), "profile")
        return {k: getattr(p, k) for k, _ in p._fields_}

    def close(self):
        """Destroys the operators and maps made on this context, then the context."""
        if getattr(self, "handle", None):
            for child in list(self._children):
                child.close()
            self._lib.ds_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _WFVector:
    """Common body of WFVectorSN / WFVectorW (lib/wf_vector.h:14-96)."""

    FORM = None

    def __init__(self, ctx: Context, records, s_params: SignalCovarParams):
        self.ctx = ctx
        self._lib = ctx._lib
        rec = _f64(records)
        if rec.ndim != 2 or rec.shape[1] != 5:
            raise ValueError("records must have shape (n, 5)")
        self.n = rec.shape[0]
        self.s_params = s_params
        kp = s_params.as_c()
        h = C.c_void_p()
        ctx.check(self._lib.ds_operator_create(ctx.handle, self.FORM, self.n, _ptr(rec),
                                               C.byref(kp), C.byref(h)), "ds_operator_create")
        self.handle = h
        ctx._adopt(self)

    def close(self):
        if getattr(self, "handle", None):
            self._lib.ds_operator_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_dense(self, enable: bool = True):
        """Build the dense operator in HBM (or free it) for the following calls."""
        self.ctx.check(self._lib.ds_operator_set_dense(self.handle, int(bool(enable))),
                       "ds_operator_set_dense")

    _DENSE_ARITH = {"auto": 0, "float_pair": 1, "fp64": 2}

    def set_dense_arith(self, arith: str = "auto"):
        """Arithmetic of the dense matvec: "float_pair" (FP64 entries split
        into float pairs, float-float sums on the FP32 pipe; the HBM-rate
        one), "fp64" (FP64 FMAs) or "auto" (float pairs when the entries'
        range allows)."""
        self.ctx.check(self._lib.ds_operator_set_dense_arith(self.handle,
                                                             self._DENSE_ARITH[arith]),
                       "ds_operator_set_dense_arith")

    def dense_arith(self) -> str:
        """The dense matvec's arithmetic in use ("float_pair" or "fp64")."""
        v = C.c_int()
        self.ctx.check(self._lib.ds_operator_get_dense_arith(self.handle, C.byref(v)),
                       "ds_operator_get_dense_arith")
        return {1: "float_pair", 2: "fp64"}[v.value]

    def set_inner_matvec(self, variant: str = "auto"):
        """Inner matvec of solve_mixed: "cuda_core" (the CUDA-core pair
        kernel), "tensor" (pair exponents on the tensor cores where the
        expanded form applies), "structured" (the FP32 structured operator of
        set_skewer_grid) or "auto" (structured when a skewer grid is
        installed, else the CUDA-core pair kernel)."""
        v = {"auto": _lib.DS_INNER_AUTO, "cuda_core": _lib.DS_INNER_CUDA_CORE,
             "tensor": _lib.DS_INNER_TENSOR, "structured": _lib.DS_INNER_STRUCTURED}[variant]
        self.ctx.check(self._lib.ds_operator_set_inner_matvec(self.handle, v),
                       "ds_operator_set_inner_matvec")

    def set_iteration_form(self, form: str = "auto"):
        """How solve_mixed launches its iterations: "auto" (one persistent
        cooperative launch with the structured inner operator and a band
        preconditioner, else a replayed CUDA graph) or "graph" (always the
        graph of eight iterations)."""
        v = {"auto": _lib.DS_ITER_AUTO, "graph": _lib.DS_ITER_GRAPH}[form]
        self.ctx.check(self._lib.ds_operator_set_iteration_form(self.handle, v),
                       "ds_operator_set_iteration_form")

    def persistent_profile(self, reset: bool = True):
        """Phase timers of the persistent solve launches since the last reset
        (device %globaltimer): launches, kernel_ms, ctas, barrier_us (one
        empty grid barrier) and, per phase (levels0, product, step,
        levels64, update), us_per_visit, cta_mean_us, cta_max_us, visits;
        product_loads / product_rows: the neighbour values / distinct rows
        one product loads (resident form; 0 for the general form).  None
        before the first persistent launch."""
        out = (C.c_double * 26)()
        m = C.c_int(0)
        self.ctx.check(self._lib.ds_operator_get_persistent_profile(
            self.handle, out, 26, int(bool(reset)), C.byref(m)),
            "ds_operator_get_persistent_profile")
        if m.value == 0:
            return None
        v = list(out)
        prof = {"launches": int(v[0]), "kernel_ms": v[1], "ctas": int(v[2]), "barrier_us": v[3]}
        for c, name in enumerate(["levels0", "product", "step", "levels64", "update"]):
            o = v[4 + 4 * c: 8 + 4 * c]
            prof[name] = {"us_per_visit": o[0], "cta_mean_us": o[1], "cta_max_us": o[2],
                          "visits": int(o[3])}
        prof["product_loads"] = int(v[24])  # neighbour values loaded per product
        prof["product_rows"] = int(v[25])
        return prof

    def set_cluster_preconditioner(self, n_skewers: int, n_per: int, cluster: int = 4,
                                   band: int = 16) -> int:
        """Preconditions solve_mixed with the cluster factor M^-1 = G G^T
        (clusters of `cluster` neighbouring skewers, FSAI factor with `band`
        sub-diagonals) instead of Jacobi; cluster = 0 removes it.  Records
        must be skewer-contiguous (n_skewers x n_per).  Returns the number of
        columns that fell back to Jacobi."""
        nf = C.c_int(0)
        self.ctx.check(self._lib.ds_operator_set_cluster_preconditioner(
            self.handle, int(n_skewers), int(n_per), int(cluster), int(band), C.byref(nf)),
            "ds_operator_set_cluster_preconditioner")
        return nf.value

    def set_skewer_grid(self, n_skewers: int, n_per: int):
        """Installs (n_skewers > 0) or removes (0) the structured FP64
        operator for skewers on one uniform z grid (records skewer-contiguous,
        n_skewers x n_per); while installed, solve_mixed's FP64-accurate outer
        residual uses it."""
        self.ctx.check(self._lib.ds_operator_set_skewer_grid(self.handle, int(n_skewers),
                                                             int(n_per)),
                       "ds_operator_set_skewer_grid")

    def skewer_product(self, v, residual: bool = False):
        """A v (or b - A v) with the structured operator (host in, host out)."""
        import torch

        vt = torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64), device="cuda")
        out = torch.empty_like(vt)
        torch.cuda.synchronize()
        self.ctx.check(self._lib.ds_operator_skewer_product_dev(
            self.handle, int(bool(residual)), C.c_void_p(vt.data_ptr()),
            C.c_void_p(out.data_ptr())), "ds_operator_skewer_product_dev")
        self.ctx.synchronize()
        return out.cpu().numpy()

    def info(self) -> dict:
        inf = _lib.OperatorInfoC()
        self.ctx.check(self._lib.ds_operator_get_info(self.handle, C.byref(inf)), "info")
        return {k: getattr(inf, k) for k, _ in inf._fields_}

    def _vec_call(self, fn, v, name):
        v = _f64(v, self.n, name)
        out = np.empty(self.n)
        self.ctx.check(fn(self.handle, _ptr(v), _ptr(out)), fn.__name__)
        return out

    def A_product(self, a):
        return self._vec_call(self._lib.ds_A_product, a, "a")

    def A_residual(self, x):
        return self._vec_call(self._lib.ds_A_residual, x, "x")

    def A_residual_ff(self, x):
        """b - A x with the exact kernel in float-float arithmetic (the mixed
        form's outer residual)."""
        return self._vec_call(self._lib.ds_A_residual_ff, x, "x")

    def preconditioner_solve(self, b):
        return self._vec_call(self._lib.ds_preconditioner_solve, b, "b")

    def A_product_dev(self, a, b):
        _torch_done()
        self.ctx.check(self._lib.ds_A_product_dev(self.handle, _dev_ptr(a, self.n),
                                                  _dev_ptr(b, self.n)), "ds_A_product_dev")
        self.ctx.synchronize()

    def A_residual_dev(self, x, r):
        _torch_done()
        self.ctx.check(self._lib.ds_A_residual_dev(self.handle, _dev_ptr(x, self.n),
                                                   _dev_ptr(r, self.n)), "ds_A_residual_dev")
        self.ctx.synchronize()

    def norm_b(self) -> float:
        v = C.c_double()
        self.ctx.check(self._lib.ds_norm_b(self.handle, C.byref(v)), "ds_norm_b")
        return v.value

    def A(self, i, j, exact=None):
        """A(i, j, exact) for scalars or arrays of indices."""
        ii = np.ascontiguousarray(np.atleast_1d(i), dtype=np.int32)
        jj = np.ascontiguousarray(np.atleast_1d(j), dtype=np.int32)
        if ii.shape != jj.shape:
            raise ValueError("i and j must have the same shape")
        out = np.empty(ii.size)
        ev = -1 if exact is None else (_lib.DS_EVAL_EXACT if exact else _lib.DS_EVAL_TABLE)
        self.ctx.check(self._lib.ds_A_entries(self.handle, ev, ii.size,
                                              ii.ctypes.data_as(C.POINTER(C.c_int)),
                                              jj.ctypes.data_as(C.POINTER(C.c_int)), _ptr(out)),
                       "ds_A_entries")
        return out if np.ndim(i) else float(out[0])

    def _solve(self, fn, pp: PCGParams, x, dev: bool):
        c = _lib.PcgParamsC(pp.max_iter, pp.step_r, pp.tol, int(bool(pp.verbose)))
        res = _lib.PcgResultC()
        hist = np.zeros(max(pp.max_iter, 1) + 1)
        if dev:
            _torch_done()
        xp = _dev_ptr(x, self.n) if dev else _ptr(x)
        rc = fn(self.handle, C.byref(c), xp, C.byref(res), _ptr(hist))
        if dev:
            self.ctx.synchronize()
        if rc not in (_lib.DS_OK, _lib.DS_ERR_NOT_CONVERGED, _lib.DS_ERR_NORM_B):
            self.ctx.check(rc, fn.__name__)
        nh = 0 if rc == _lib.DS_ERR_NORM_B else min(hist.size, max(res.n_inner, 0) + 1)
        return PCGResult(bool(res.success), res.num_iters, hist[:nh].copy(), res.norm_b,
                         res.final_norm, rc, res.seconds, res.n_outer, res.n_inner)

    def solve_pcg(self, pcg_params: PCGParams, x=None):
        """Returns (x, PCGResult); x is the initial guess (zeros if None)."""
        x = np.zeros(self.n) if x is None else _f64(x, self.n, "x").copy()
        res = self._solve(self._lib.ds_solve_pcg, pcg_params, x, False)
        return x, res

    def solve_pcg_dev(self, pcg_params: PCGParams, x):
        """In-place solve on a CUDA float64 tensor (initial guess in, solution out)."""
        return self._solve(self._lib.ds_solve_pcg_dev, pcg_params, x, True)

    def _solve_mixed(self, fn, mp: MixedParams, x, dev: bool):
        c = mp.as_c()
        res = _lib.PcgResultC()
        hist = np.zeros(max(mp.max_iter, 1) + 2)
        if dev:
            _torch_done()
        xp = _dev_ptr(x, self.n) if dev else _ptr(x)
        rc = fn(self.handle, C.byref(c), xp, C.byref(res), _ptr(hist))
        if dev:
            self.ctx.synchronize()
        if rc not in (_lib.DS_OK, _lib.DS_ERR_NOT_CONVERGED, _lib.DS_ERR_NORM_B):
            self.ctx.check(rc, fn.__name__)
        nh = 0 if rc == _lib.DS_ERR_NORM_B else min(hist.size, res.n_inner + 1)
        return PCGResult(bool(res.success), res.num_iters, hist[:nh].copy(), res.norm_b,
                         res.final_norm, rc, res.seconds, res.n_outer, res.n_inner)

    def solve_mixed(self, mp: MixedParams = None, x=None):
        """Mixed-precision solve (exact kernel); returns (x, PCGResult)."""
        mp = mp or MixedParams()
        x = np.zeros(self.n) if x is None else _f64(x, self.n, "x").copy()
        return x, self._solve_mixed(self._lib.ds_solve_mixed, mp, x, False)

    def solve_mixed_dev(self, mp: MixedParams, x):
        return self._solve_mixed(self._lib.ds_solve_mixed_dev, mp, x, True)


class WFVectorSN(_WFVector):
    """x = (S + N)^-1 d over NPixel records {x, y, z, N, d}."""

    FORM = _lib.DS_FORM_SN


class WFVectorW(_WFVector):
    """x = w (w S w + I)^-1 w d over WPixel records {x, y, z, w, wd}."""

    FORM = _lib.DS_FORM_W


@dataclasses.dataclass
class BatchResult:
    """Per-(chunk, RHS) outcome of a batched solve, arrays of (n_chunks, n_rhs)."""

    iters: np.ndarray
    converged: np.ndarray
    n_updates: np.ndarray
    rel_resid: np.ndarray
    seconds: float
    status: int


class BatchSolver:
    """Independent chunks (each one WFVector operator) with n_rhs right-hand
    sides each, solved together by the mixed-precision method.

    ``chunks`` is a list of (n_c, 5) record arrays in the form's layout;
    right-hand sides and solutions are (n_total, n_rhs) arrays over the
    concatenated records."""

    VARIANTS = {"auto": _lib.DS_BATCH_AUTO, "cuda_core": _lib.DS_BATCH_CUDA_CORE,
                "tensor": _lib.DS_BATCH_TENSOR}

    def __init__(self, ctx: Context, form: str, chunks, s_params: SignalCovarParams,
                 n_rhs: int, inner_cutoff: float = 0.0):
        self.ctx = ctx
        self._lib = ctx._lib
        recs = [_f64(c) for c in chunks]
        for r in recs:
            if r.ndim != 2 or r.shape[1] != 5 or r.shape[0] == 0:
                raise ValueError("every chunk must be a non-empty (n, 5) record array")
        self.sizes = np.array([r.shape[0] for r in recs], dtype=np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        allrec = np.ascontiguousarray(np.concatenate(recs, axis=0))
        self.n_total = allrec.shape[0]
        self.n_chunks = len(recs)
        self.n_rhs = int(n_rhs)
        kp = s_params.as_c()
        h = C.c_void_p()
        ctx.check(self._lib.ds_batch_create(ctx.handle, FORMS[form], self.n_chunks,
                                            self.sizes.ctypes.data_as(C.POINTER(C.c_int)),
                                            _ptr(allrec), C.byref(kp), self.n_rhs,
                                            float(inner_cutoff), C.byref(h)),
                  "ds_batch_create")
        self.handle = h
        ctx._adopt(self)

    def close(self):
        if getattr(self, "handle", None):
            self._lib.ds_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        inf = _lib.BatchInfoC()
        self.ctx.check(self._lib.ds_batch_get_info(self.handle, C.byref(inf)), "info")
        return {k: getattr(inf, k) for k, _ in inf._fields_}

    def set_variant(self, variant: str = "auto", rhs_block: int = 0):
        self.ctx.check(self._lib.ds_batch_set_variant(self.handle, self.VARIANTS[variant],
                                                      int(rhs_block)), "ds_batch_set_variant")

    def _solve(self, fn, mp, rhs_ptr, x_ptr):
        shape = (self.n_chunks, self.n_rhs)
        iters = np.zeros(shape, dtype=np.int32)
        conv = np.zeros(shape, dtype=np.int32)
        nupd = np.zeros(shape, dtype=np.int32)
        rel = np.zeros(shape)
        secs = C.c_double()
        c = (mp or MixedParams()).as_c()
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
        rc = fn(self.handle, C.byref(c), rhs_ptr, x_ptr, ip(iters), ip(conv), ip(nupd),
                _ptr(rel), C.byref(secs))
        if rc not in (_lib.DS_OK, _lib.DS_ERR_NOT_CONVERGED):
            self.ctx.check(rc, fn.__name__)
        return BatchResult(iters, conv.astype(bool), nupd, rel, secs.value, rc)

    def solve_mixed(self, rhs, mp: MixedParams = None):
        """rhs: (n_total, n_rhs); returns (x, BatchResult)."""
        b = _f64(rhs, self.n_total * self.n_rhs, "rhs")
        x = np.zeros((self.n_total, self.n_rhs))
        res = self._solve(self._lib.ds_batch_solve_mixed, mp, _ptr(b), _ptr(x))
        return x, res

    def solve_mixed_dev(self, rhs, x, mp: MixedParams = None):
        """rhs, x: CUDA float64 tensors of n_total * n_rhs elements."""
        n = self.n_total * self.n_rhs
        _torch_done()
        return self._solve(self._lib.ds_batch_solve_mixed_dev, mp, _dev_ptr(rhs, n),
                           _dev_ptr(x, n))

    def product_f32_dev(self, p, q):
        n = self.n_total * self.n_rhs
        _torch_done()
        self.ctx.check(self._lib.ds_batch_product_f32_dev(self.handle, _dev_ptr(p, n),
                                                          _dev_ptr(q, n)),
                       "ds_batch_product_f32_dev")
        self.ctx.synchronize()


class MapGrid:
    """Map points sorted and tiled on the device once (for repeated products)."""

    def __init__(self, ctx: Context, points):
        self.ctx = ctx
        self._lib = ctx._lib
        pts = _f64(points)
        if pts.ndim != 2 or pts.shape[1] != 3:
            raise ValueError("points must have shape (n_map, 3)")
        self.n_map = pts.shape[0]
        h = C.c_void_p()
        ctx.check(self._lib.ds_map_create(ctx.handle, self.n_map, _ptr(pts), C.byref(h)),
                  "ds_map_create")
        self.handle = h
        ctx._adopt(self)

    def set_column_grid(self, n_columns: int, nz: int):
        """Declares the points a grid of n_columns columns of nz points (point
        c nz + j at column c's (x, y) and the j-th z), the layout of
        uniform_map_coords; with an operator that has a skewer grid,
        product_f32 is then the structured FP64 map.  0 removes it."""
        self.ctx.check(self._lib.ds_map_set_column_grid(self.handle, int(n_columns), int(nz)),
                       "ds_map_set_column_grid")

    def product(self, op: _WFVector, x):
        """smp_product with the operator's pixels and kernel."""
        x = _f64(x, op.n, "x")
        m = np.empty(self.n_map)
        self.ctx.check(self._lib.ds_map_product(self.handle, op.handle, _ptr(x), _ptr(m)),
                       "ds_map_product")
        return m

    def product_dev(self, op: _WFVector, x, m):
        """Device product on the context's stream (torch's pending work is
        finished first; the caller orders the read of m on the stream)."""
        _torch_done()
        self.ctx.check(self._lib.ds_map_product_dev(self.handle, op.handle, _dev_ptr(x, op.n),
                                                    _dev_ptr(m, self.n_map)),
                       "ds_map_product_dev")

    def product_f32(self, op: _WFVector, x, cutoff: float = 0.0):
        """FP32-evaluated exact-kernel map product with FP64 accumulation."""
        x = _f64(x, op.n, "x")
        m = np.empty(self.n_map)
        self.ctx.check(self._lib.ds_map_product_f32(self.handle, op.handle, cutoff, _ptr(x),
                                                    _ptr(m)), "ds_map_product_f32")
        return m

    def product_f32_dev(self, op: _WFVector, x, m, cutoff: float = 0.0):
        _torch_done()
        self.ctx.check(self._lib.ds_map_product_f32_dev(self.handle, op.handle, cutoff,
                                                        _dev_ptr(x, op.n),
                                                        _dev_ptr(m, self.n_map)),
                       "ds_map_product_f32_dev")

    def close(self):
        if getattr(self, "handle", None):
            self._lib.ds_map_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def smp_product(ctx: Context, pixel_coords, map_coords, s_params: SignalCovarParams, x):
    """lib/map.cc:20-43 with the reference's argument list."""
    pix = _f64(pixel_coords)
    mp = _f64(map_coords)
    x = _f64(x, pix.shape[0], "x")
    m = np.empty(mp.shape[0])
    kp = s_params.as_c()
    ctx.check(ctx._lib.ds_smp_product(ctx.handle, pix.shape[0], _ptr(pix), mp.shape[0], _ptr(mp),
                                      C.byref(kp), _ptr(x), _ptr(m)), "ds_smp_product")
    return m


def solve_cf(ctx: Context, form: str, records, s_params: SignalCovarParams):
    """WFVector{SN,W}::solve_cf: dense FP64 Cholesky solve on the GPU."""
    rec = _f64(records)
    x = np.empty(rec.shape[0])
    kp = s_params.as_c()
    ctx.check(ctx._lib.ds_solve_cf(ctx.handle, FORMS[form], rec.shape[0], _ptr(rec), C.byref(kp),
                                   _ptr(x)), "ds_solve_cf")
    return x


def map_covar_diag(ctx: Context, npixels, map_coords, s_params: SignalCovarParams,
                   pcg_params: PCGParams):
    """MapCovarDiag::solve_pcg; returns (sigma_m, iters, success)."""
    rec = _f64(npixels)
    mp = _f64(map_coords)
    m = mp.shape[0]
    out = np.zeros(m)
    iters = np.zeros(m, np.int32)
    ok = np.zeros(m, np.int32)
    kp = s_params.as_c()
    pp = _lib.PcgParamsC(pcg_params.max_iter, pcg_params.step_r, pcg_params.tol, 0)
    ctx.check(ctx._lib.ds_map_covar_diag(ctx.handle, rec.shape[0], _ptr(rec), m, _ptr(mp),
                                         C.byref(kp), C.byref(pp), _ptr(out),
                                         iters.ctypes.data_as(C.POINTER(C.c_int)),
                                         ok.ctypes.data_as(C.POINTER(C.c_int))),
              "ds_map_covar_diag")
    return out, iters, ok.astype(bool)


def sigma_m_noise_dom(ctx: Context, npixels, map_coords, s_params: SignalCovarParams):
    """lib/map_covar.cc:11-38."""
    rec = _f64(npixels)
    mp = _f64(map_coords)
    out = np.empty(mp.shape[0])
    kp = s_params.as_c()
    ctx.check(ctx._lib.ds_sigma_m_noise_dom(ctx.handle, rec.shape[0], _ptr(rec), mp.shape[0],
                                            _ptr(mp), C.byref(kp), _ptr(out)),
              "ds_sigma_m_noise_dom")
    return out


# Pixel format conversions (lib/pixel.cc:9-71), host-side like the reference.
def points_from_pixels(pixels):
    return np.ascontiguousarray(np.asarray(pixels, dtype=np.float64)[:, :3])


def pixel_to_npixel(pixels):
    p = np.array(pixels, dtype=np.float64, copy=True)
    p[:, 3] = p[:, 3] * p[:, 3]
    return p


def npixel_to_pixel(npixels):
    p = np.array(npixels, dtype=np.float64, copy=True)
    p[:, 3] = np.sqrt(p[:, 3])
    return p


def pixel_to_wpixel(pixels):
    p = np.array(pixels, dtype=np.float64, copy=True)
    n = p[:, 3].copy()
    p[:, 3] = 1.0 / n
    p[:, 4] = p[:, 4] / n
    return p


def wpixel_to_pixel(wpixels):
    p = np.array(wpixels, dtype=np.float64, copy=True)
    w = p[:, 3].copy()
    p[:, 3] = 1.0 / w
    p[:, 4] = p[:, 4] / w
    return p


def read_pixel_data(path, num_pixels):
    """lib/util.cc:11-23, with the record count checked against the file size."""
    data = np.fromfile(path, dtype=np.float64)
    if data.size < 5 * num_pixels:
        raise ValueError(f"{path}: {data.size // 5} records, expected {num_pixels}")
    return data[: 5 * num_pixels].reshape(num_pixels, 5).copy()


def init_uniform_map_coords(lx, ly, lz, nx, ny, nz):
    """lib/util.cc:25-46: cell centres, z fastest."""
    from .synth import uniform_map_coords

    return uniform_map_coords(lx, ly, lz, nx, ny, nz)
