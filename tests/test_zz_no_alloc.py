"""GPU test of ds_solve_pcg_noalloc, the solve entry point that allocates no
device memory (for callers that own all device memory through their own pool
or must not call cudaMalloc mid-run).  It is called through the C ABI with
device buffers the test owns, and its output is checked against the regular
entry point ds_solve_pcg on the same inputs, with the tolerances of the other
PCG tests: the solution within 1e-8 relative at a forced equal iteration
count, and converged iteration counts within 2.  Two calls in a row check
that the shared work space is re-initialised by each call, and around a
call made after a warm-up the device's free memory and torch's reserved
memory stay unchanged (the call allocates nothing).

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from dachshund_gb300 import (PCGParams, SignalCovarParams, WFVectorSN, WFVectorW, _lib,
                             pixel_to_npixel, pixel_to_wpixel, synth)

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA
MAX_N = 32768


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def raw_call(form, n, d_rec, sp, pp, d_x, stream):
    """One ds_solve_pcg_noalloc call on device buffers the caller owns."""
    lib = _lib.load()
    kp = sp.as_c()
    c = _lib.PcgParamsC(pp.max_iter, pp.step_r, pp.tol, 0)
    res = _lib.PcgResultC()
    hist = np.zeros(max(pp.max_iter, 1) + 1)
    rc = lib.ds_solve_pcg_noalloc(_lib.DS_FORM_SN if form == "sn" else _lib.DS_FORM_W, n,
                                  C.c_void_p(d_rec.data_ptr()), C.byref(kp), C.byref(c),
                                  C.c_void_p(d_x.data_ptr()), C.byref(res),
                                  hist.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_void_p(stream.cuda_stream))
    return rc, res, hist


def noalloc_solve(form, rec, sp, pp, x0, stream):
    import torch

    d_rec = torch.tensor(rec, dtype=torch.float64, device="cuda").contiguous()
    d_x = torch.tensor(x0, dtype=torch.float64, device="cuda").contiguous()
    torch.cuda.synchronize()
    rc, res, hist = raw_call(form, rec.shape[0], d_rec, sp, pp, d_x, stream)
    return rc, d_x.cpu().numpy(), res, hist


@pytest.mark.parametrize("form", ["w", "sn"])
@pytest.mark.parametrize("ev", ["table", "exact"])
def test_noalloc_matches_regular_entry_point(ctx, form, ev):
    import torch

    stream = torch.cuda.Stream()
    sp = SignalCovarParams(VS, LP, LQ, eval=ev)
    w = synth.small(20, 40, 13.0, seed=31)
    rec = pixel_to_wpixel(w.pixels) if form == "w" else pixel_to_npixel(w.pixels)
    op = (WFVectorW if form == "w" else WFVectorSN)(ctx, rec, sp)
    x_ref, r_ref = op.solve_pcg(PCGParams(1000, 50, 1e-8))
    assert r_ref.success
    it = r_ref.num_iters
    xf_ref, _ = op.solve_pcg(PCGParams(it + 1, 50, 0.0))
    for call in range(2):  # two calls in a row share the work space
        rc, x, res, hist = noalloc_solve(form, rec, sp, PCGParams(1000, 50, 1e-8),
                                         np.zeros(w.n), stream)
        assert rc == _lib.DS_OK and res.success, (call, rc)
        assert abs(res.num_iters - r_ref.num_iters) <= 2
        assert res.final_norm <= 1e-8 * res.norm_b
        # Both converged to |r| <= 1e-8 |b|, possibly an iteration apart:
        # their solutions agree to about tol * cond(A) (cond < 100 here).
        assert rel(x, x_ref) < 1e-6
        k = min(20, r_ref.residual_norms.size)
        np.testing.assert_allclose(hist[:k], r_ref.residual_norms[:k], rtol=1e-9)
        # Forced equal iteration count (tol 0): the same number of CG steps,
        # solutions within 1e-8 relative.
        rc, xf, res, _ = noalloc_solve(form, rec, sp, PCGParams(it + 1, 50, 0.0),
                                       np.zeros(w.n), stream)
        assert rc == _lib.DS_ERR_NOT_CONVERGED and res.num_iters == it + 1
        assert rel(xf, xf_ref) < 1e-8


def test_noalloc_initial_guess_and_limits(ctx):
    import torch

    stream = torch.cuda.Stream()
    sp = SignalCovarParams(VS, LP, LQ)
    w = synth.small(10, 30, 10.0, seed=5)
    rec = pixel_to_wpixel(w.pixels)
    op = WFVectorW(ctx, rec, sp)
    x0 = np.random.default_rng(1).standard_normal(w.n)
    x_ref, r_ref = op.solve_pcg(PCGParams(500, 10, 1e-9), x0)
    rc, x, res, _ = noalloc_solve("w", rec, sp, PCGParams(500, 10, 1e-9), x0, stream)
    assert rc == _lib.DS_OK and abs(res.num_iters - r_ref.num_iters) <= 2
    assert rel(x, x_ref) < 1e-7
    xf_ref, _ = op.solve_pcg(PCGParams(r_ref.num_iters + 1, 10, 0.0), x0)
    rc, xf, _, _ = noalloc_solve("w", rec, sp, PCGParams(r_ref.num_iters + 1, 10, 0.0), x0,
                                 stream)
    assert rc == _lib.DS_ERR_NOT_CONVERGED and rel(xf, xf_ref) < 1e-8
    # beyond the fixed work space: rejected before any device work
    big = np.tile(rec, (MAX_N // w.n + 1, 1))[: MAX_N + 1]
    rc, _, _, _ = noalloc_solve("w", big, sp, PCGParams(10, 10, 1e-8), np.zeros(MAX_N + 1),
                                stream)
    assert rc == _lib.DS_ERR_ARG


def test_noalloc_call_allocates_nothing(ctx):
    """After a warm-up call (which, with CUDA's lazy module loading, is when
    the work space is reserved on the device), a call leaves the device's free
    memory and torch's reserved memory as they were."""
    import torch

    stream = torch.cuda.Stream()
    sp = SignalCovarParams(VS, LP, LQ, eval="exact")
    w = synth.small(16, 40, 12.0, seed=41)
    rec = pixel_to_wpixel(w.pixels)
    d_rec = torch.tensor(rec, dtype=torch.float64, device="cuda").contiguous()
    d_x = torch.zeros(w.n, dtype=torch.float64, device="cuda")
    pp = PCGParams(1000, 50, 1e-8)
    torch.cuda.synchronize()
    rc, res, _ = raw_call("w", w.n, d_rec, sp, pp, d_x, stream)  # warm-up
    assert rc == _lib.DS_OK and res.success
    x1 = d_x.cpu().numpy()
    d_x.zero_()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    rc, res, _ = raw_call("w", w.n, d_rec, sp, pp, d_x, stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == _lib.DS_OK and res.success
    assert free1 == free0 and torch.cuda.memory_reserved() == reserved0
    assert rel(d_x.cpu().numpy(), x1) == 0.0  # same inputs, same work, same result


@pytest.mark.parametrize("max_iter,success", [(0, True), (1, False)])
def test_noalloc_max_iter_edges(ctx, max_iter, success):
    """lib/pcg.h:117-158: max_iter 0 returns success with one iteration,
    max_iter 1 fails with one iteration (the loop variable leaves the loop at
    1); the regular entry point agrees."""
    import torch

    stream = torch.cuda.Stream()
    sp = SignalCovarParams(VS, LP, LQ)
    w = synth.small(6, 20, 8.0, seed=7)
    rec = pixel_to_wpixel(w.pixels)
    rc, _, res, _ = noalloc_solve("w", rec, sp, PCGParams(max_iter, 50, 1e-8), np.zeros(w.n),
                                  stream)
    assert bool(res.success) == success and res.num_iters == 1
    assert rc == (_lib.DS_OK if success else _lib.DS_ERR_NOT_CONVERGED)
    op = WFVectorW(ctx, rec, sp)
    _, r = op.solve_pcg(PCGParams(max_iter, 50, 1e-8))
    assert bool(r.success) == success and r.num_iters == 1
    op.close()
