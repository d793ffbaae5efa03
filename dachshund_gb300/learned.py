"""Learned warm start + skewer-band preconditioner (Python face of the
ds_learned_* C ABI) and the workflow around it: seeded synthetic systems of
the 262,144-pixel geometry generated on the GPU, their solutions from the
solver itself, training, and the A/B comparison against Jacobi-PCG.

The network, its losses and its kernels are described in
``csrc/learned.cu``; this module only moves data and loops over systems.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import _lib
from .api import (Context, DsError, MixedParams, SignalCovarParams, WFVectorW, _dev_ptr,
                  _f64)
from . import synth


def _fptr(t):
    import torch

    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32
            and t.is_contiguous()):
        raise TypeError("expected a contiguous CUDA float32 tensor")
    return C.c_void_p(t.data_ptr())


class LearnedPreconditioner:
    """The network: hidden width ``hidden``, band ``band`` (ds_learned_create)."""

    def __init__(self, ctx: Context, s_params: SignalCovarParams, hidden: int = 128,
                 band: int = 2, seed: int = 0):
        self.ctx, self._lib = ctx, ctx._lib
        self.hidden, self.band = hidden, band
        kp = s_params.as_c()
        h = C.c_void_p()
        ctx.check(self._lib.ds_learned_create(ctx.handle, C.byref(kp), hidden, band, seed,
                                              C.byref(h)), "ds_learned_create")
        self.handle = h
        n = C.c_longlong()
        self._lib.ds_learned_num_params(h, C.byref(n))
        self.n_params = n.value
        ctx._adopt(self)

    def close(self):
        if getattr(self, "handle", None):
            self._lib.ds_learned_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _vec(self, fn, arr=None):
        a = np.empty(self.n_params, dtype=np.float32) if arr is None else \
            np.ascontiguousarray(arr, dtype=np.float32)
        if a.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters")
        self.ctx.check(fn(self.handle, a.ctypes.data_as(C.POINTER(C.c_float))), fn.__name__)
        return a

    def get_params(self):
        return self._vec(self._lib.ds_learned_get_params)

    def set_params(self, params):
        self._vec(self._lib.ds_learned_set_params, params)

    def get_grads(self):
        return self._vec(self._lib.ds_learned_get_grads)

    def save(self, path):
        self.ctx.check(self._lib.ds_learned_save(self.handle, str(path).encode()), "save")

    def load(self, path):
        self.ctx.check(self._lib.ds_learned_load(self.handle, str(path).encode()), "load")

    def set_inference(self, tensor_cores: bool = True):
        """Message-passing layers of forward_dev on the tensor cores (TF32
        activations, the default) or on the CUDA cores in FP32 as in training."""
        self.ctx.check(self._lib.ds_learned_set_inference(self.handle, int(bool(tensor_cores))),
                       "ds_learned_set_inference")

    def forward_dev(self, n_sk, n_per, rec_dev, y0_dev=None):
        """(y0, L_rows) device tensors for W-form records ``rec_dev`` (n x 5).
        The library works on the context's stream: torch's pending work is
        finished before the call and the context's after it."""
        import torch

        torch.cuda.synchronize()
        n = n_sk * n_per
        L = torch.empty(n * (self.band + 1), dtype=torch.float32, device=rec_dev.device)
        y0 = y0_dev if y0_dev is not None else torch.empty(n, dtype=torch.float64,
                                                           device=rec_dev.device)
        self.ctx.check(self._lib.ds_learned_forward_dev(self.handle, n_sk, n_per,
                                                        _dev_ptr(rec_dev, n * 5),
                                                        _dev_ptr(y0, n), _fptr(L)),
                       "ds_learned_forward_dev")
        self.ctx.synchronize()
        return y0, L

    def train_step_dev(self, n_sk, n_per, rec_dev, ystar_dev, probe_dev, lr=1e-3, w_x=1.0,
                       w_p=1.0, update=True):
        import torch

        torch.cuda.synchronize()
        n = n_sk * n_per
        losses = np.zeros(2)
        self.ctx.check(self._lib.ds_learned_train_step_dev(
            self.handle, n_sk, n_per, _dev_ptr(rec_dev, n * 5), _dev_ptr(ystar_dev, n),
            _fptr(probe_dev), float(lr), float(w_x), float(w_p), int(bool(update)),
            losses.ctypes.data_as(C.POINTER(C.c_double))), "ds_learned_train_step_dev")
        self.ctx.synchronize()
        return losses


def set_skewer_preconditioner(op: WFVectorW, n_sk, n_per, band, L_rows):
    """Install (or, with L_rows None, remove) M^-1 = L L^T on the operator."""
    import torch

    if L_rows is None:
        ptr = None
    elif isinstance(L_rows, torch.Tensor):
        ptr = _fptr(L_rows)
    else:
        L_rows = np.ascontiguousarray(L_rows, dtype=np.float32)
        ptr = L_rows.ctypes.data_as(C.c_void_p)
    op.ctx.check(op._lib.ds_operator_set_skewer_preconditioner(op.handle, n_sk, n_per, band,
                                                                 ptr),
                 "ds_operator_set_skewer_preconditioner")


# ---- synthetic systems on the GPU ------------------------------------------------

def gpu_system(seed, n_sk=1024, n_per=256, box=80.0, dz=synth.DZ, device="cuda",
               var_s=synth.VAR_S, l_perp=synth.L_PERP, l_para=synth.L_PARA):
    """W-form records (n x 5, float64, device) of one seeded system of the
    skewer workload's law: skewer (x, y) uniform in [0, box)^2, pixels at
    z_k = (k + 1/2) dz, noise n ~ U[0.05, 0.3], d = GRF (Gaussian power
    spectrum of the kernel, 1 Mpc/h periodic grid, trilinear) + n N(0, 1).
    Generated with torch's seeded generator on the GPU (same law as
    ``synth.wf262144``, different random streams)."""
    import torch

    g = torch.Generator(device=device).manual_seed(int(seed))
    f64 = torch.float64
    n = n_sk * n_per
    xy = torch.rand(n_sk, 2, generator=g, device=device, dtype=f64) * box
    z = (torch.arange(n_per, device=device, dtype=f64) + 0.5) * dz
    noise = 0.05 + 0.25 * torch.rand(n, generator=g, device=device, dtype=f64)
    shape = (int(round(box)), int(round(box)), int(round(n_per * dz)))
    kx = 2 * math.pi * torch.fft.fftfreq(shape[0], d=1.0, device=device, dtype=f64)
    ky = 2 * math.pi * torch.fft.fftfreq(shape[1], d=1.0, device=device, dtype=f64)
    kz = 2 * math.pi * torch.fft.rfftfreq(shape[2], d=1.0, device=device, dtype=f64)
    kp2 = kx[:, None, None] ** 2 + ky[None, :, None] ** 2
    P = var_s * (2 * math.pi) ** 1.5 * l_perp ** 2 * l_para * torch.exp(
        -(kp2 * l_perp ** 2 + kz[None, None, :] ** 2 * l_para ** 2) / 2)
    white = torch.randn(shape, generator=g, device=device, dtype=f64)
    field = torch.fft.irfftn(torch.fft.rfftn(white) * torch.sqrt(P), s=shape)
    pts = torch.stack([xy[:, 0].repeat_interleave(n_per), xy[:, 1].repeat_interleave(n_per),
                       z.repeat(n_sk)], dim=1)
    gpos = pts - 0.5
    i0 = torch.floor(gpos).long()
    fr = gpos - i0
    sig = torch.zeros(n, device=device, dtype=f64)
    for dx in (0, 1):
        wx = fr[:, 0] if dx else 1 - fr[:, 0]
        ix = (i0[:, 0] + dx) % shape[0]
        for dy in (0, 1):
            wy = fr[:, 1] if dy else 1 - fr[:, 1]
            iy = (i0[:, 1] + dy) % shape[1]
            for dzz in (0, 1):
                wz = fr[:, 2] if dzz else 1 - fr[:, 2]
                iz = (i0[:, 2] + dzz) % shape[2]
                sig += wx * wy * wz * field[ix, iy, iz]
    d = sig + noise * torch.randn(n, generator=g, device=device, dtype=f64)
    rec = torch.empty(n, 5, device=device, dtype=f64)
    rec[:, :3] = pts
    rec[:, 3] = 1.0 / noise
    rec[:, 4] = d / noise
    return rec


def solve_reference(ctx, rec_dev, s_params, tol=1e-8, max_iter=3000):
    """The solver's own solution y* (unscaled W variable) of a system, with
    the Jacobi-preconditioned mixed-precision PCG (FP64 residual <= tol |b|)."""
    import torch

    op = WFVectorW(ctx, rec_dev.cpu().numpy(), s_params)
    x = torch.zeros(rec_dev.shape[0], dtype=torch.float64, device=rec_dev.device)
    torch.cuda.synchronize()
    res = op.solve_mixed_dev(MixedParams(max_iter=max_iter, tol=tol), x)
    if not res.success:
        raise DsError(_lib.DS_ERR_NOT_CONVERGED, "reference solve did not converge")
    y = x / rec_dev[:, 3]
    return op, y, res


def train(net: LearnedPreconditioner, ctx, s_params, seeds, n_sk=1024, n_per=256, box=80.0,
          lr=1e-3, lr_min=2e-5, w_x=1.0, w_p=1.0, log_every=100, log=print):
    """One pass over the systems of ``seeds``: generate, solve, one step each
    (cosine learning-rate decay).  Returns the per-step losses."""
    import torch

    hist = []
    n = n_sk * n_per
    pg = torch.Generator(device="cuda").manual_seed(12345)
    t0 = time.time()
    for step, seed in enumerate(seeds):
        rec = gpu_system(seed, n_sk, n_per, box)
        op, y, _ = solve_reference(ctx, rec, s_params)
        op.close()
        probe = torch.randn(n, generator=pg, device="cuda", dtype=torch.float32)
        frac = step / max(1, len(seeds) - 1)
        lr_t = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * frac))
        ls = net.train_step_dev(n_sk, n_per, rec, y.contiguous(), probe, lr_t, w_x, w_p)
        hist.append(ls)
        if log and (step % log_every == 0 or step == len(seeds) - 1):
            log(f"step {step} seed {seed} loss_x {ls[0]:.4f} loss_p {ls[1]:.4f} "
                f"lr {lr_t:.2e} {time.time() - t0:.1f}s")
    return np.array(hist)


def compare(net: LearnedPreconditioner, ctx, s_params, seeds, n_sk=1024, n_per=256, box=80.0,
            tol=1e-8):
    """Per system: mixed-precision PCG from 0 with Jacobi against the learned
    form (warm start y0 + M^-1 = L L^T); device times, iterations and FP64
    residuals, and the learned solution's difference from Jacobi's."""
    import torch

    out = []
    mp = MixedParams(max_iter=3000, tol=tol)
    for seed in seeds:
        rec = gpu_system(seed, n_sk, n_per, box)
        op = WFVectorW(ctx, rec.cpu().numpy(), s_params)
        x_j = torch.zeros(rec.shape[0], dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rj = op.solve_mixed_dev(mp, x_j)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        y0, L = net.forward_dev(n_sk, n_per, rec)
        e1.record()
        e1.synchronize()
        t_net = e0.elapsed_time(e1) * 1e-3
        set_skewer_preconditioner(op, n_sk, n_per, net.band, L)
        x_l = y0.clone()
        torch.cuda.synchronize()
        rl = op.solve_mixed_dev(mp, x_l)
        set_skewer_preconditioner(op, n_sk, n_per, net.band, None)
        fallback = not rl.success
        if fallback:  # Jacobi-PCG is the fallback
            x_l = torch.zeros_like(x_j)
            torch.cuda.synchronize()
            rl = op.solve_mixed_dev(mp, x_l)
        x0_err = float(torch.linalg.norm(y0 * rec[:, 3] - x_j) / torch.linalg.norm(x_j))
        out.append({
            "seed": int(seed),
            "jacobi_iters": rj.num_iters, "jacobi_s": rj.seconds,
            "learned_iters": rl.num_iters, "learned_s": rl.seconds + t_net,
            "net_s": t_net, "fallback": fallback,
            "x0_rel_err": x0_err,
            "learned_rel_resid": rl.final_norm / rl.norm_b,
            "x_diff": float(torch.max(torch.abs(x_l - x_j)) / torch.max(torch.abs(x_j))),
        })
        op.close()
    return out


def main(argv=None):
    """Training and evaluation on the 262,144-pixel geometry:

      python -m dachshund_gb300.learned train --out W.bin [--first 1 --last 2000]
      python -m dachshund_gb300.learned evaluate --weights W.bin [--first 10001 --last 10100]
    """
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["train", "evaluate"])
    ap.add_argument("--out", default=None)
    ap.add_argument("--weights", default=None)
    ap.add_argument("--first", type=int, default=None)
    ap.add_argument("--last", type=int, default=None)
    ap.add_argument("--hidden", type=int, default=128)
    ap.add_argument("--band", type=int, default=2)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--json", default=None, help="write the per-system results here")
    a = ap.parse_args(argv)
    ctx = Context(0)
    sp = SignalCovarParams(synth.VAR_S, synth.L_PERP, synth.L_PARA, eval="exact")
    net = LearnedPreconditioner(ctx, sp, hidden=a.hidden, band=a.band, seed=0)
    if a.mode == "train":
        first, last = a.first or 1, a.last or 2000
        t0 = time.time()
        hist = train(net, ctx, sp, range(first, last + 1), lr=a.lr)
        out = {"seeds": [first, last], "seconds": time.time() - t0,
               "loss_first": hist[:10].mean(0).tolist(), "loss_last": hist[-10:].mean(0).tolist()}
        if a.out:
            net.save(a.out)
        print(json.dumps(out), flush=True)
    else:
        if a.weights:
            net.load(a.weights)
        first, last = a.first or 10001, a.last or 10100
        rows = compare(net, ctx, sp, range(first, last + 1))
        summ = {
            "systems": len(rows),
            "jacobi_iters_mean": float(np.mean([r["jacobi_iters"] for r in rows])),
            "learned_iters_mean": float(np.mean([r["learned_iters"] for r in rows])),
            "jacobi_s_mean": float(np.mean([r["jacobi_s"] for r in rows])),
            "learned_s_mean": float(np.mean([r["learned_s"] for r in rows])),
            "net_s_mean": float(np.mean([r["net_s"] for r in rows])),
            "fallbacks": int(sum(r["fallback"] for r in rows)),
            "x0_rel_err_mean": float(np.mean([r["x0_rel_err"] for r in rows])),
            "max_rel_resid": float(max(r["learned_rel_resid"] for r in rows)),
            "max_x_diff": float(max(r["x_diff"] for r in rows)),
        }
        if a.json:
            with open(a.json, "w") as f:
                json.dump({"summary": summ, "rows": rows}, f)
        print(json.dumps(summ), flush=True)


if __name__ == "__main__":
    main()
