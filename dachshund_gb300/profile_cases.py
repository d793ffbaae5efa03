"""One invocation of a single hot kernel on a workload of the benchmark's
shapes, for kernel profilers (``ncu -k <kernel> -c 1 python -m
dachshund_gb300.profile_cases <case>``):

  ff_residual    b - A x of the 262,144-pixel operator in float-float
                 arithmetic (k_pair_ff_resid), random x
  f32_matvec     one mixed-precision solve of the 262,144-pixel system
                 (k_pair_f32 launches, one per iteration)
  tc_matvec      one batched FP32 product of 64 chunks x 64 RHS with the
                 tensor-core variant (k_pack_panels + k_batch_mv_tc)
"""
from __future__ import annotations

import sys

import numpy as np


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    case = argv[0] if argv else "ff_residual"
    import torch

    from dachshund_gb300 import (BatchSolver, Context, MixedParams, SignalCovarParams,
                                 WFVectorW, pixel_to_wpixel, synth)

    ctx = Context(0)
    sp = SignalCovarParams(synth.VAR_S, synth.L_PERP, synth.L_PARA, eval="exact")
    if case in ("ff_residual", "f32_matvec"):
        w = synth.config3(0)
        rec = pixel_to_wpixel(w.pixels)
        op = WFVectorW(ctx, rec, sp)
        if case == "ff_residual":
            x = np.random.default_rng(1).standard_normal(w.n)
            r = op.A_residual_ff(x)
            print("ff_residual |r|", float(np.linalg.norm(r)))
        else:
            x, res = op.solve_mixed(MixedParams(tol=1e-8))
            print("f32_matvec iters", res.num_iters)
    elif case == "tc_matvec":
        pixes, rhs = synth.chunks(64, 0, n_rhs=64)
        recs = [pixel_to_wpixel(p) for p in pixes]
        bs = BatchSolver(ctx, "w", recs, sp, n_rhs=64)
        bs.set_variant("tensor")
        p = torch.randn(bs.n_total * 64, dtype=torch.float64, device="cuda")
        q = torch.zeros_like(p)
        bs.product_f32_dev(p, q)
        print("tc_matvec |q|", float(torch.linalg.norm(q)))
    else:
        raise SystemExit(f"unknown case {case}")
    ctx.close()


if __name__ == "__main__":
    main()
