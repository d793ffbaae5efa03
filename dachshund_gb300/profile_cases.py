"""One invocation of a single hot kernel on a workload of the benchmark's
shapes, for kernel profilers (``ncu -k <kernel> -c 1 python -m
dachshund_gb300.profile_cases <case>``):

  ff_residual    b - A x of the 262,144-pixel operator in float-float
                 arithmetic (k_pair_ff_resid), random x
  f32_matvec     one mixed-precision solve of the 262,144-pixel system
                 (k_pair_f32 launches, one per iteration)
  tc_matvec      one batched FP32 product of 64 chunks x 64 RHS with the
                 tensor-core variant (k_pack_panels + k_batch_mv_tc)
  tc_inner       one mixed-precision solve of the 262,144-pixel system with
                 the tensor-core inner matvec (k_tc_columns + k_pair_tc)
  learned_solve  one held-out 262,144-pixel system: Jacobi mixed solve, the
                 network's forward pass and the learned-preconditioned solve
                 (trained weights in dachshund_gb300/weights)
  pipe_rates     per-SM throughput of FP64 FMA, FP32 FMA, MUFU ex2, FP64
                 exp() and FP64 -> int32 (probes/pipe_rates.cu, compiled here
                 for sm_103a; the rates behind the pair kernels' rooflines)
"""
from __future__ import annotations

import sys

import numpy as np


def pipe_rates() -> None:
    """Compile probes/pipe_rates.cu for sm_103a and run it."""
    import importlib
    import os
    import subprocess

    build = importlib.import_module("dachshund_gb300.build")  # the module, not build()
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "probes", "pipe_rates.cu")
    os.makedirs(build.BUILD, exist_ok=True)
    exe = os.path.join(build.BUILD, "pipe_rates")
    subprocess.run([build.nvcc()] + build.ARCH + ["-O3", "-std=c++17", src, "-o", exe],
                   check=True)
    subprocess.run([exe], check=True)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    case = argv[0] if argv else "ff_residual"
    if case == "pipe_rates":
        pipe_rates()
        return
    import torch

    from dachshund_gb300 import (BatchSolver, Context, MixedParams, SignalCovarParams,
                                 WFVectorW, pixel_to_wpixel, synth)

    ctx = Context(0)
    sp = SignalCovarParams(synth.VAR_S, synth.L_PERP, synth.L_PARA, eval="exact")
    if case in ("ff_residual", "f32_matvec", "tc_inner"):
        w = synth.wf262144(0)
        rec = pixel_to_wpixel(w.pixels)
        op = WFVectorW(ctx, rec, sp)
        if case == "ff_residual":
            x = np.random.default_rng(1).standard_normal(w.n)
            r = op.A_residual_ff(x)
            print("ff_residual |r|", float(np.linalg.norm(r)))
        else:
            if case == "tc_inner":
                op.set_inner_matvec("tensor")
            x, res = op.solve_mixed(MixedParams(tol=1e-8))
            print(case, "iters", res.num_iters)
    elif case == "tc_matvec":
        pixes, rhs = synth.chunks(64, 0, n_rhs=64)
        recs = [pixel_to_wpixel(p) for p in pixes]
        bs = BatchSolver(ctx, "w", recs, sp, n_rhs=64)
        bs.set_variant("tensor")
        p = torch.randn(bs.n_total * 64, dtype=torch.float64, device="cuda")
        q = torch.zeros_like(p)
        bs.product_f32_dev(p, q)
        print("tc_matvec |q|", float(torch.linalg.norm(q)))
    elif case == "learned_solve":
        import os

        from dachshund_gb300.learned import LearnedPreconditioner, compare

        net = LearnedPreconditioner(ctx, sp, hidden=128, band=2)
        net.load(os.path.join(os.path.dirname(__file__), "weights", "learned_wf262144.bin"))
        row = compare(net, ctx, sp, [10001])[0]
        print("learned_solve", {k: row[k] for k in ("jacobi_iters", "learned_iters",
                                                    "jacobi_s", "learned_s", "net_s")})
        net.close()
    else:
        raise SystemExit(f"unknown case {case}")
    ctx.close()


if __name__ == "__main__":
    main()
