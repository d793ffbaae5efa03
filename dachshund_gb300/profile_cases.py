"""One invocation of a single hot kernel on a workload of the benchmark's
shapes, for kernel profilers (``ncu --clock-control none -k <kernel> -c 1
python -m dachshund_gb300.profile_cases <case>``; ``--clock-control none``
leaves the GPU's clocks as they are):

  ff_residual    b - A x of the 262,144-pixel operator in float-float
                 arithmetic (k_pair_ff_resid), random x
  f32_matvec     one mixed-precision solve of the 262,144-pixel system
                 (k_pair_f32 launches, one per iteration)
  e2e_parts      the end-to-end call sequence of the benchmark's chosen form
                 from pinned host buffers (operator, preconditioner, skewer
                 grid, solve, map grid, column grid, map product), each call
                 timed on the host after a synchronize (second pass printed)
  chosen_step    one step of the benchmark's chosen form on the 262,144-pixel
                 system, after one untimed warm-up step: cluster
                 preconditioner and skewer grid installed, the mixed solve
                 (the start kernels, then one persistent launch of
                 k_mixed_resident) and the 80 x 80 x 512 structured map
                 (k_mc_split + k_mc_fused)
  tc_matvec      one batched FP32 product of 64 chunks x 64 RHS with the
                 tensor-core variant (k_pack_panels + k_batch_mv_tc)
  tc_inner       one mixed-precision solve of the 262,144-pixel system with
                 the tensor-core inner matvec (k_tc_columns + k_pair_tc)
  learned_solve  one held-out 262,144-pixel system: Jacobi mixed solve, the
                 network's forward pass and the learned-preconditioned solve
                 (trained weights in dachshund_gb300/weights)
  plain_matvec   one FP64 product A a of the 262,144-pixel operator, exact
                 kernel (k_pair_f64<EXACT, PRODUCT>), random a
  dense_matvec   the dense operator of a 16,384-pixel system of the
                 32,768-pixel workload's density (128 skewers x 128 pixels
                 in [0,28.3)^2 x [0,256) Mpc/h, 16,384^2 FP64 = 2.1 GB):
                 built, then three products (k_split_vec + k_dense_mv each)
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
    if case == "e2e_parts":
        import time

        from dachshund_gb300 import MapGrid

        w = synth.wf262144(0)
        rec = torch.from_numpy(pixel_to_wpixel(w.pixels)).pin_memory().numpy()
        pts = torch.from_numpy(synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny,
                                                        w.map_nz)).pin_memory().numpy()
        for rep in range(2):
            t = {}

            def mark(name, t0):
                ctx.synchronize()
                torch.cuda.synchronize()
                t[name] = round((time.perf_counter() - t0) * 1e3, 2)
                return time.perf_counter()

            t0 = time.perf_counter()
            op = WFVectorW(ctx, rec, sp)
            t0 = mark("operator", t0)
            op.set_cluster_preconditioner(w.n_skewers, w.pix_per_skewer, 4, 16)
            t0 = mark("cluster_pc", t0)
            op.set_skewer_grid(w.n_skewers, w.pix_per_skewer)
            t0 = mark("skewer_grid", t0)
            x, res = op.solve_mixed(MixedParams(max_iter=3000, tol=1e-8))
            t0 = mark("solve", t0)
            grid = MapGrid(ctx, pts)
            t0 = mark("map_grid", t0)
            grid.set_column_grid(w.map_nx * w.map_ny, w.map_nz)
            t0 = mark("column_grid", t0)
            m = grid.product_f32(op, x)
            t0 = mark("map_product", t0)
            m = grid.product_f32(op, x)
            t0 = mark("map_product_again", t0)
            x, res = op.solve_mixed(MixedParams(max_iter=3000, tol=1e-8))
            t0 = mark("solve_again", t0)
            grid.close()
            op.close()
            mark("close", t0)
        print(case, "ms", t)
    elif case == "chosen_step":
        from dachshund_gb300 import MapGrid

        w = synth.wf262144(0)
        rec = pixel_to_wpixel(w.pixels)
        op = WFVectorW(ctx, rec, sp)
        op.set_cluster_preconditioner(w.n_skewers, w.pix_per_skewer, 4, 16)
        op.set_skewer_grid(w.n_skewers, w.pix_per_skewer)
        grid = MapGrid(ctx, synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny,
                                                     w.map_nz))
        grid.set_column_grid(w.map_nx * w.map_ny, w.map_nz)
        x = torch.zeros(w.n, dtype=torch.float64, device="cuda")
        m = torch.empty(w.n_map, dtype=torch.float64, device="cuda")
        for _ in range(2):
            torch.cuda.synchronize()
            x.zero_()
            torch.cuda.synchronize()
            res = op.solve_mixed_dev(MixedParams(max_iter=3000, tol=1e-8), x)
            grid.product_f32_dev(op, x, m)
            ctx.synchronize()
        print(case, "iters", res.num_iters, "updates", res.n_outer)
        grid.close()
    elif case in ("ff_residual", "f32_matvec", "tc_inner", "plain_matvec"):
        w = synth.wf262144(0)
        rec = pixel_to_wpixel(w.pixels)
        op = WFVectorW(ctx, rec, sp)
        if case == "plain_matvec":
            b = op.A_product(np.random.default_rng(1).standard_normal(w.n))
            print("plain_matvec |b|", float(np.linalg.norm(b)))
        elif case == "ff_residual":
            x = np.random.default_rng(1).standard_normal(w.n)
            r = op.A_residual_ff(x)
            print("ff_residual |r|", float(np.linalg.norm(r)))
        else:
            if case == "tc_inner":
                op.set_inner_matvec("tensor")
            x, res = op.solve_mixed(MixedParams(tol=1e-8))
            print(case, "iters", res.num_iters)
    elif case == "dense_matvec":
        w = synth.grf_workload("wf-16384px-grf", 128, 128, 40.0 / np.sqrt(2.0), 0,
                               (28, 28, 256), 1e-8)
        op = WFVectorW(ctx, pixel_to_wpixel(w.pixels), sp)
        op.set_dense(True)
        a = np.random.default_rng(1).standard_normal(w.n)
        for _ in range(3):
            b = op.A_product(a)
        print("dense_matvec", op.dense_arith(), "|b|", float(np.linalg.norm(b)))
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
