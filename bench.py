#!/usr/bin/env python3
"""Wiener-filter solve benchmark on GB300.

One step = one full Wiener-filter solve of the chosen form on the 262,144-pixel
workload (1,024 skewers x 256 pixels in [0,80)^2 x [0,512) Mpc/h, GRF data,
exact Gaussian kernel var_s 0.0625, l_perp 2.5, l_para 2.0): mixed-precision
PCG (FP32 inner, FP64 reliable updates) from x = 0 to |b - A x| <= 1e-8 |b|,
then the map m = S_mp x on the 80 x 80 x 512 grid (FP32 evaluation, FP64
accumulation).  The plain FP64 GPU PCG + FP64 map on the same system is run
once beside it, as the metric asks ("chosen form vs plain FP64 GPU PCG").

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (the solve does not shard here); rank 0
prints one JSON line.  ``--impl reference`` times the reference's algorithm
on the host cores (the C/OpenMP restatement in oracle/, bit-exact with the
reference; the reference's sources are not part of this repository, so the
reference itself is not built where the benchmark runs) on a bounded sample
of rows, extrapolated to the full solve.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "WF solve time & CG iters to 1e-8 resid: chosen form vs plain FP64 GPU PCG"
SMS = 152
# Per-SM pipe rates measured on a GB300 (profiles/pipe_rates_gb300.md):
# FP32 FMA 128 lanes/clk, MUFU ex2 32/clk, FP64 FMA 2/clk.
FMA_LANES, MUFU_RATE, DFMA_RATE = 128.0, 32.0, 2.0
# FP32 inner kernel (EXPANDED): 4 FMA lanes + 1 ex2 per pair; map kernel
# (DIRECT): 7 FMA lanes + 1 ex2 per pair.
PAIRS_PER_CLK = {"expanded": min(FMA_LANES / 4, MUFU_RATE), "direct": min(FMA_LANES / 7, MUFU_RATE)}
# DRAM traffic of one k_pair_f32 launch on the 262,144-pixel workload, measured
# once with ncu (dram__bytes_read.sum + dram__bytes_write.sum)
K_PAIR_F32_DRAM_BYTES = 9_174_528
# DRAM bytes of one structured FP32 inner product (k_sg32_levels +
# k_sg32_apply) on the 262,144-pixel workload, from one ncu capture
# (profiles/k_sg32_inner_wf262144.md)
K_SG32_DRAM_BYTES = 16_603_136  # k_sg32_levels 4,202,496 + k_sg32_apply 12,400,640
# DRAM bytes (read + write) of one launch of the persistent solve on the
# 262,144-pixel workload (profiles/k_mixed_resident_wf262144.md)
K_PERSIST_DRAM_BYTES = 44_619_520  # read 43,064,576 + write 1,554,944
# the structured inner operator's cutoff (DS_DEFAULT_STRUCTURED_INNER_CUTOFF)
SG_INNER_CUT = 14.0
# FP64-pipe instructions per evaluated pair of the plain FP64 kernel
# k_pair_f64<EXACT, PRODUCT> on the 262,144-pixel workload, from one ncu
# capture (FP64-pipe busy fraction x 2 per clock x active SM cycles / the
# launch's evaluated pairs; profiles/k_pair_f64_exact_wf262144.md)
K_PAIR_F64_EXACT_OPS = 17.4
# Plain FP64 iteration count of the workload (tol 1e-8, exact kernel), for the
# CPU-baseline extrapolation of the reference arm.
REF_ITERS = {"wf-262144px-grf": 162, "wf-32768px-grf": 150}
# The chosen form's preconditioner: skewers per cluster and sub-diagonals of
# the FSAI factor (ds_operator_set_cluster_preconditioner).
PC_CLUSTER, PC_BAND = 4, 16


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="wf262144", choices=["wf32768", "wf262144"])
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-chunks (512 chunks x 64 RHS) measurement")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-preconditioner measurement")
    ap.add_argument("--no-pair-form", action="store_true",
                    help="skip the pair-kernel form of the solve (k_pair_f32 roofline)")
    ap.add_argument("--no-wf4096", action="store_true",
                    help="skip the 4,096-pixel app-path measurement (GPU and CPU, whole)")
    ap.add_argument("--no-map-covar", action="store_true",
                    help="skip the MapCovarDiag measurement")
    ap.add_argument("--no-wf32768", action="store_true",
                    help="skip the 32,768-pixel dense / matrix-free measurement")
    ap.add_argument("--cpu-sample-s", type=float, default=6.0,
                    help="seconds of CPU work per baseline sample")
    return ap.parse_args()


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region
    (every 20 ms; only the samples taken between mark_start() and mark_end()
    count, all of them if none fell inside)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
            return
        deadline = time.perf_counter() + 5.0  # sampling is live before the region starts
        while not self.lines and time.perf_counter() < deadline and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        lines = self.lines
        if self.t0 is not None and self.t1 is not None:
            inside = [x for x in lines if self.t0 <= x[0] <= self.t1]
            lines = inside or lines
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(name):
    from dachshund_gb300 import synth

    return getattr(synth, name)()


def cpu_baseline(w, iters, target_s):
    """Times the C/OpenMP restatement of the reference (oracle port, bit-exact
    with it) on the host cores on rows of one A_product and of smp_product and
    extrapolates to the full solve (iters matvecs + 1 residual + iters //
    step_r residuals + the map).  It runs the reference's table kernel, the
    one its app uses, which costs less per pair than exp."""
    import numpy as np

    import oracle
    from dachshund_gb300 import api, synth

    rec = api.pixel_to_wpixel(w.pixels)
    a = np.random.default_rng(0).standard_normal(w.n)
    pts = synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny, w.map_nz)

    def rate(fn, rows_total, cols):
        r = 64
        t0 = time.perf_counter()
        fn(0, r)
        dt = time.perf_counter() - t0
        r = int(min(rows_total, max(256, target_s / 2 / max(dt / r, 1e-9))))
        t0 = time.perf_counter()
        fn(0, r)
        dt = time.perf_counter() - t0
        return dt / (r * cols), r, dt

    t_op, r_op, d_op = rate(lambda r0, r1: oracle.A_product_rows(
        "w", rec, a, r0, r1, w.var_s, w.l_perp, w.l_para, exact=False), w.n, w.n)
    t_map, r_map, d_map = rate(lambda r0, r1: oracle.smp_product_rows(
        w.pixels[:, :3], pts, a, r0, r1, w.var_s, w.l_perp, w.l_para, exact=False), w.n_map, w.n)
    matvecs = iters + 1 + iters // w.pcg_step_r
    total = t_op * w.n * w.n * matvecs + t_map * w.n_map * w.n
    cores = os.cpu_count()
    return {
        "value": total, "unit": "s", "cores": cores, "kind": "port",
        "sample": (f"rows [0,{r_op}) of A_product ({d_op:.1f} s) and rows [0,{r_map}) of "
                   f"smp_product ({d_map:.1f} s), the reference's table kernel (its app path; "
                   f"cheaper per pair than exp), OpenMP on {cores} host threads; "
                   f"extrapolated to {matvecs} matvecs + the {w.n_map}-point map"),
        "ns_per_pair": t_op * 1e9,
        "rows_A_product": r_op, "rows_smp_product": r_map,
        "sample_s": d_op + d_map,
        "extrapolated_to": f"{matvecs} A_product calls of {w.n} rows + smp_product of {w.n_map} rows",
    }


def dist_barrier():
    """Barrier over the ranks of the default process group (no-op without one)."""
    import torch.distributed as td

    if td.is_available() and td.is_initialized() and td.get_world_size() > 1:
        td.barrier()


def dist_max(v: float) -> float:
    """Maximum of v over the ranks (v itself without a process group): the
    whole job's step time is the slowest replica's."""
    import torch
    import torch.distributed as td

    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return v
    dev = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, world):
    """The reference arm: the reference's own algorithm for this path (its
    table-kernel A_product and smp_product, lib/wf_vector.cc:196-220 and
    lib/map.cc:20-43, via the bit-exact C/OpenMP restatement in oracle/) on
    all host cores.  A full solve of the workload takes tens of minutes on
    the host, so each step times a bounded sample of rows and extrapolates;
    the config says what was sampled and that the kernel is the table one
    (the GPU arm evaluates exp)."""
    if rank != 0:
        return
    w = workload(args.workload)
    iters = REF_ITERS[w.name]
    vals = []
    base = None
    for step in range(args.warmup + args.steps):
        base = cpu_baseline(w, iters, args.cpu_sample_s)
        if step >= args.warmup:
            vals.append(base["value"])
    value = statistics.mean(vals)
    base["value"] = value
    line = {
        "metric": METRIC, "value": value, "unit": "s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "n_pixels": w.n, "n_map": w.n_map,
                   "kernel": "table (the reference's A_product / smp_product kernel; "
                             "the GPU arm evaluates exp)",
                   "form": "W", "tol": w.pcg_tol, "iters": iters,
                   "sample": "bounded row sample per step, extrapolated to the full solve",
                   "sampled_rows": {"A_product": base["rows_A_product"],
                                    "smp_product": base["rows_smp_product"]},
                   "sampled_seconds": base["sample_s"],
                   "extrapolated_to": base["extrapolated_to"]},
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    emit(line)


def emit(line: dict):
    """Prints the result line on a line of its own: the library's C stdio
    buffer (its PCG warnings) is flushed first, so that nothing it still holds
    lands inside the JSON."""
    import ctypes

    sys.stdout.flush()
    try:
        ctypes.CDLL(None).fflush(None)
    except (OSError, AttributeError):
        pass
    print("\n" + json.dumps(line), flush=True)


def pipe_calibration(device: int):
    """Pair throughput of the FP32 FMA + MUFU pipes in the pair kernel's
    instruction mix, measured on this GPU now (bench_pipes.cu beside this
    file, compiled for sm_103a into _build/): the practical ceiling reported
    beside the FP32 pair kernel's nominal roofline.  None when it cannot be
    built or run."""
    src = os.path.join(ROOT, "bench_pipes.cu")
    exe = os.path.join(ROOT, "_build", "bench_pipes")
    try:
        os.makedirs(os.path.dirname(exe), exist_ok=True)
        if not (os.path.exists(exe) and os.path.getmtime(exe) >= os.path.getmtime(src)):
            nvcc = os.environ.get("NVCC") or "nvcc"
            subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                            src], check=True, capture_output=True, timeout=300)
        env = dict(os.environ, CUDA_VISIBLE_DEVICES=str(device))
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120,
                             env=env).stdout
        return json.loads(out.strip().splitlines()[-1])
    except (OSError, subprocess.SubprocessError, ValueError, IndexError):
        return None


def measured_peaks():
    """Measured HBM copy bandwidth and cuBLAS bf16 rate of this GPU model
    (MEASURED_PEAKS.json beside this file), if present."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def run_batched(ctx, n_chunks=512, n_rhs=64, seed=0, plain_samples=6):
    """Batched uneven chunks: n_chunks independent sub-volumes (16-192 skewers x
    64-128 pixels, box side 2.5 sqrt(n_skewers) Mpc/h, GRF signal), each with
    n_rhs noise realisations, solved together to 1e-8 per (chunk, RHS) by the
    batched mixed-precision solver (autotuned matvec variant), timed with CUDA
    events.  Beside it: plain FP64 GPU PCG (the exact-kernel single-operator
    solve) on a few sampled (chunk, RHS) systems, extrapolated to all of them
    by pixel count."""
    import numpy as np
    import torch

    from dachshund_gb300 import (BatchSolver, MixedParams, PCGParams, SignalCovarParams,
                                 WFVectorW, pixel_to_wpixel, synth)

    sp = SignalCovarParams(synth.VAR_S, synth.L_PERP, synth.L_PARA, eval="exact")
    pixes, rhs = synth.chunks(n_chunks, seed, n_rhs=n_rhs)
    noise = np.concatenate([p[:, 3] for p in pixes])
    recs = [pixel_to_wpixel(p) for p in pixes]
    b = np.ascontiguousarray(rhs / noise[:, None])
    t0 = time.perf_counter()
    bs = BatchSolver(ctx, "w", recs, sp, n_rhs=n_rhs)
    t_create = time.perf_counter() - t0
    bs.set_variant("auto")
    info = bs.info()
    bd = torch.tensor(b, device="cuda")
    xd = torch.zeros_like(bd)
    mp = MixedParams(max_iter=3000, tol=1e-8)
    bs.solve_mixed_dev(bd, xd, mp)  # warm-up
    launches0 = ctx.profile()["kernel_launches"]
    res = bs.solve_mixed_dev(bd, xd, mp)
    launches = ctx.profile()["kernel_launches"] - launches0
    loop_its = bs.info()["graph_replays"]
    ctx.set_profiling(True)
    resp = bs.solve_mixed_dev(bd, xd, mp)
    prof = ctx.profile()
    ctx.set_profiling(False)
    mv_ms = prof["f32_ms"] / max(prof["f32_launches"], 1)
    mv_flops = 2.0 * prof["f32_evaluated"] / (prof["f32_ms"] * 1e-3) if prof["f32_ms"] else None
    # end to end through the host API (records already in the batch; rhs in,
    # solutions and per-(chunk, RHS) results out)
    t0 = time.perf_counter()
    xh, reh = bs.solve_mixed(b, mp)
    e2e = time.perf_counter() - t0
    # plain FP64 GPU PCG on sampled (chunk, RHS) systems
    rng = np.random.default_rng(1)
    picks = rng.choice(n_chunks, size=plain_samples, replace=False)
    offs = bs.offsets
    t_sum, n_sum, it_sum, errs = 0.0, 0, 0, []
    for c in picks:
        r = int(rng.integers(n_rhs))
        rec = recs[c].copy()
        rec[:, 4] = b[offs[c]:offs[c + 1], r]
        op = WFVectorW(ctx, rec, sp)
        xp = torch.zeros(rec.shape[0], dtype=torch.float64, device="cuda")
        rp = op.solve_pcg_dev(PCGParams(3000, 50, 1e-8), xp)
        t_sum += rp.seconds
        n_sum += rec.shape[0]
        it_sum += rp.num_iters
        xb = xh[offs[c]:offs[c + 1], r]
        xpn = xp.cpu().numpy()
        errs.append(float(np.max(np.abs(xb - xpn)) / np.max(np.abs(xpn))))
        op.close()
    n_solves = n_chunks * n_rhs
    plain_est = t_sum / n_sum * bs.n_total * n_rhs
    bs.close()
    return {
        "workload": (f"{n_chunks} chunks x {n_rhs} RHS (16-192 skewers x 64-128 px, "
                     f"{bs.n_total} px, box side 2.5 sqrt(n_sk) Mpc/h, GRF + noise realisations)"),
        "solves": n_solves, "value": res.seconds, "unit": "s",
        "ms_per_solve": res.seconds / n_solves * 1e3,
        "create_s": t_create, "e2e_s": e2e,
        "e2e_h2d_bytes": int(b.nbytes), "e2e_d2h_bytes": int(xh.nbytes + reh.iters.nbytes * 4),
        "iters_max": int(res.iters.max()), "iters_mean": float(res.iters.mean()),
        "fp64_updates_max": int(res.n_updates.max()),
        "all_converged": bool(res.converged.all()),
        "max_rel_residual": float(res.rel_resid.max()),
        "variant": {0: "cuda_core", 1: "tensor (tcgen05 BF16 hi/lo)"}.get(info["variant"]),
        "matvec_ms": mv_ms, "matvec_algorithmic_tflops": mv_flops / 1e12 if mv_flops else None,
        "matvec_tensor_frac_of_bf16_peak": None,
        "fp64_residual_ms_per_solve": prof["f64_ms"],
        "kernel_launches_per_solve": launches,
        "graph_launches_per_solve": 1,
        "device_loop_iterations": loop_its,
        "host_loop": ("none: after the first iteration the solve is one graph launch, a "
                      "WHILE conditional node whose body is an iteration and a kernel that "
                      "continues while a chunk is active"),
        "plain_fp64": {"sampled_solves": plain_samples, "sample_s": t_sum,
                       "iters_mean": it_sum / plain_samples,
                       "extrapolated_s": plain_est, "basis": "sample time per pixel x all pixels x RHS"},
        "speedup_vs_plain": plain_est / res.seconds,
        "x_err_vs_plain_fp64_max": max(errs),
    }


def run_wf32768(ctx, hbm_gbs):
    """The 32,768-pixel workload (256 skewers x 128 pixels in [0,40)^2 x
    [0,256) Mpc/h, GRF data, exact kernel, W form, tol 1e-8, map 40 x 40 x
    256), solved four ways from x = 0: the plain FP64 PCG with the dense
    operator in HBM (32,768^2 FP64 = 8.6 GB, float-pair matvec), the plain
    FP64 PCG with the matrix-free FP64 kernel, the mixed-precision form with
    the pair kernels (+ FP32 map), and the chosen form (cluster factor,
    structured operator, structured FP64 map).  Device times from CUDA events; the dense matvec's
    achieved HBM bandwidth = 8 n_pad^2 bytes per product / its event time,
    against the measured copy bandwidth."""
    import numpy as np
    import torch

    from dachshund_gb300 import (MapGrid, MixedParams, PCGParams, SignalCovarParams,
                                 WFVectorW, pixel_to_wpixel, synth)

    w = synth.wf32768(0)
    rec = pixel_to_wpixel(w.pixels)
    sp = SignalCovarParams(w.var_s, w.l_perp, w.l_para, eval="exact")
    pts = synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny, w.map_nz)
    mf = WFVectorW(ctx, rec, sp)
    dn = WFVectorW(ctx, rec, sp)
    grid = MapGrid(ctx, pts)
    pp = PCGParams(3000, w.pcg_step_r, w.pcg_tol)
    n_pad = mf.info()["n_pad"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dn.set_dense(True)
    build_s = time.perf_counter() - t0
    out = {"workload": f"{w.name}: 256 skewers x 128 px, [0,40)^2 x [0,256) Mpc/h, exact kernel",
           "n_pixels": w.n, "n_pad": n_pad, "dense_bytes": 8 * n_pad * n_pad,
           "dense_build_s": build_s, "dense_arith": dn.dense_arith()}
    xd = torch.zeros(w.n, dtype=torch.float64, device="cuda")
    dn.solve_pcg_dev(pp, xd)  # warm-up
    for arith in ("float_pair", "fp64"):
        dn.set_dense_arith(arith)
        xd.zero_()
        ctx.set_profiling(True)
        rd = dn.solve_pcg_dev(pp, xd)
        prof = ctx.profile()
        ctx.set_profiling(False)
        mv_s = prof["dense_ms"] * 1e-3 / max(prof["dense_launches"], 1)
        gbs = 8.0 * n_pad * n_pad / mv_s / 1e9
        out[f"dense_{arith}"] = {
            "solve_s": rd.seconds, "iters": rd.num_iters, "success": rd.success,
            "matvecs": prof["dense_launches"], "matvec_ms": mv_s * 1e3,
            "matvec_GBps": gbs, "frac_of_measured_hbm": gbs / hbm_gbs if hbm_gbs else None}
    dn.set_dense_arith("auto")
    xd.zero_()
    rd = dn.solve_pcg_dev(pp, xd)
    xm = torch.zeros_like(xd)
    rm = mf.solve_pcg_dev(pp, xm)
    mref = torch.empty(w.n_map, dtype=torch.float64, device="cuda")
    grid.product_dev(mf, xm, mref)
    mp = MixedParams(max_iter=3000, tol=w.pcg_tol)
    xc = torch.zeros_like(xd)
    mf.solve_mixed_dev(mp, xc)  # warm-up
    mc = torch.empty_like(mref)
    times = []
    for _ in range(3):
        xc.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream = torch.cuda.ExternalStream(ctx.stream)
        e0.record(stream)
        rc = mf.solve_mixed_dev(mp, xc)
        grid.product_f32_dev(mf, xc, mc)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    # the chosen form: cluster factor, structured operator and structured map
    mf.set_cluster_preconditioner(w.n_skewers, w.pix_per_skewer, PC_CLUSTER, PC_BAND)
    mf.set_skewer_grid(w.n_skewers, w.pix_per_skewer)
    grid.set_column_grid(w.map_nx * w.map_ny, w.map_nz)
    xs = torch.zeros_like(xd)
    ms = torch.empty_like(mref)
    mf.solve_mixed_dev(mp, xs)  # warm-up
    grid.product_f32_dev(mf, xs, ms)
    ctimes = []
    for _ in range(3):
        xs.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream = torch.cuda.ExternalStream(ctx.stream)
        e0.record(stream)
        rs = mf.solve_mixed_dev(mp, xs)
        grid.product_f32_dev(mf, xs, ms)
        e1.record(stream)
        e1.synchronize()
        ctimes.append(e0.elapsed_time(e1) / 1e3)
    # FP64 residuals of the dense and mixed solutions with the matrix-free operator
    wv = torch.tensor(rec[:, 3], device="cuda")
    nb = float(np.linalg.norm(rec[:, 4]))
    r = torch.empty_like(xd)

    def rel_resid(x):
        mf.A_residual_dev(x / wv, r)
        return float(torch.linalg.norm(r).item()) / nb

    xmax = float(torch.max(torch.abs(xm)).item())
    out.update({
        "dense_solve_s": rd.seconds, "dense_iters": rd.num_iters,
        "dense_rel_residual_fp64": rel_resid(xd),
        "matrix_free_fp64_solve_s": rm.seconds, "matrix_free_fp64_iters": rm.num_iters,
        "mixed_solve_plus_map_s": statistics.mean(times), "mixed_iters": rc.num_iters,
        "mixed_fp64_updates": rc.n_outer, "mixed_rel_residual_fp64": rel_resid(xc),
        "x_dense_vs_matrix_free": float(torch.max(torch.abs(xd - xm)).item()) / xmax,
        "x_mixed_vs_matrix_free": float(torch.max(torch.abs(xc - xm)).item()) / xmax,
        "map_err_mixed_vs_fp64": float(torch.max(torch.abs(mc - mref)).item())
        / float(torch.max(torch.abs(mref)).item()),
        "speedup_dense_vs_matrix_free": rm.seconds / rd.seconds,
        "chosen_solve_plus_map_s": statistics.mean(ctimes), "chosen_iters": rs.num_iters,
        "chosen_fp64_updates": rs.n_outer, "chosen_rel_residual_fp64": rel_resid(xs),
        "x_chosen_vs_matrix_free": float(torch.max(torch.abs(xs - xm)).item()) / xmax,
        "map_err_chosen_vs_fp64": float(torch.max(torch.abs(ms - mref)).item())
        / float(torch.max(torch.abs(mref)).item()),
        "chosen_form": "cluster FSAI factor (4 skewers, band 16), structured operator and map",
    })
    grid.close()
    dn.close()
    mf.close()
    return out


def run_wf4096(ctx):
    """The reference's own CPU-runnable configuration, run whole on both sides
    (no extrapolation): 4,096 pixels (64 skewers x 64 in [0,32)^2 x [0,128)
    Mpc/h, dense-Cholesky data), the reference's app path (W form, table
    kernel, PCG to 1e-5, at most 200 iterations, step_r 50) + the FP64 map on
    the 32 x 32 x 128 grid.  GPU: the plain FP64 path through the library
    (host buffers in and out, the operator and map grid created in the timed
    region).  CPU baseline leg: the oracle port of the reference (bit-exact
    with it) on all host threads, the same solve and map."""
    import numpy as np

    import oracle
    from dachshund_gb300 import (MapGrid, PCGParams, SignalCovarParams, WFVectorW,
                                 pixel_to_wpixel, synth)

    w = synth.wf4096(0)
    rec = pixel_to_wpixel(w.pixels)
    sp = SignalCovarParams(w.var_s, w.l_perp, w.l_para)  # table kernel
    pts = synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny, w.map_nz)
    pp = PCGParams(w.pcg_max_iter, w.pcg_step_r, w.pcg_tol)
    times = []
    for k in range(4):
        ctx.synchronize()
        t0 = time.perf_counter()
        op = WFVectorW(ctx, rec, sp)
        x, res = op.solve_pcg(pp)
        grid = MapGrid(ctx, pts)
        m = grid.product(op, x)
        if k:
            times.append(time.perf_counter() - t0)
        grid.close()
        op.close()
    t0 = time.perf_counter()
    xo, ok, it_o, _ = oracle.solve_pcg("w", rec, w.var_s, w.l_perp, w.l_para, w.pcg_max_iter,
                                       w.pcg_step_r, w.pcg_tol)
    mo = oracle.smp_product(w.pixels[:, :3], pts, xo, w.var_s, w.l_perp, w.l_para)
    cpu_s = time.perf_counter() - t0
    gpu_s = statistics.mean(times)
    return {"workload": f"{w.name}: the reference's app path (W form, table kernel, tol "
                        f"{w.pcg_tol}, step_r {w.pcg_step_r}) + FP64 map 32 x 32 x 128",
            "gpu_s": gpu_s, "gpu_iters": res.num_iters, "gpu_success": res.success,
            "cpu_s": cpu_s, "cpu_iters": int(it_o), "cpu_cores": os.cpu_count(),
            "cpu_kind": "port (C/OpenMP restatement, bit-exact with the reference)",
            "speedup_vs_cpu": cpu_s / gpu_s,
            "map_err_vs_cpu": float(np.max(np.abs(m - mo)) / np.max(np.abs(mo)))}


def run_map_covar(ctx, n_points=256):
    """MapCovarDiag (lib/map_covar.cc:73-113) on the 4,096-pixel workload
    (64 skewers x 64 pixels, tol 1e-5 as its app run, step_r 50) for
    n_points map-grid points: the reference's table kernel (multi-RHS FP64
    PCG, 16 points per solve) and the exact kernel (batched mixed precision,
    64 points per solve); wall time per map point and the iteration counts."""
    import numpy as np

    from dachshund_gb300 import PCGParams, SignalCovarParams, map_covar_diag, pixel_to_npixel, synth

    w = synth.wf4096(0)
    nrec = pixel_to_npixel(w.pixels)
    pts = synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny, w.map_nz)
    pts = pts[np.linspace(0, pts.shape[0] - 1, n_points).astype(int)]
    pp = PCGParams(w.pcg_max_iter, w.pcg_step_r, w.pcg_tol)
    out = {"workload": f"{w.name}, {n_points} map-grid points, tol {w.pcg_tol}"}
    for ev in ("table", "exact"):
        sp = SignalCovarParams(w.var_s, w.l_perp, w.l_para, eval=ev)
        map_covar_diag(ctx, nrec, pts[:16], sp, pp)  # warm-up
        t0 = time.perf_counter()
        sig, iters, ok = map_covar_diag(ctx, nrec, pts, sp, pp)
        dt = time.perf_counter() - t0
        out[ev] = {"s": dt, "ms_per_point": dt / n_points * 1e3,
                   "iters_mean": float(np.mean(iters[ok])) if ok.any() else None,
                   "success": int(ok.sum())}
    return out


def run_learned(ctx, seeds=(10001, 10002, 10003, 10004, 10005)):
    """Learned warm start + skewer-band preconditioner on held-out systems of
    the 262,144-pixel geometry (seeds outside the 1-2000 training range),
    against Jacobi, both with the mixed-precision PCG to 1e-8; wall time of
    the learned form includes the network's forward pass."""
    import numpy as np

    from dachshund_gb300 import SignalCovarParams, synth
    from dachshund_gb300.learned import LearnedPreconditioner, compare

    path = os.path.join(ROOT, "dachshund_gb300", "weights", "learned_wf262144.bin")
    if not os.path.exists(path):
        return None
    sp = SignalCovarParams(synth.VAR_S, synth.L_PERP, synth.L_PARA, eval="exact")
    net = LearnedPreconditioner(ctx, sp, hidden=128, band=2)
    net.load(path)
    compare(net, ctx, sp, seeds[:1])  # warm-up
    rows = compare(net, ctx, sp, seeds)
    net.close()
    mean = lambda k: float(np.mean([r[k] for r in rows]))  # noqa: E731
    return {
        "workload": "262,144 px (1,024 skewers x 256), GRF systems generated on the GPU, "
                    f"held-out seeds {seeds[0]}-{seeds[-1]}; network trained on seeds 1-2000",
        "jacobi_iters": mean("jacobi_iters"), "learned_iters": mean("learned_iters"),
        "jacobi_s": mean("jacobi_s"), "learned_s": mean("learned_s"),
        "network_forward_s": mean("net_s"),
        "iters_ratio": mean("learned_iters") / mean("jacobi_iters"),
        "time_ratio": mean("learned_s") / mean("jacobi_s"),
        "warm_start_rel_err": mean("x0_rel_err"),
        "fallbacks": int(sum(r["fallback"] for r in rows)),
        "max_rel_residual": float(max(r["learned_rel_resid"] for r in rows)),
    }


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    from dachshund_gb300 import (Context, MapGrid, MixedParams, PCGParams, SignalCovarParams,
                                 WFVectorW, pixel_to_wpixel, synth)

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))

    barrier = dist_barrier
    allmax = dist_max

    w = workload(args.workload)
    ctx = Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    sp = SignalCovarParams(w.var_s, w.l_perp, w.l_para, eval="exact")
    rec = pixel_to_wpixel(w.pixels)
    pts = synth.uniform_map_coords(w.lx, w.ly, w.lz, w.map_nx, w.map_ny, w.map_nz)
    op = WFVectorW(ctx, rec, sp)
    # Jacobi-preconditioned mixed solve of the same system, once, for the
    # iteration counts and time the cluster preconditioner is measured against
    mp = MixedParams(max_iter=3000, tol=w.pcg_tol)
    xj = torch.zeros(w.n, dtype=torch.float64, device="cuda")
    op.solve_mixed_dev(mp, xj)
    torch.cuda.synchronize()
    rj = op.solve_mixed_dev(mp, xj.zero_())
    jacobi = {"iters": rj.num_iters, "solve_s": rj.seconds, "fp64_updates": rj.n_outer}
    # the chosen form's preconditioner: FSAI over clusters of 4 neighbouring
    # skewers, built once per pixel set like the operator's tiling
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_fb = op.set_cluster_preconditioner(w.n_skewers, w.pix_per_skewer, PC_CLUSTER, PC_BAND)
    pc_info = {"kind": f"FSAI over clusters of {PC_CLUSTER} neighbouring skewers, band {PC_BAND}",
               "build_s": time.perf_counter() - t0, "jacobi_fallback_columns": n_fb}
    # and the FP64-accurate outer residual by the structured operator
    # (skewers on one z grid: perpendicular factor x Toeplitz z taps)
    t0 = time.perf_counter()
    op.set_skewer_grid(w.n_skewers, w.pix_per_skewer)
    pc_info["skewer_grid_build_s"] = time.perf_counter() - t0
    del xj
    grid = MapGrid(ctx, pts)
    # the map points are the uniform column grid: the structured FP64 map
    grid.set_column_grid(w.map_nx * w.map_ny, w.map_nz)
    x = torch.zeros(w.n, dtype=torch.float64, device="cuda")
    m = torch.empty(w.n_map, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def step():
        with torch.cuda.stream(stream):
            x.zero_()
        res = op.solve_mixed_dev(mp, x)
        grid.product_f32_dev(op, x, m)
        return res

    for _ in range(args.warmup):
        step()
    ctx.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    times, results, parts = [], [], []
    op.persistent_profile(reset=True)  # the phase timers of the timed steps only
    launches0 = ctx.profile()["kernel_launches"]
    clocks.mark_start()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        ctx.synchronize()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        em = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        with torch.cuda.stream(stream):
            x.zero_()
        res = op.solve_mixed_dev(mp, x)
        em.record(stream)
        grid.product_f32_dev(op, x, m)
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        barrier()
        times.append(e0.elapsed_time(e1) / 1e3)
        parts.append((e0.elapsed_time(em) / 1e3, em.elapsed_time(e1) / 1e3, res.seconds))
        results.append(res)
    clocks.mark_end()
    launches = (ctx.profile()["kernel_launches"] - launches0) / args.steps
    clk = clocks.stop()
    step_s = allmax(statistics.mean(times))
    phases = op.persistent_profile(reset=True)
    # the step's two calls (CUDA events between them) and the solve's own
    # device time (the library's events around its launches)
    step_parts = {"solve": statistics.mean(p[0] for p in parts),
                  "map": statistics.mean(p[1] for p in parts),
                  "solve_device": statistics.mean(p[2] for p in parts)}

    # One more step, untimed, with CUDA events around every pair-kernel launch
    # (the per-kernel times below; the events and the uncaptured launches make
    # this step slower than the timed ones).
    with torch.cuda.stream(stream):
        flush.zero_()
    ctx.synchronize()
    ctx.set_profiling(True)
    with torch.cuda.stream(stream):
        x.zero_()
    op.solve_mixed_dev(mp, x)
    grid.product_f32_dev(op, x, m)
    ctx.synchronize()
    prof = ctx.profile()
    ctx.set_profiling(False)
    solve_prof, map_prof = [prof], [prof]
    prof_steps = 1

    # Kernel rooflines (CUDA events around every pair-kernel launch).
    sm_hz = (clk["sm_mhz"] or 1900.0) * 1e6

    def agg(profs, key):
        return sum(p[key] for p in profs)

    f32_ms = agg(solve_prof, "f32_ms")
    f32_pairs = agg(solve_prof, "f32_evaluated")
    f32_n = agg(solve_prof, "f32_launches")
    f64_ms = agg(solve_prof, "f64_ms")
    f64_pairs = agg(solve_prof, "f64_evaluated")
    f64_n = agg(solve_prof, "f64_launches")
    map_ms = agg(map_prof, "map_ms")
    map_pairs = agg(map_prof, "map_evaluated")
    # Bytes one structured FP32 inner product must move at least (HBM
    # roofline): per pixel p (4) and wr (8) in, the z-convolved column values
    # written once per level and read back once (2 x 4 (lmax + 1)), wl and e
    # (8 + 8), q out (4); per neighbour entry 16 (index, level, factor, pointer
    # share).  lmax: the z taps within the inner cutoff.
    c_para = 1.0 / (2 * w.l_para ** 2)
    lmax = 0
    while lmax + 1 < w.pix_per_skewer and c_para * ((lmax + 1) * synth.DZ) ** 2 < SG_INNER_CUT:
        lmax += 1
    terms_per_product = (f32_pairs / f32_n) if f32_n else 0.0
    sg_bytes = w.n * (4 + 8 + 8 * (lmax + 1) + 8 + 8 + 4) + 16 * terms_per_product / w.pix_per_skewer
    sg_us = (f32_ms / f32_n * 1e3) if f32_n else None
    kernels = {
        "fp32_inner_product": {
            "kernel": "structured FP32 inner product (k_sg32_levels + k_sg32_apply)",
            "launches_per_step": f32_n / prof_steps, "ms_per_step": f32_ms / prof_steps,
            "us_per_product": sg_us,
            "terms_per_product": terms_per_product,
            "term": "one FP32 FMA of a (skewer pair, pixel): perpendicular factor x "
                    "z-convolved column value",
            "algorithmic_bytes_per_product": sg_bytes},
        "fp64_outer_residual": {
            "kernel": "structured FP64 outer residual (k_sg_levels + k_sg_apply)",
            "launches_per_step": f64_n / prof_steps, "ms_per_step": f64_ms / prof_steps,
            "Gterm_per_s": f64_pairs / (f64_ms * 1e-3) / 1e9 if f64_ms else None,
            "term": "one FP64 FMA of a (skewer pair, pixel): perpendicular factor x "
                    "z-convolved column value"},
        "map": {
            "kernel": "structured map, fused float-pair form (k_mc_split + k_mc_fused)",
            "ms_per_step": map_ms / prof_steps,
            "Gterm_per_s": map_pairs / (map_ms * 1e-3) / 1e9 if map_ms else None,
            "term": "one (map column, skewer, map z) triple of the FP64 form (the fused form "
                    "does 256 float-pair multiply-adds per (column, skewer) pair instead of 512 "
                    "FP64 FMAs)"},
    }
    hbm = measured_peaks().get("hbm_gbs")
    # The timed step's dominant kernel is the persistent solve (one cooperative
    # launch per solve, ~89% of the step: profiles/launch_list_wf262144_chosen.md).
    # Its algorithmic bytes per launch: the start loads each block's state
    # into shared memory (x 8, p z r 4 each, wl wr e 8 each per pixel; the
    # FSAI planes 4 (band + 1) per slot, the slot map 4; the inner lists 12
    # per entry), every iteration writes the z-convolution levels of z once
    # and reads them back once (2 x 4 (lmax + 1) per pixel), every FP64 update
    # does the same for the float-pair levels of x (2 x 8 (lmax64 + 1)) and
    # reads wl wr e b as float pairs (32) and the outer lists (16 per entry),
    # and the end writes x (8).  The clusters re-read the neighbours' levels
    # from L2 every iteration (each distinct (neighbour, level) row of a
    # cluster once): that traffic and the barriers, not HBM, bound it.
    c_para = 1.0 / (2 * w.l_para ** 2)
    lmax64 = 0
    while lmax64 + 1 < w.pix_per_skewer and \
            c_para * ((lmax64 + 1) * synth.DZ) ** 2 < 40.0:  # DS_DEFAULT_EXACT_CUTOFF
        lmax64 += 1
    r_last = results[-1]
    n_it, n_up = r_last.num_iters, r_last.n_outer
    entries_in = terms_per_product / w.pix_per_skewer
    entries_out = (f64_pairs / f64_n / w.pix_per_skewer) if f64_n else entries_in
    persist_bytes = (w.n * (8 + 12 + 24 + 4 * (PC_BAND + 1) + 4 + 8) + 12 * entries_in
                     + n_it * w.n * 2 * 4 * (lmax + 1)
                     + n_up * (w.n * (2 * 8 * (lmax64 + 1) + 32) + 16 * entries_out))
    persist_us = (phases["kernel_ms"] / phases["launches"] * 1e3) \
        if phases and phases["launches"] else None
    persist_gbs = persist_bytes / (persist_us * 1e-6) / 1e9 if persist_us else None
    # the neighbours' level values one product loads from L2: each distinct
    # (neighbour, level) row of a cluster once (the resident form's items)
    loads = (phases or {}).get("product_loads") or terms_per_product
    l2_reads = n_it * loads * 4
    roofline = {
        "kernel": "persistent structured mixed solve (k_mixed_resident<16>), the dominant "
                  "kernel of the chosen form's step",
        "bound": "hbm", "unit": "GB/s",
        "achieved": persist_gbs, "peak": hbm,
        "frac": (persist_gbs / hbm) if (persist_gbs and hbm) else None,
        "peak_basis": "MEASURED_PEAKS.json hbm_gbs (of measured)",
        "algorithmic_bytes_per_launch": persist_bytes,
        "launch_us": persist_us,
        "iterations_per_launch": n_it, "fp64_updates_per_launch": n_up,
        # DRAM bytes (read + write) of one launch, from one ncu capture of this
        # workload (profiles/k_mixed_resident_wf262144.md); the state stays in
        # shared memory and L2 for the whole solve
        "traffic": K_PERSIST_DRAM_BYTES,
        "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
        "l2_neighbour_reads_per_launch": l2_reads,
        "neighbour_values_per_product": loads,
        "skewer_pair_terms_per_product": terms_per_product,
        "l2_neighbour_read_GBps": l2_reads / (persist_us * 1e-6) / 1e9 if persist_us else None,
    }

    # Plain FP64 GPU PCG on the same system (once, untimed by the step loop).
    plain = None
    r0 = results[-1]
    m_chosen = m.cpu().numpy()
    if not args.no_plain:
        xp = torch.zeros_like(x)
        mpl = torch.empty_like(m)
        torch.cuda.synchronize()
        ctx.set_profiling(True)
        rp = op.solve_pcg_dev(PCGParams(3000, w.pcg_step_r, w.pcg_tol), xp)
        pprof = ctx.profile()
        ctx.set_profiling(False)
        p_gps = pprof["f64_evaluated"] / (pprof["f64_ms"] * 1e-3) if pprof["f64_ms"] else None
        p_peak = DFMA_RATE / K_PAIR_F64_EXACT_OPS * SMS * sm_hz
        kernels["fp64_plain_matvec"] = {
            "kernel": "k_pair_f64<EXACT> (plain FP64 PCG products and residuals)",
            "launches_per_solve": pprof["f64_launches"],
            "ms_per_launch": pprof["f64_ms"] / max(pprof["f64_launches"], 1),
            "Gpair_per_s": p_gps / 1e9 if p_gps else None,
            "fp64_ops_per_pair": K_PAIR_F64_EXACT_OPS,
            "peak_Gpair_per_s": p_peak / 1e9,
            "frac": p_gps / p_peak if p_gps else None,
            "peak_basis": (f"FP64 pipe: {DFMA_RATE:.0f} FP64 instructions/clk/SM x {SMS} SMs "
                           f"x median SM clock / {K_PAIR_F64_EXACT_OPS} FP64 instructions per "
                           "evaluated pair (ncu capture)")}
        t0 = time.perf_counter()
        grid.product_dev(op, xp, mpl)
        ctx.synchronize()
        t_map = time.perf_counter() - t0
        mref = mpl.cpu().numpy()
        plain = {"solve_s": rp.seconds, "map_s": t_map, "total_s": rp.seconds + t_map,
                 "iters": rp.num_iters, "success": rp.success}
        map_err = float(np.max(np.abs(m_chosen - mref)) / np.max(np.abs(mref)))
        x_err = float(torch.max(torch.abs(x - xp)).item() / torch.max(torch.abs(xp)).item())

    # The same solve with the matrix-free pair kernels instead of the
    # structured operator (FP32 k_pair_f32 inner products, float-float outer
    # residuals; same cluster preconditioner): the general path for pixels on
    # no shared z grid, and the FP32 FMA/MUFU roofline of its pair kernel.
    pair_form = None
    if not args.no_pair_form:
        op.set_skewer_grid(0, 0)
        xq = torch.zeros_like(x)
        op.solve_mixed_dev(mp, xq)
        rq = None
        for _ in range(3):
            xq.zero_()
            torch.cuda.synchronize()
            r_ = op.solve_mixed_dev(mp, xq)
            rq = r_ if (rq is None or r_.seconds < rq.seconds) else rq
        xq.zero_()
        torch.cuda.synchronize()
        ctx.set_profiling(True)
        op.solve_mixed_dev(mp, xq)
        pq = ctx.profile()
        ctx.set_profiling(False)
        op.set_skewer_grid(w.n_skewers, w.pix_per_skewer)
        gps = pq["f32_evaluated"] / (pq["f32_ms"] * 1e-3) / 1e9 if pq["f32_ms"] else None
        peak = PAIRS_PER_CLK["expanded"] * SMS * sm_hz / 1e9
        cal = pipe_calibration(local) if rank == 0 else None
        mix = None
        if cal and cal.get("mix_pairs_per_s") and gps:
            mix = {
                "Gpair_per_s": cal["mix_pairs_per_s"] / 1e9,
                "pairs_per_clk_per_sm": cal["mix_pairs_per_s"] / (SMS * sm_hz),
                "ex2_per_clk_per_sm": cal["ex2_per_s"] / (SMS * sm_hz),
                "ffma_lanes_per_clk_per_sm": cal["ffma_lanes_per_s"] / (SMS * sm_hz),
                "frac": gps * 1e9 / cal["mix_pairs_per_s"],
                "basis": ("bench_pipes.cu in this run: 3 FFMA2 + 2 ex2 + 1 FFMA2 per two pairs "
                          "in independent chains, no memory traffic, best of 20-64 warps/SM and "
                          "1-8 chains per thread, at the sampled SM clock")}
        pair_form = {
            "solve_s": rq.seconds, "iters": rq.num_iters, "fp64_updates": rq.n_outer,
            "success": rq.success,
            "x_err_vs_structured": float(torch.max(torch.abs(xq - x)).item()
                                         / torch.max(torch.abs(x)).item()),
            "roofline": {
                "kernel": "k_pair_f32 (FP32 matrix-free inner matvec, exact kernel, MUFU ex2)",
                "bound": "fp32-fma+mufu", "unit": "Gpair/s", "achieved": gps, "peak": peak,
                "frac": gps / peak if gps else None,
                "peak_basis": (f"{PAIRS_PER_CLK['expanded']:.0f} pairs/clk/SM (FMA 128 lanes and "
                               f"ex2 32 per clk per SM, nominal; each measured alone within 7%) "
                               f"x {SMS} SMs x median SM clock under load"),
                "launches": pq["f32_launches"],
                "ms_per_launch": pq["f32_ms"] / max(pq["f32_launches"], 1),
                "measured_mix_ceiling": mix,
                "traffic": K_PAIR_F32_DRAM_BYTES,
                "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + "
                                "dram__bytes_write.sum)"},
            "ff_residual_ms": pq["f64_ms"],
        }

    # End to end through the public API with host buffers: the records and the
    # map points sit in pinned (page-locked) host memory, numpy views of
    # pinned tensors that the binding passes to the C ABI without a copy.
    rec_pin_t = torch.from_numpy(rec).pin_memory()
    pts_pin_t = torch.from_numpy(pts).pin_memory()
    rec_pin, pts_pin = rec_pin_t.numpy(), pts_pin_t.numpy()
    e2e_times = []
    h2d = rec.nbytes + w.n * 8 + pts.nbytes
    d2h = w.n * 8 + w.n_map * 8
    E2E_WARMUP = 2  # untimed passes: the memory pool grows to its working size
    for k in range(E2E_WARMUP + min(args.steps, 3)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op_h = WFVectorW(ctx, rec_pin, sp)
        op_h.set_cluster_preconditioner(w.n_skewers, w.pix_per_skewer, PC_CLUSTER, PC_BAND)
        op_h.set_skewer_grid(w.n_skewers, w.pix_per_skewer)
        xh, rh = op_h.solve_mixed(mp)
        grid_h = MapGrid(ctx, pts_pin)
        grid_h.set_column_grid(w.map_nx * w.map_ny, w.map_nz)
        mh = grid_h.product_f32(op_h, xh)
        if k >= E2E_WARMUP:
            e2e_times.append(time.perf_counter() - t0)
        grid_h.close()
        op_h.close()
    e2e = allmax(statistics.mean(e2e_times))

    base = cpu_baseline(w, plain["iters"] if plain else REF_ITERS[w.name], args.cpu_sample_s) \
        if rank == 0 else None
    batched = None if args.no_batched else run_batched(ctx)
    learned = None if args.no_learned else run_learned(ctx)
    wf32768 = None if args.no_wf32768 else run_wf32768(ctx, measured_peaks().get("hbm_gbs"))
    map_covar = None if args.no_map_covar else run_map_covar(ctx)
    wf4096 = None if (args.no_wf4096 or rank != 0) else run_wf4096(ctx)
    if batched and batched["matvec_algorithmic_tflops"] and batched["variant"].startswith("tensor"):
        peak = measured_peaks().get("bf16_tflops")
        if peak:
            # three BF16 MMAs (hi/lo split) per algorithmic multiply-add
            batched["matvec_tensor_frac_of_bf16_peak"] = \
                3 * batched["matvec_algorithmic_tflops"] / peak

    if rank == 0:
        line = {
            "metric": METRIC, "value": step_s, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 inner / f64 outer",
            "data": "synthetic (seeded GRF skewers of the workload's shapes)",
            "config": {"workload": w.name, "n_pixels": w.n, "n_map": w.n_map,
                       "kernel": "exact (var_s 0.0625, l_perp 2.5, l_para 2.0)", "form": "W",
                       "tol": w.pcg_tol, "parallelism": f"replicas x{world}",
                       "l2": "flushed between steps (256 MiB write)"},
            "cg_iters": r0.num_iters, "fp64_updates": r0.n_outer,
            "step_parts_s": step_parts,
            "persistent_phases": phases,
            "preconditioner": pc_info,
            "jacobi_mixed": jacobi,
            "final_rel_residual": r0.final_norm / r0.norm_b,
            "plain_fp64": plain,
            "speedup_vs_plain": (plain["total_s"] / step_s) if plain else None,
            "map_err_vs_fp64": map_err if plain else None,
            "x_err_vs_fp64": x_err if plain else None,
            "roofline": roofline,
            "pair_kernel_form": pair_form,
            "kernels": kernels,
            "cpu_baseline": base,
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "host_inputs": "pinned (records, map points)",
                    "steps_s": [round(t, 5) for t in e2e_times]},
            "gpu_launches": launches,
            "clocks": clk,
            "batched_chunks": batched,
            "learned_preconditioner": learned,
            "wf32768_dense_and_matrix_free": wf32768,
            "map_covar_diag": map_covar,
            "wf4096_app_path": wf4096,
        }
        emit(line)
    if world > 1:
        import torch.distributed as td

        td.destroy_process_group()


def main():
    args = parse()
    rank, world, local = dist()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
