"""GPU tests of the learned warm start + skewer-band preconditioner: the
hand-written forward / backward kernels against the CPU oracle
(oracle/learned_ref.py), the preconditioned mixed solve, and what a trained
network gains over Jacobi-PCG on held-out systems."""
import numpy as np
import pytest

from oracle import learned_ref as lr
from dachshund_gb300 import MixedParams, SignalCovarParams, WFVectorW, synth
from dachshund_gb300.learned import (LearnedPreconditioner, compare, gpu_system,
                                     set_skewer_preconditioner, solve_reference, train)

pytestmark = pytest.mark.gpu

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA
C_PERP, C_PARA = 1 / (2 * LP ** 2), 1 / (2 * LQ ** 2)
EXACT = SignalCovarParams(VS, LP, LQ, eval="exact")


def slot_views(flat, H, B):
    out, off = {}, 0
    for name, r, c in lr.layout(H, B):
        out[name] = flat[off:off + r * c]
        off += r * c
    return out


@pytest.mark.parametrize("H,B", [(32, 2), (64, 2)])
def test_loss_and_gradients_vs_oracle(ctx, H, B):
    import torch

    n_sk, n_per = 12, 16
    rec = gpu_system(3, n_sk, n_per, box=2.5 * np.sqrt(n_sk))
    rec_h = rec.cpu().numpy()
    rng = np.random.default_rng(5)
    ystar = 0.05 * rng.standard_normal(n_sk * n_per)
    probe = rng.standard_normal(n_sk * n_per).astype(np.float32)
    net = LearnedPreconditioner(ctx, EXACT, hidden=H, band=B, seed=7)
    flat = net.get_params().astype(np.float64)
    flat += 0.05 * rng.standard_normal(flat.size)  # nonzero biases too
    net.set_params(flat.astype(np.float32))
    flat = net.get_params().astype(np.float64)
    losses = net.train_step_dev(n_sk, n_per, rec, torch.tensor(ystar, device="cuda"),
                                torch.tensor(probe, device="cuda"), update=False)
    g_gpu = net.get_grads().astype(np.float64)
    (lx, lp), g_ref, Y = lr.loss_and_grad(flat, rec_h, ystar, probe, n_sk, n_per, H, B, VS,
                                          C_PERP, C_PARA)
    assert abs(losses[0] - lx) <= 1e-4 * lx and abs(losses[1] - lp) <= 1e-4 * lp
    gg, gr = slot_views(g_gpu, H, B), slot_views(g_ref, H, B)
    for name in gr:
        err = np.linalg.norm(gg[name] - gr[name]) / max(np.linalg.norm(gr[name]), 1e-30)
        assert err < 2e-3, (name, err)
    # forward outputs
    y0, L = net.forward_dev(n_sk, n_per, rec)
    Lb = lr.band_L(Y, rec_h, n_sk, n_per, B, VS).reshape(-1, B + 1)
    assert np.max(np.abs(y0.cpu().numpy() - lr.XS * Y[:, 0])) <= 1e-4 * np.max(np.abs(lr.XS * Y[:, 0]))
    assert np.max(np.abs(L.cpu().numpy().reshape(-1, B + 1) - Lb)) <= 1e-4 * np.max(np.abs(Lb))
    net.close()


def test_preconditioned_solve_and_weight_file(ctx, tmp_path):
    import torch

    n_sk, n_per = 36, 32
    rec = gpu_system(11, n_sk, n_per, box=2.5 * np.sqrt(n_sk))
    op, y_ref, res_ref = solve_reference(ctx, rec, EXACT)
    net = LearnedPreconditioner(ctx, EXACT, hidden=32, band=2, seed=1)
    y0, L = net.forward_dev(n_sk, n_per, rec)
    set_skewer_preconditioner(op, n_sk, n_per, 2, L)
    x = y0.clone()
    torch.cuda.synchronize()
    res = op.solve_mixed_dev(MixedParams(tol=1e-8), x)
    assert res.success and res.final_norm <= 1e-8 * res.norm_b
    y = (x / rec[:, 3]).cpu().numpy()
    r = op.A_residual(y)
    assert np.linalg.norm(r) <= 1e-8 * res.norm_b * (1 + 1e-6)
    assert np.max(np.abs(x.cpu().numpy() - (y_ref * rec[:, 3]).cpu().numpy())) <= \
        1e-6 * float(torch.max(torch.abs(y_ref * rec[:, 3])))
    # host L, identity band (L = I: plain CG) also converges; removal restores Jacobi
    Lid = np.zeros((n_sk * n_per, 4), dtype=np.float32)
    Lid[:, 0] = 1.0
    set_skewer_preconditioner(op, n_sk, n_per, 3, Lid)
    xi = torch.zeros_like(x)
    torch.cuda.synchronize()
    assert op.solve_mixed_dev(MixedParams(tol=1e-8, max_iter=4000), xi).success
    set_skewer_preconditioner(op, n_sk, n_per, 3, None)
    xj = torch.zeros_like(x)
    torch.cuda.synchronize()
    rj = op.solve_mixed_dev(MixedParams(tol=1e-8), xj)
    assert rj.num_iters == res_ref.num_iters
    # weight file round trip
    path = tmp_path / "w.bin"
    net.save(path)
    net2 = LearnedPreconditioner(ctx, EXACT, hidden=32, band=2, seed=99)
    net2.load(path)
    assert np.array_equal(net.get_params(), net2.get_params())
    net3 = LearnedPreconditioner(ctx, EXACT, hidden=64, band=2, seed=99)
    from dachshund_gb300 import DsError
    with pytest.raises(DsError):
        net3.load(path)
    op.close()


def test_trained_network_beats_jacobi(ctx):
    """Train on 400 small systems (64 skewers x 64 pixels at the workload's
    skewer density), then on 4 held-out systems the learned form (warm start
    + skewer-band preconditioner) must need at most 0.85x the CG iterations of
    Jacobi and reach the same FP64 residual and solution."""
    n_sk, n_per, box = 64, 64, 20.0
    net = LearnedPreconditioner(ctx, EXACT, hidden=64, band=2, seed=0)
    hist = train(net, ctx, EXACT, range(1, 401), n_sk, n_per, box, lr=1e-3, log=None)
    assert hist[-20:, 0].mean() < 0.5 * hist[:5, 0].mean()
    assert hist[-20:, 1].mean() < 0.5 * hist[:5, 1].mean()
    rows = compare(net, ctx, EXACT, range(10001, 10005), n_sk, n_per, box)
    for r in rows:
        assert not r["fallback"] and r["learned_rel_resid"] <= 1e-8
        assert r["x_diff"] < 1e-6
    assert sum(r["learned_iters"] for r in rows) <= 0.85 * sum(r["jacobi_iters"] for r in rows)


def test_tensor_core_inference_matches_cuda_core(ctx):
    """The trained network (H = 128) with its message-passing layers on the
    tensor cores (TF32 activations) against the FP32 CUDA-core forward pass:
    warm start and L within 2e-2 relative, and the preconditioned solve
    reaches 1e-8 in at most 5% more iterations."""
    import os

    import torch

    path = os.path.join(os.path.dirname(__file__), "..", "dachshund_gb300", "weights",
                        "learned_wf262144.bin")
    net = LearnedPreconditioner(ctx, EXACT, hidden=128, band=2)
    net.load(path)
    n_sk, n_per = 128, 256
    rec = gpu_system(10001, n_sk, n_per, 80.0 * (128 / 1024) ** 0.5)
    net.set_inference(False)
    y_c, L_c = net.forward_dev(n_sk, n_per, rec)
    y_c, L_c = y_c.clone(), L_c.clone()
    net.set_inference(True)
    y_t, L_t = net.forward_dev(n_sk, n_per, rec)
    rel = lambda a, b: float(torch.max(torch.abs(a - b)) / torch.max(torch.abs(b)))  # noqa: E731
    assert rel(y_t, y_c) < 2e-2 and rel(L_t, L_c) < 2e-2
    op = WFVectorW(ctx, rec.cpu().numpy(), EXACT)
    iters = []
    for y0, L in ((y_c, L_c), (y_t, L_t)):
        set_skewer_preconditioner(op, n_sk, n_per, 2, L)
        x = y0.clone()
        r = op.solve_mixed_dev(MixedParams(max_iter=3000, tol=1e-8), x)
        assert r.success and r.final_norm <= 1e-8 * r.norm_b * (1 + 1e-6)
        iters.append(r.num_iters)
    set_skewer_preconditioner(op, n_sk, n_per, 2, None)
    assert iters[1] <= 1.05 * iters[0] + 2
    op.close()
    net.close()
