"""CPU checks of the learned network's oracle (oracle/learned_ref.py): its
hand-written backward pass against central finite differences of its forward
pass (float64, exact weights), and the BF16 rounding it applies to the
forward weights."""
import numpy as np

from oracle import learned_ref as lr

VAR_S, C_PERP, C_PARA = 0.0625, 1 / (2 * 2.5 ** 2), 1 / (2 * 2.0 ** 2)


def small_system(n_sk=10, n_per=8, seed=0):
    rng = np.random.default_rng(seed)
    xy = rng.uniform(0, 6.0, size=(n_sk, 2))
    rec = np.empty((n_sk * n_per, 5))
    rec[:, 0] = np.repeat(xy[:, 0], n_per)
    rec[:, 1] = np.repeat(xy[:, 1], n_per)
    rec[:, 2] = np.tile((np.arange(n_per) + 0.5) * 2.0, n_sk)
    noise = rng.uniform(0.05, 0.3, size=n_sk * n_per)
    rec[:, 3] = 1 / noise
    rec[:, 4] = rng.standard_normal(n_sk * n_per) / noise
    ystar = 0.05 * rng.standard_normal(n_sk * n_per)
    probe = rng.standard_normal(n_sk * n_per).astype(np.float32)
    return rec, ystar, probe


def test_oracle_gradient_vs_finite_differences():
    H, B, n_sk, n_per = 4, 2, 10, 8
    rec, ystar, probe = small_system(n_sk, n_per)
    n_params = sum(r * c for _, r, c in lr.layout(H, B))
    rng = np.random.default_rng(1)
    flat = 0.4 * rng.standard_normal(n_params)

    def total(f):
        ls, _, _ = lr.loss_and_grad(f, rec, ystar, probe, n_sk, n_per, H, B, VAR_S, C_PERP,
                                    C_PARA, use_bf16=False)
        return ls[0] + ls[1]

    _, g, _ = lr.loss_and_grad(flat, rec, ystar, probe, n_sk, n_per, H, B, VAR_S, C_PERP,
                               C_PARA, use_bf16=False)
    idx = rng.choice(n_params, size=40, replace=False)
    eps = 1e-6
    for i in idx:
        fp, fm = flat.copy(), flat.copy()
        fp[i] += eps
        fm[i] -= eps
        fd = (total(fp) - total(fm)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -3.14159, 0.0])
    r = lr.bf16(x)
    assert r[0] == 1.0
    # ties to even: 1 + 2^-8 is exactly halfway between 1 and 1 + 2^-7
    assert r[1] == 1.0 and r[2] == 1.0 and r[3] == 1.0 + 2 ** -7
    assert abs(r[4] - (-3.140625)) < 1e-12 and r[5] == 0.0
