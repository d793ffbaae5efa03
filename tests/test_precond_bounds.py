"""CPU check of the preconditioner design (no GPU, no reference counterpart;
the reference's PCG is Jacobi, lib/wf_vector.cc:42-49,185-194).

On a W-form system at the 262,144-pixel workload's skewer density (24
skewers x 128 pixels in a box of the same density, GRF data, exact kernel)
numpy FP64 PCG to 1e-8 with

* Jacobi,
* the exact inverse of every skewer's own block (the best any per-skewer
  factor L with M^-1 = L L^T can do, whatever its band),
* the factorized sparse approximate inverse (FSAI) of every cluster of four
  neighbouring skewers, pixels in (z, skewer) order, 16 sub-diagonals (the
  library's cluster preconditioner, built here from its definition),

shows why the library preconditions clusters rather than single skewers:
the per-skewer optimum saves under a third of the Jacobi iterations, the
cluster factor about half.  With the full pattern the FSAI factor is exactly
the Cholesky factor of the cluster block's inverse (checked to 1e-10).
"""
import numpy as np

from dachshund_gb300 import synth

VS, LP, LQ = synth.VAR_S, synth.L_PERP, synth.L_PARA
C_PERP, C_PARA = 1 / (2 * LP ** 2), 1 / (2 * LQ ** 2)


def system(n_sk=24, n_per=128, seed=5):
    box = 80.0 * np.sqrt(n_sk / 1024)
    w = synth.grf_workload("t", n_sk, n_per, box, seed, (4, 4, 32), 1e-8)
    pix = w.pixels
    S = synth.exact_covariance(pix[:, :3])
    wv = 1.0 / pix[:, 3]
    A = (wv[:, None] * S) * wv[None, :]
    A[np.diag_indices_from(A)] += 1.0
    return pix, A, wv * pix[:, 4]


def pcg_iters(A, b, apply_m, tol=1e-8, max_iter=5000):
    x = np.zeros_like(b)
    r = b.copy()
    z = apply_m(r)
    d = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for it in range(1, max_iter):
        q = A @ d
        alpha = rz / (d @ q)
        x += alpha * d
        r -= alpha * q
        if np.linalg.norm(r) <= tol * nb:
            return it
        z = apply_m(r)
        rz_new = r @ z
        d = z + (rz_new / rz) * d
        rz = rz_new
    return max_iter


def fsai(Ab, band):
    """Lower G with G[J, j] = g / sqrt(g_0), A[J, J] g = e_0, J = j .. j + band."""
    m = Ab.shape[0]
    G = np.zeros_like(Ab)
    for j in range(m):
        J = np.arange(j, min(m, j + band + 1))
        e = np.zeros(len(J))
        e[0] = 1.0
        g = np.linalg.solve(Ab[np.ix_(J, J)], e)
        G[J, j] = g / np.sqrt(g[0])
    return G


def clusters(pix, n_sk, n_per, size):
    """Greedy groups of `size` nearest skewers, each in (z, skewer) order."""
    xy = pix[::n_per, :2]
    left = list(range(n_sk))
    out = []
    while left:
        s0 = left.pop(0)
        d = np.sum((xy[left] - xy[s0]) ** 2, axis=1)
        pick = [left[i] for i in np.argsort(d)[:size - 1]]
        for p in pick:
            left.remove(p)
        members = [s0] + pick
        out.append(np.array([s * n_per + k for k in range(n_per) for s in members]))
    return out


def block_apply(blocks):
    def apply_m(r):
        out = np.empty_like(r)
        for idx, M in blocks:
            out[idx] = M @ r[idx]
        return out
    return apply_m


def test_cluster_factor_beats_every_per_skewer_factor():
    n_sk, n_per = 24, 128
    pix, A, b = system(n_sk, n_per)
    jac = np.diag(A).copy()
    it_jacobi = pcg_iters(A, b, lambda r: r / jac)
    skewer_blocks = []
    for s in range(n_sk):
        idx = np.arange(s * n_per, (s + 1) * n_per)
        skewer_blocks.append((idx, np.linalg.inv(A[np.ix_(idx, idx)])))
    it_skewer = pcg_iters(A, b, block_apply(skewer_blocks))
    cl_blocks = []
    for idx in clusters(pix, n_sk, n_per, 4):
        G = fsai(A[np.ix_(idx, idx)], 16)
        cl_blocks.append((idx, G @ G.T))
    it_cluster = pcg_iters(A, b, block_apply(cl_blocks))
    assert it_skewer >= 0.7 * it_jacobi, (it_skewer, it_jacobi)
    assert it_cluster <= 0.6 * it_jacobi, (it_cluster, it_jacobi)
    assert it_cluster < it_skewer


def test_fsai_full_pattern_is_cholesky_of_inverse():
    pix, A, _ = system(4, 24, seed=2)
    idx = np.arange(48)
    Ab = A[np.ix_(idx, idx)]
    G = fsai(Ab, 47)
    C = np.linalg.cholesky(np.linalg.inv(Ab))
    assert np.max(np.abs(G - C)) <= 1e-10 * np.max(np.abs(C))
    assert np.max(np.abs(G @ G.T @ Ab - np.eye(48))) < 1e-10
