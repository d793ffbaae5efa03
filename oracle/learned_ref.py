"""CPU oracle of the learned warm start / skewer-band preconditioner network.

Test infrastructure only: the forward pass, both losses and the backward pass
of the network that dachshund_gb300/csrc/learned.cu runs on the GPU, written
out by hand in numpy float64 (no autograd), with the forward weights rounded
to BF16 as on the GPU (``bf16=False`` keeps them exact, for finite-difference
checks of the oracle itself).  The network has no counterpart in the
reference; it is checked here against its own definition:

  inputs   x0 = 2 k / (n_per - 1) - 1, x1 = (log n - LOGN0) / LOGNS,
           x2 = w d / 2, x3..x10 = exp(-c_perp d_perp^2) to the 8 nearest
           skewers (ties by skewer index)
  embed    h0 = relu(X W_in + b_in)
  layers   h_l = h_{l-1} + relu([h | A_z h | A_n h] W_l + b_l)
  head     Y = h_4 W_o + b_o;  y0 = XS Y0,
           L_kk = exp(SD tanh(Y1)) / sqrt(1 + w_k^2 var_s),
           L_{k,k-1} = a1 L_kk, L_{k,k-2} = a2 L_kk (band 2) with
           a2 = AC tanh(Y3), a1 = AC (1 + a2) tanh(Y2)
  losses   w_x sum (y0 - y*)^2 / sum y*^2  and
           w_p sum_s |L L^T A_bb v - v|^2 / n,  A_bb = I + w S_bb w (the
           skewer's own block, exact kernel)
"""
from __future__ import annotations

import numpy as np

F_IN, N_LAYERS, NB_K = 11, 4, 8
XS, SD, AC = 0.3, 1.0, 0.9
LOGN0, LOGNS = -2.1, 0.6


def bf16(a):
    """Round-to-nearest-even to BF16 (returned as float64)."""
    x = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    x = (x + 0x7FFF + ((x >> 16) & 1)) & 0xFFFF0000
    return x.astype(np.uint32).view(np.float32).astype(np.float64)


def layout(H, B):
    """(name, rows, cols) of the flat parameter vector, in order."""
    NO = 2 + B
    out = [("W_in", F_IN, H), ("b_in", 1, H)]
    for l in range(N_LAYERS):
        out += [(f"W_{l}", 3 * H, H), (f"b_{l}", 1, H)]
    out += [("W_o", H, NO), ("b_o", 1, NO)]
    return out


def unpack(flat, H, B):
    p, off = {}, 0
    for name, r, c in layout(H, B):
        p[name] = np.asarray(flat[off:off + r * c], dtype=np.float64).reshape(r, c)
        off += r * c
    assert off == len(flat)
    return p


def pack(d, H, B):
    return np.concatenate([d[name].ravel() for name, _, _ in layout(H, B)])


def knn(rec, n_sk, n_per, c_perp):
    xy = rec[::n_per, :2]
    d2 = ((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    nbr = np.argsort(d2, axis=1, kind="stable")[:, :NB_K]
    dn = np.take_along_axis(d2, nbr, axis=1)
    g = np.exp(-dn * c_perp).astype(np.float32).astype(np.float64)
    return nbr, g


def features(rec, n_sk, n_per, g):
    n = n_sk * n_per
    k = np.tile(np.arange(n_per), n_sk)
    X = np.empty((n, F_IN))
    X[:, 0] = 2.0 * k / (n_per - 1) - 1.0 if n_per > 1 else 0.0
    X[:, 1] = (-np.log(rec[:, 3]) - LOGN0) / LOGNS
    X[:, 2] = 0.5 * rec[:, 4]
    X[:, 3:] = np.repeat(g, n_per, axis=0)
    return X


def agg(h, n_sk, n_per, nbr, g):
    H = h.shape[1]
    hs = h.reshape(n_sk, n_per, H)
    az = np.zeros_like(hs)
    az[:, 1:] += hs[:, :-1]
    az[:, :-1] += hs[:, 1:]
    an = np.einsum("sm,smkc->skc", g, hs[nbr])
    return np.concatenate([h, az.reshape(-1, H), an.reshape(-1, H)], axis=1)


def agg_adjoint(dcat, n_sk, n_per, nbr, g, H):
    d0 = dcat[:, :H].reshape(n_sk, n_per, H)
    dz = dcat[:, H:2 * H].reshape(n_sk, n_per, H)
    dn = dcat[:, 2 * H:].reshape(n_sk, n_per, H)
    out = d0.copy()
    out[:, :-1] += dz[:, 1:]
    out[:, 1:] += dz[:, :-1]
    for m in range(NB_K):
        np.add.at(out, nbr[:, m], g[:, m, None, None] * dn)
    return out.reshape(-1, H)


def jacobi_factor(rec, var_s):
    return (1.0 / np.sqrt(1.0 + rec[:, 3] ** 2 * var_s)).astype(np.float32).astype(np.float64)


def band_L(Y, rec, n_sk, n_per, B, var_s):
    """[n_sk, n_per, B + 1] rows of L (L[k][k - m] at m)."""
    assert B == 2
    L = np.zeros((n_sk * n_per, B + 1))
    L[:, 0] = jacobi_factor(rec, var_s) * np.exp(SD * np.tanh(Y[:, 1]))
    a2 = AC * np.tanh(Y[:, 3])
    a1 = AC * (1 + a2) * np.tanh(Y[:, 2])
    k = np.tile(np.arange(n_per), n_sk)
    L[:, 1] = np.where(k >= 1, a1 * L[:, 0], 0.0)
    L[:, 2] = np.where(k >= 2, a2 * L[:, 0], 0.0)
    return L.reshape(n_sk, n_per, B + 1)


def dense_L(Lb):
    n_per, B1 = Lb.shape
    M = np.zeros((n_per, n_per))
    for k in range(n_per):
        for m in range(B1):
            if k - m >= 0:
                M[k, k - m] = Lb[k, m]
    return M


def forward(flat, rec, n_sk, n_per, H, B, c_perp, use_bf16=True):
    p = unpack(flat, H, B)
    rw = bf16 if use_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    nbr, g = knn(rec, n_sk, n_per, c_perp)
    X = features(rec, n_sk, n_per, g)
    cache = {"nbr": nbr, "g": g, "X": X}
    Z0 = X @ rw(p["W_in"]) + p["b_in"]
    h = np.maximum(Z0, 0)
    cache["Z"] = [Z0]
    cache["h"] = [h]
    cache["cat"] = []
    for l in range(N_LAYERS):
        cat = agg(h, n_sk, n_per, nbr, g)
        Zl = cat @ rw(p[f"W_{l}"]) + p[f"b_{l}"]
        h = h + np.maximum(Zl, 0)
        cache["cat"].append(cat)
        cache["Z"].append(Zl)
        cache["h"].append(h)
    Y = h @ rw(p["W_o"]) + p["b_o"]
    cache["Y"] = Y
    return Y, cache


def losses_and_dY(Y, rec, ystar, probe, n_sk, n_per, B, var_s, c_para, w_x, w_p):
    n = n_sk * n_per
    NO = 2 + B
    dY = np.zeros_like(Y)
    y0 = XS * Y[:, 0]
    t2 = float(np.sum(ystar ** 2))
    lx = w_x * float(np.sum((y0 - ystar) ** 2)) / t2
    dY[:, 0] = w_x * 2.0 * (y0 - ystar) * XS / t2
    Lb = band_L(Y, rec, n_sk, n_per, B, var_s)
    Jf = jacobi_factor(rec, var_s)
    lp = 0.0
    for s in range(n_sk):
        sl = slice(s * n_per, (s + 1) * n_per)
        z, w, v = rec[sl, 2], rec[sl, 3], probe[sl].astype(np.float64)
        T = np.exp(-c_para * (z[:, None] - z[None, :]) ** 2)
        u = v + w * var_s * (T @ (w * v))
        L = dense_L(Lb[s])
        t = L.T @ u
        sv = L @ t
        rho = sv - v
        lp += w_p * float(rho @ rho) / n
        gs = 2.0 * w_p * rho / n
        gt = L.T @ gs
        dLd = np.outer(gs, t) + np.outer(u, gt)  # d loss / d L[k][j]
        Ys = Y[sl]
        for k in range(n_per):
            th1, th2, th3 = np.tanh(Ys[k, 1]), np.tanh(Ys[k, 2]), np.tanh(Ys[k, 3])
            dk = Jf[s * n_per + k] * np.exp(SD * th1)
            a2 = AC * th3
            a1 = AC * (1 + a2) * th2
            dl = [dLd[k, k - m] if k - m >= 0 else 0.0 for m in range(3)]
            i = s * n_per + k
            dY[i, 1] = (dl[0] + dl[1] * a1 + dl[2] * a2) * dk * SD * (1 - th1 * th1)
            dY[i, 2] = dl[1] * AC * (1 + a2) * (1 - th2 * th2) * dk
            dY[i, 3] = (dl[1] * AC * th2 + dl[2]) * AC * (1 - th3 * th3) * dk
    assert dY.shape[1] == NO
    return (lx, lp), dY


def backward(flat, cache, dY, n_sk, n_per, H, B, use_bf16=True):
    p = unpack(flat, H, B)
    rw = bf16 if use_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    gr = {}
    h4 = cache["h"][N_LAYERS]
    gr["W_o"] = h4.T @ dY
    gr["b_o"] = dY.sum(0, keepdims=True)
    dh = dY @ rw(p["W_o"]).T
    for l in reversed(range(N_LAYERS)):
        dZ = dh * (cache["Z"][l + 1] > 0)
        cat = cache["cat"][l]
        gr[f"W_{l}"] = cat.T @ dZ
        gr[f"b_{l}"] = dZ.sum(0, keepdims=True)
        dcat = dZ @ rw(p[f"W_{l}"]).T
        dh = dh + agg_adjoint(dcat, n_sk, n_per, cache["nbr"], cache["g"], H)
    dZ0 = dh * (cache["Z"][0] > 0)
    gr["W_in"] = cache["X"].T @ dZ0
    gr["b_in"] = dZ0.sum(0, keepdims=True)
    return pack(gr, H, B)


def loss_and_grad(flat, rec, ystar, probe, n_sk, n_per, H, B, var_s, c_perp, c_para,
                  w_x=1.0, w_p=1.0, use_bf16=True):
    """(losses (l_x, l_p), flat gradient, Y)."""
    Y, cache = forward(flat, rec, n_sk, n_per, H, B, c_perp, use_bf16)
    ls, dY = losses_and_dY(Y, rec, ystar, probe, n_sk, n_per, B, var_s, c_para, w_x, w_p)
    return ls, backward(flat, cache, dY, n_sk, n_per, H, B, use_bf16), Y
