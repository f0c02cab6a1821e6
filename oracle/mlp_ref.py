"""CPU restatement of the sizing network (test infrastructure only).

Checks the device kernels of ``pierce_gb300/csrc/sizing.cu``: the forward
pass, the mean-squared-error loss on standardised log counts, its gradient
(hand-derived backpropagation, float64) and one Adam step.  Nothing in the
product imports this module.

Definitions (same as the device):
  z  = (x - x_mean) * x_scale
  h1 = relu(W1 z + b1), h2 = relu(W2 h1 + b2), o = W3 . h2 + b3
  t  = (y - y_mean) / y_std, loss = mean((o - t)^2)
  prediction = o * y_std + y_mean
"""
from __future__ import annotations

import numpy as np

NI, NH = 32, 64
NP = NH * NI + NH + NH * NH + NH + NH + 1


def unpack(w):
    w = np.asarray(w, np.float64)
    i = 0
    out = {}
    for name, shape in (("W1", (NH, NI)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NH,)),
                        ("b3", (1,))):
        n = int(np.prod(shape))
        out[name] = w[i:i + n].reshape(shape)
        i += n
    return out


def pack(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[k], np.float64).reshape(-1) for k in ("W1", "b1", "W2", "b2", "W3", "b3")])


def forward(w, x_mean, x_scale, X):
    p = unpack(w)
    Z = (np.asarray(X, np.float64) - np.asarray(x_mean, np.float64)) * np.asarray(x_scale, np.float64)
    A1 = Z @ p["W1"].T + p["b1"]
    H1 = np.maximum(A1, 0.0)
    A2 = H1 @ p["W2"].T + p["b2"]
    H2 = np.maximum(A2, 0.0)
    O = H2 @ p["W3"] + p["b3"][0]
    return Z, H1, H2, O


def predict(w, x_mean, x_scale, y_mean, y_std, X) -> np.ndarray:
    return forward(w, x_mean, x_scale, X)[3] * float(y_std) + float(y_mean)


def loss_and_grad(w, x_mean, x_scale, y_mean, y_std, X, y):
    """Mean squared error over the samples and its gradient (flat, NP)."""
    p = unpack(w)
    Z, H1, H2, O = forward(w, x_mean, x_scale, X)
    T = (np.asarray(y, np.float64) - float(y_mean)) / float(y_std)
    n = len(T)
    R = O - T
    loss = float(np.mean(R * R))
    dO = 2.0 * R / n
    g = {"W3": H2.T @ dO, "b3": np.array([dO.sum()])}
    D2 = np.outer(dO, p["W3"]) * (H2 > 0)
    g["W2"] = D2.T @ H1
    g["b2"] = D2.sum(0)
    D1 = (D2 @ p["W2"]) * (H1 > 0)
    g["W1"] = D1.T @ Z
    g["b1"] = D1.sum(0)
    return loss, pack(g)


def adam_step(w, m, v, g, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015); step counts from 1."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def fit_normalization(X, y):
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    sd = X.std(0)
    x_scale = np.where(sd > 1e-6, 1.0 / np.where(sd > 1e-6, sd, 1.0), 1.0)
    ys = y.std()
    return X.mean(0), x_scale, float(y.mean()), float(ys if ys > 1e-6 else 1.0)


def train(w, X, y, epochs=400, batch=64, lr=1e-3, seed=0):
    """Reference training loop (plain shuffles; used to show the method
    learns, not to reproduce the device's sample order)."""
    x_mean, x_scale, y_mean, y_std = fit_normalization(X, y)
    w = np.asarray(w, np.float64).copy()
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    rng = np.random.default_rng(seed)
    step = 0
    n = len(y)
    for _ in range(epochs):
        order = rng.permutation(n)
        for b0 in range(0, n, batch):
            idx = order[b0:b0 + batch]
            _, g = loss_and_grad(w, x_mean, x_scale, y_mean, y_std, X[idx], y[idx])
            step += 1
            w, m, v = adam_step(w, m, v, g, step, lr)
    return w, x_mean, x_scale, y_mean, y_std


def join_features(va, ia, ta, na, vb, ib, tb, nb, step=100):
    """The 32 join features from host arrays (vertices (V,3) float32,
    indices (F,3), tri_to_object (F,), object count) of both sides."""
    def side(v, idx, t2o, n):
        v = np.asarray(v, np.float32).reshape(-1, 3)
        idx = np.asarray(idx).reshape(-1, 3).astype(np.int64)
        t2o = np.asarray(t2o).astype(np.int64)
        lo = np.full((n, 3), np.inf, np.float32)
        hi = np.full((n, 3), -np.inf, np.float32)
        tri = v[idx]                                   # (F, 3 vertices, 3)
        np.minimum.at(lo, t2o, tri.min(1))
        np.maximum.at(hi, t2o, tri.max(1))
        cnt = np.bincount(t2o, minlength=n)[:n]
        ok = cnt > 0
        ext = (hi[ok].astype(np.float64) - lo[ok].astype(np.float64))
        m = ext.mean(0) if ok.any() else np.zeros(3)
        var = np.maximum((ext * ext).mean(0) - m * m, 0.0) if ok.any() else np.zeros(3)
        bins = np.clip(np.floor(np.log2(cnt[ok])).astype(np.int64) // 2 - 2, 0, 7)
        hist = np.bincount(bins, minlength=8)[:8] / max(int(ok.sum()), 1)
        f = np.concatenate([[np.log1p(n)], np.log1p(m), np.log1p(var), hist])
        return f, lo, hi, ok, m
    fa, loa, hia, oka, ma = side(va, ia, ta, na)
    fb, lob, hib, okb, mb = side(vb, ib, tb, nb)
    sa = np.arange(0, na, step)
    sa = sa[oka[sa]]
    la, ha = loa[sa], hia[sa]
    lb, hb = lob[okb], hib[okb]
    hits = 0
    for i in range(len(sa)):
        hits += int(np.all((la[i] <= hb) & (lb <= ha[i]), axis=1).sum())
    ns = (na + step - 1) // step
    f30 = np.log1p(hits * na / ns) if ns else 0.0
    lo = np.minimum(loa[oka].min(0), lob[okb].min(0)).astype(np.float64)
    hi = np.maximum(hia[oka].max(0), hib[okb].max(0)).astype(np.float64)
    vol = np.prod(np.maximum(hi - lo, 1e-6))
    f31 = np.log1p(na * nb / vol * np.prod(ma + mb))
    return np.concatenate([fa, fb, [f30, f31]]).astype(np.float64)
