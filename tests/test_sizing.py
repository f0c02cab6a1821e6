"""Learned output sizing: the network's kernels against the CPU oracle and
torch, the join features against a numpy restatement, and learned-sizing
joins against the two-pass method (identical pair sets, overflow fallback).
"""
import numpy as np
import pytest

import pierce_gb300 as pg
from oracle import mlp_ref as R

NP_ = R.NP


def random_case(seed, n):
    rng = np.random.default_rng(seed)
    w = rng.normal(0, 0.2, NP_)
    X = rng.normal(0, 1, (n, R.NI)).astype(np.float32)
    y = (X[:, :3].sum(1) + 0.1 * rng.normal(size=n)).astype(np.float32)
    return w, X, y


def test_oracle_gradient_matches_finite_differences():
    w, X, y = random_case(1, 40)
    xm, xs, ym, ys = R.fit_normalization(X, y)
    loss, g = R.loss_and_grad(w, xm, xs, ym, ys, X, y)
    rng = np.random.default_rng(2)
    for i in rng.choice(NP_, 60, replace=False):
        e = np.zeros(NP_)
        e[i] = 1e-6
        fd = (R.loss_and_grad(w + e, xm, xs, ym, ys, X, y)[0] - R.loss_and_grad(w - e, xm, xs, ym, ys, X, y)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i])


def test_oracle_gradient_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    w, X, y = random_case(3, 50)
    xm, xs, ym, ys = R.fit_normalization(X, y)
    loss, g = R.loss_and_grad(w, xm, xs, ym, ys, X, y)
    p = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in R.unpack(w).items()}
    Z = (torch.tensor(X, dtype=torch.float64) - torch.tensor(xm)) * torch.tensor(xs)
    h1 = torch.relu(Z @ p["W1"].T + p["b1"])
    h2 = torch.relu(h1 @ p["W2"].T + p["b2"])
    o = h2 @ p["W3"] + p["b3"][0]
    t = (torch.tensor(y, dtype=torch.float64) - ym) / ys
    L = torch.mean((o - t) ** 2)
    L.backward()
    gt = R.pack({k: v.grad.numpy() for k, v in p.items()})
    assert abs(L.item() - loss) < 1e-12
    np.testing.assert_allclose(g, gt, rtol=1e-10, atol=1e-12)


def test_sweep_covers_the_selectivity_range():
    from pierce_gb300 import sizing as S
    specs = S.sweep(7, 400)
    n = np.array([[s.n_a, s.n_b] for s in specs])
    sel = np.array([s.target_selectivity for s in specs])
    assert n.min() >= 1000 and n.max() <= 200_000
    assert sel.min() >= 1e-7 and sel.max() <= 1e-2
    assert sel.min() < 1e-6 and sel.max() > 1e-3
    assert np.all(sel <= 100.0 / n.max(1) + 1e-12)
    assert {s.family_a for s in specs} == {0, 1}


def test_trained_network_beats_the_estimates_it_is_given():
    """What the network gains over sizing without it: on held-out joins of
    the committed sweep, its log-count error is well below that of the two
    estimates among its inputs (the 1% box-overlap sample and the
    uniform-placement box-overlap expectation)."""
    from pierce_gb300 import sizing as S
    if not S.TRAINING_SET.exists():
        pytest.skip("sweep training set not generated")
    with np.load(S.TRAINING_SET) as z:
        X, pairs = z["features"], z["pairs"]
    y = S.targets(pairs)
    n_train = len(y) - 200 if len(y) > 400 else len(y) // 2
    w0 = np.random.default_rng(0).normal(0, 0.1, NP_)
    w, xm, xs, ym, ys = R.train(w0, X[:n_train], y[:n_train], epochs=150)
    pred = R.predict(w, xm, xs, ym, ys, X[n_train:])
    err = np.abs(pred - y[n_train:])
    err_sample = np.abs(X[n_train:, 30] - y[n_train:])
    err_uniform = np.abs(X[n_train:, 31] - y[n_train:])
    assert err.mean() < 0.6 * min(err_sample.mean(), err_uniform.mean())


# ---- device kernels -----------------------------------------------------------

def model_from(ctx, w, xm, xs, ym, ys):
    from pierce_gb300 import sizing as S
    return S.SizingModel(ctx, S.arrays_to_params({"weights": w, "x_mean": xm, "x_scale": xs, "y_mean": ym,
                                                  "y_std": ys}))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [7, 64, 200])
def test_device_gradient_matches_oracle_and_torch(ctx, n):
    torch = pytest.importorskip("torch")
    w, X, y = random_case(10 + n, n)
    xm, xs, ym, ys = R.fit_normalization(X, y)
    w32 = w.astype(np.float32)
    m = model_from(ctx, w32, xm, xs, ym, ys)
    g, loss = m.gradient(X, y)
    # oracle on the float32 parameters the device holds
    xm32, xs32 = np.float32(xm).astype(np.float64), np.float32(xs).astype(np.float64)
    lo, go = R.loss_and_grad(w32.astype(np.float64), xm32, xs32, float(np.float32(ym)), float(np.float32(ys)), X, y)
    assert abs(loss - lo) <= 1e-5 * max(1.0, lo)
    scale = np.abs(go).max()
    np.testing.assert_allclose(g, go, rtol=2e-4, atol=2e-5 * scale)
    # torch float32 autograd of the same network
    p = {k: torch.tensor(v, dtype=torch.float32, requires_grad=True) for k, v in R.unpack(w32).items()}
    Z = (torch.tensor(X) - torch.tensor(np.float32(xm))) * torch.tensor(np.float32(xs))
    o = torch.relu(torch.relu(Z @ p["W1"].T + p["b1"]) @ p["W2"].T + p["b2"]) @ p["W3"] + p["b3"][0]
    t = (torch.tensor(y) - float(np.float32(ym))) / float(np.float32(ys))
    torch.mean((o - t) ** 2).backward()
    gt = R.pack({k: v.grad.numpy() for k, v in p.items()})
    np.testing.assert_allclose(g, gt, rtol=2e-3, atol=1e-4 * scale)


@pytest.mark.gpu
def test_device_predict_matches_oracle(ctx):
    w, X, y = random_case(21, 300)
    xm, xs, ym, ys = R.fit_normalization(X, y)
    w32 = w.astype(np.float32)
    m = model_from(ctx, w32, xm, xs, ym, ys)
    got = m.predict(X)
    want = R.predict(w32.astype(np.float64), np.float32(xm).astype(np.float64), np.float32(xs).astype(np.float64),
                     float(np.float32(ym)), float(np.float32(ys)), X)
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_device_adam_step_matches_oracle(ctx):
    """One epoch over <= 64 samples is one full-batch Adam step."""
    w, X, y = random_case(31, 50)
    xm, xs, ym, ys = R.fit_normalization(X, y)
    w32 = w.astype(np.float32)
    m = model_from(ctx, w32, xm, xs, ym, ys)
    m.train(X, y, epochs=1, lr=1e-2, fit_normalization=False)
    from pierce_gb300 import sizing as S
    got = np.ctypeslib.as_array(m.params().weights).astype(np.float64)
    f = lambda a: np.float32(a).astype(np.float64)
    _, g = R.loss_and_grad(w32.astype(np.float64), f(xm), f(xs), float(f(ym)), float(f(ys)), X, y)
    want, _, _ = R.adam_step(w32.astype(np.float64), np.zeros(NP_), np.zeros(NP_), g, 1, lr=1e-2)
    # an Adam step moves each weight by about lr * sign(g): compare the moves
    np.testing.assert_allclose(got - w32, want - w32, atol=2e-4)


@pytest.mark.gpu
def test_device_training_learns(ctx):
    from pierce_gb300 import sizing as S
    rng = np.random.default_rng(5)
    X = rng.normal(0, 1, (2000, R.NI)).astype(np.float32)
    y = (np.abs(X[:, 0]) * 2 + X[:, 1] * X[:, 2] + 5).astype(np.float32)
    m = S.SizingModel(ctx, seed=3)
    loss = m.train(X[:1600], y[:1600], epochs=200, lr=2e-3)
    assert loss[-1] < 0.1 * loss[0]
    pred = m.predict(X[1600:])
    assert np.mean((pred - y[1600:]) ** 2) < 0.35 * np.var(y[1600:])


@pytest.mark.gpu
def test_join_features_match_numpy(ctx):
    from pierce_gb300 import join as J, sizing as S
    ia = pg.instances(51, 700, pg.SPHERES, 1, 3, hi=120.0)
    ib = pg.instances(52, 900, pg.ELLIPSOIDS, 1, 2, hi=120.0)
    A = J.Dataset.from_instances(ctx, ia, J.default_tuning(defer_build=1))
    B = J.Dataset.from_instances(ctx, ib, J.default_tuning(defer_build=1))
    f = S.join_features(ctx, A, B)
    a, b = A.download(), B.download()
    want = R.join_features(a["vertices"], a["indices"], a["tri_to_object"], 700,
                           b["vertices"], b["indices"], b["tri_to_object"], 900)
    np.testing.assert_allclose(f, want, rtol=1e-5, atol=1e-5)


@pytest.mark.gpu
def test_learned_join_equals_two_pass_and_falls_back(ctx):
    from pierce_gb300 import join as J, sizing as S
    ia = pg.instances(61, 2000, pg.SPHERES, 2, 3, hi=60.0)
    ib = pg.instances(62, 2000, pg.ELLIPSOIDS, 2, 3, p0=1.0, p1=2.0, hi=60.0)
    A = J.Dataset.from_instances(ctx, ia, J.default_tuning(defer_build=1))
    B = J.Dataset.from_instances(ctx, ib, J.default_tuning(defer_build=1))
    ref = J.overlap_join_two_pass(ctx, A, B)
    assert len(ref.pairs) > 2000
    # a network that predicts the true count exactly (bias only)
    w = np.zeros(NP_, np.float32)
    exact = S.SizingModel(ctx, S.arrays_to_params({"weights": w, "x_mean": np.zeros(32), "x_scale": np.ones(32),
                                                   "y_mean": np.log1p(len(ref.pairs)), "y_std": 1.0}))
    r = J.run_join(ctx, A, B, J.make_opts(predicate="overlap", sizing="learned", sizing_model=exact))
    assert np.array_equal(r.pairs, ref.pairs)
    assert r.stats["sizing_overflow"] == 0
    assert abs(r.stats["predicted_pairs"] - len(ref.pairs)) < 0.01 * len(ref.pairs)
    assert r.stats["result_capacity"] <= 1.2 * len(ref.pairs) + 2
    # a network that predicts one tenth: the pairs overflow, two-pass reruns
    low = S.SizingModel(ctx, S.arrays_to_params({"weights": w, "x_mean": np.zeros(32), "x_scale": np.ones(32),
                                                 "y_mean": np.log1p(len(ref.pairs) / 10), "y_std": 1.0}))
    r2 = J.run_join(ctx, A, B, J.make_opts(predicate="overlap", sizing="learned", sizing_model=low))
    assert r2.stats["sizing_overflow"] == 1
    assert np.array_equal(r2.pairs, ref.pairs)
    # intersection with learned sizing gives the same set as two-pass
    ri = J.run_join(ctx, A, B, J.make_opts(predicate="intersection", sizing="learned", sizing_model=exact))
    assert np.array_equal(ri.pairs, J.intersection_join(ctx, A, B, sizing="two_pass").pairs)
