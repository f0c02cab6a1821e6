"""Learned output sizing: join features, the 32-64-64-1 network, and the
selectivity sweep it is trained and judged on.

The network lives on the device (``pierce_mlp`` in ``libpierce_gb300.so``);
training, gradients and inference are the library's own FP32 kernels.  A join
run with ``sizing="learned"`` computes the 32 features of its two datasets,
predicts log(1 + unique pairs), sizes its hash set and result buffer for
prediction x ``output_safety`` and, when the pairs do not fit, reruns with
the two-pass method, which is both the fallback and the source of the
training counts.  The prediction never decides a predicate: the pair set is
the same in every sizing mode.

Sweep workload (per join): meshes per side log-uniform in [1k, 200k];
each side spheres (radius lognormal(ln 1.5, 0.3)) or ellipsoids (semi-axes
U[2, 5], random rotation, 5% radial value noise), subdivision level uniform
in {2, 3, 4} per mesh; the cube side is chosen for a target selectivity
(pairs per candidate) log-uniform in [1e-7, min(1e-2, 100 / max(nA, nB))] --
the upper bound keeps every mesh at <= 100 expected partners so the densest
corner of the sweep stays a join rather than a pile of coincident meshes.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, asdict
from pathlib import Path

import numpy as np

from . import capi
from .capi import check
from .geometry import ELLIPSOIDS, SPHERES, instances

DATA_DIR = Path(__file__).resolve().parent / "data"
TRAINING_SET = DATA_DIR / "sizing_joins.npz"
TRAINED_MODEL = DATA_DIR / "sizing_mlp.npz"

N_INPUTS, N_HIDDEN, N_PARAMS = capi.MLP_INPUTS, capi.MLP_HIDDEN, capi.MLP_PARAMS
FIXED_MEMORY_SLOTS = 1 << 30   # 8 GiB pair table: the fixed-memory mode


def split_params(w: np.ndarray) -> dict:
    """Views of a flat parameter vector as W1, b1, W2, b2, W3, b3."""
    w = np.asarray(w)
    i, H, I = 0, N_HIDDEN, N_INPUTS
    out = {}
    for name, shape in (("W1", (H, I)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H,)), ("b3", (1,))):
        n = int(np.prod(shape))
        out[name] = w[i:i + n].reshape(shape)
        i += n
    assert i == N_PARAMS
    return out


class SizingModel:
    """A device-resident sizing network."""

    def __init__(self, ctx, params: capi.MlpParams | None = None, seed: int = 1):
        self.ctx = ctx
        self._lib = capi.lib()
        if params is None:
            params = capi.MlpParams()
            check(self._lib.pierce_mlp_init_params(C.byref(params), C.c_uint64(seed)), "mlp_init_params")
        h = C.c_void_p()
        check(self._lib.pierce_mlp_create(ctx.handle, C.byref(params), C.byref(h)), "mlp_create")
        self._h = h
        ctx.adopt(self)

    @property
    def handle(self):
        return self._h

    def params(self) -> capi.MlpParams:
        p = capi.MlpParams()
        check(self._lib.pierce_mlp_get(self.ctx.handle, self._h, C.byref(p)), "mlp_get")
        return p

    def train(self, X, y, epochs: int = 400, lr: float = 1e-3, seed: int = 1, fit_normalization: bool = True):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, N_INPUTS)
        y = np.ascontiguousarray(y, np.float32).reshape(-1)
        o = capi.MlpTrainOpts()
        self._lib.pierce_default_mlp_train_opts(C.byref(o))
        o.epochs, o.lr, o.seed, o.fit_normalization = int(epochs), float(lr), int(seed), int(fit_normalization)
        loss = np.zeros(epochs, np.float32)
        check(self._lib.pierce_mlp_train(self.ctx.handle, self._h, X.ctypes.data, y.ctypes.data, len(y),
                                         C.byref(o), loss.ctypes.data), "mlp_train")
        return loss

    def gradient(self, X, y):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, N_INPUTS)
        y = np.ascontiguousarray(y, np.float32).reshape(-1)
        g = np.zeros(N_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        check(self._lib.pierce_mlp_gradient(self.ctx.handle, self._h, X.ctypes.data, y.ctypes.data, len(y),
                                            g.ctypes.data, loss.ctypes.data), "mlp_gradient")
        return g, float(loss[0])

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32).reshape(-1, N_INPUTS)
        out = np.zeros(len(X), np.float32)
        check(self._lib.pierce_mlp_predict(self.ctx.handle, self._h, X.ctypes.data, len(X), out.ctypes.data),
              "mlp_predict")
        return out

    def save(self, path) -> None:
        save_params(self.params(), path)

    @classmethod
    def load(cls, ctx, path) -> "SizingModel":
        return cls(ctx, load_params(path))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pierce_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def params_to_arrays(p: capi.MlpParams) -> dict:
    return {"weights": np.ctypeslib.as_array(p.weights).copy(), "x_mean": np.ctypeslib.as_array(p.x_mean).copy(),
            "x_scale": np.ctypeslib.as_array(p.x_scale).copy(), "y_mean": np.float32(p.y_mean),
            "y_std": np.float32(p.y_std)}


def arrays_to_params(a: dict) -> capi.MlpParams:
    p = capi.MlpParams()
    np.ctypeslib.as_array(p.weights)[:] = np.asarray(a["weights"], np.float32)
    np.ctypeslib.as_array(p.x_mean)[:] = np.asarray(a["x_mean"], np.float32)
    np.ctypeslib.as_array(p.x_scale)[:] = np.asarray(a["x_scale"], np.float32)
    p.y_mean, p.y_std = float(a["y_mean"]), float(a["y_std"])
    return p


def save_params(p: capi.MlpParams, path) -> None:
    np.savez(path, **params_to_arrays(p))


def load_params(path) -> capi.MlpParams:
    with np.load(path) as z:
        return arrays_to_params({k: z[k] for k in z.files})


def join_features(ctx, a, b) -> np.ndarray:
    out = np.zeros(N_INPUTS, np.float32)
    check(capi.lib().pierce_join_features(ctx.handle, a.handle, b.handle, out.ctypes.data), "join_features")
    return out


# ---- the selectivity sweep -------------------------------------------------------

@dataclass
class JoinSpec:
    seed_a: int
    seed_b: int
    n_a: int
    n_b: int
    family_a: int
    family_b: int
    extent: float
    target_selectivity: float


def _shell_volume(fa: int, fb: int, rng: np.random.Generator, k: int = 4096) -> float:
    """E[(4/3) pi ((ra + rb)^3 - |ra - rb|^3)]: the centre-distance shell in which
    two spheres' surfaces meet (ellipsoids by their mean semi-axis)."""
    def radii(f):
        if f == SPHERES:
            return np.exp(math.log(1.5) + 0.3 * rng.standard_normal(k))
        return rng.uniform(2.0, 5.0, (k, 3)).mean(1)
    ra, rb = radii(fa), radii(fb)
    return float((4.0 / 3.0) * math.pi * np.mean((ra + rb) ** 3 - np.abs(ra - rb) ** 3))


def sweep(seed: int, count: int, n_lo: int = 1000, n_hi: int = 200_000) -> list[JoinSpec]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n_a = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        n_b = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        fa, fb = int(rng.integers(0, 2)), int(rng.integers(0, 2))
        s_hi = min(1e-2, 100.0 / max(n_a, n_b))
        sel = math.exp(rng.uniform(math.log(1e-7), math.log(s_hi)))
        extent = (_shell_volume(fa, fb, rng) / sel) ** (1.0 / 3.0)
        out.append(JoinSpec(int(rng.integers(1, 2**62)), int(rng.integers(1, 2**62)), n_a, n_b, fa, fb,
                            float(extent), float(sel)))
    return out


def make_datasets(ctx, spec: JoinSpec, level_lo: int = 2, level_hi: int = 4):
    """Both sides of a sweep join, expanded on the device (no dataset BVHs:
    the joins build per-join hierarchies, with leaves of 4 triangles)."""
    from .join import Dataset, default_tuning
    t = default_tuning(leaf_size=4, defer_build=1)
    ia = instances(spec.seed_a, spec.n_a, spec.family_a, level_lo, level_hi, hi=spec.extent)
    ib = instances(spec.seed_b, spec.n_b, spec.family_b, level_lo, level_hi, hi=spec.extent)
    return Dataset.from_instances(ctx, ia, t), Dataset.from_instances(ctx, ib, t)


def build_training_set(ctx, specs: list[JoinSpec], log=None) -> dict:
    """Features and exact two-pass unique-pair counts of the sweep joins."""
    from .join import make_opts, run_join
    X = np.zeros((len(specs), N_INPUTS), np.float32)
    counts = np.zeros(len(specs), np.int64)
    tris = np.zeros((len(specs), 2), np.int64)
    for i, sp in enumerate(specs):
        a, b = make_datasets(ctx, sp)
        X[i] = join_features(ctx, a, b)
        r = run_join(ctx, a, b, make_opts(predicate="overlap", sizing="two_pass"), download=False)
        counts[i] = r.stats["num_pairs"]
        tris[i] = (a.info().num_triangles, b.info().num_triangles)
        a.close()
        b.close()
        _bound_memory(ctx)
        if log and (i % 50 == 0 or i == len(specs) - 1):
            log(f"{i + 1}/{len(specs)} nA={sp.n_a} nB={sp.n_b} pairs={counts[i]}")
    cols = {k: np.array([getattr(s, k) for s in specs]) for k in asdict(specs[0])} if specs else {}
    return {"features": X, "pairs": counts, "triangles": tris, **{"spec_" + k: v for k, v in cols.items()}}


def _bound_memory(ctx, keep_free: float = 0.25) -> None:
    """Between joins of very different sizes: hand the context's grow-only
    scratch back to the device once free memory runs below `keep_free`."""
    free, total = ctx.device_memory()
    if free < keep_free * total:
        ctx.release_scratch()


def targets(pairs) -> np.ndarray:
    return np.log1p(np.asarray(pairs, np.float64)).astype(np.float32)


def evaluate(ctx, model: "SizingModel", specs: list[JoinSpec], log=None) -> dict:
    """Held-out comparison of the sizing modes on the same joins: two-pass,
    learned (prediction x 1.2, two-pass on overflow) and fixed memory (an
    8 GiB table).  Every mode must return the same pair set."""
    import time
    from .join import make_opts, run_join
    rows = []
    modes = {"two_pass": make_opts(predicate="overlap", sizing="two_pass"),
             "learned": make_opts(predicate="overlap", sizing="learned", sizing_model=model),
             "fixed": make_opts(predicate="overlap", sizing="fixed", hash_table_slots=FIXED_MEMORY_SLOTS)}
    for i, sp in enumerate(specs):
        a, b = make_datasets(ctx, sp)
        row = {"n_a": sp.n_a, "n_b": sp.n_b}
        ref = None
        for name, o in modes.items():
            ctx.synchronize()
            t0 = time.perf_counter()
            r = run_join(ctx, a, b, o)
            row[name + "_s"] = time.perf_counter() - t0
            row[name + "_gpu_ms"] = r.stats["ms_total"]
            row[name + "_table_bytes"] = 8 * r.stats["hash_slots"]
            row[name + "_result_bytes"] = 8 * r.stats["result_capacity"]
            if name == "learned":
                row["predicted"] = r.stats["predicted_pairs"]
                row["overflow"] = r.stats["sizing_overflow"]
            if ref is None:
                ref = r.pairs
                row["pairs"] = len(r.pairs)
            else:
                row[name + "_identical"] = bool(np.array_equal(r.pairs, ref))
        a.close()
        b.close()
        _bound_memory(ctx)
        rows.append(row)
        if log and (i % 20 == 0 or i == len(specs) - 1):
            log(f"{i + 1}/{len(specs)} pairs={row['pairs']} predicted={row['predicted']:.0f}")
    cols = {k: np.array([r[k] for r in rows]) for k in rows[0]} if rows else {}
    return cols


def summarize(ev: dict) -> dict:
    y = np.log1p(ev["pairs"].astype(np.float64))
    p = np.log1p(np.maximum(ev["predicted"], 0.0))
    out = {"joins": int(len(y)), "overflow_rate": float(ev["overflow"].mean()),
           "mean_abs_log_error": float(np.abs(p - y).mean()),
           "identical_pair_sets": bool(ev["learned_identical"].all() and ev["fixed_identical"].all())}
    for m in ("two_pass", "learned", "fixed"):
        out[m + "_total_s"] = float(ev[m + "_s"].sum())
        out[m + "_gpu_ms_total"] = float(ev[m + "_gpu_ms"].sum())
        out[m + "_mean_buffer_mib"] = float((ev[m + "_table_bytes"] + ev[m + "_result_bytes"]).mean() / 2**20)
    return out


def _main(argv=None) -> int:
    import argparse
    import json
    import sys
    import time
    from .join import Context
    ap = argparse.ArgumentParser(prog="python -m pierce_gb300.sizing")
    sub = ap.add_subparsers(dest="cmd", required=True)
    s1 = sub.add_parser("sweep", help="features + two-pass counts of sweep joins")
    s1.add_argument("--seed", type=int, default=2024)
    s1.add_argument("--count", type=int, default=2200)
    s1.add_argument("--out", default=str(TRAINING_SET))
    s2 = sub.add_parser("train", help="train the network on a sweep (GPU kernels)")
    s2.add_argument("--data", default=str(TRAINING_SET))
    s2.add_argument("--holdout", type=int, default=200)
    s2.add_argument("--epochs", type=int, default=600)
    s2.add_argument("--lr", type=float, default=1e-3)
    s2.add_argument("--out", default=str(TRAINED_MODEL))
    s3 = sub.add_parser("evaluate", help="sizing modes on the held-out joins of a sweep")
    s3.add_argument("--model", default=str(TRAINED_MODEL))
    s3.add_argument("--seed", type=int, default=2024)
    s3.add_argument("--skip", type=int, default=2000, help="sweep joins before the held-out ones")
    s3.add_argument("--count", type=int, default=200)
    s3.add_argument("--out", default="")
    a = ap.parse_args(argv)
    log = lambda m: print(m, file=sys.stderr, flush=True)
    ctx = Context(0)
    t0 = time.perf_counter()
    if a.cmd == "sweep":
        data = build_training_set(ctx, sweep(a.seed, a.count), log)
        np.savez_compressed(a.out, **data)
        log(f"sweep of {a.count} joins in {time.perf_counter() - t0:.1f} s -> {a.out}")
    elif a.cmd == "train":
        with np.load(a.data) as z:
            X, y = z["features"], targets(z["pairs"])
        n = len(y) - a.holdout
        m = SizingModel(ctx, seed=1)
        loss = m.train(X[:n], y[:n], epochs=a.epochs, lr=a.lr)
        pred = m.predict(X[n:])
        m.save(a.out)
        print(json.dumps({"train_loss_first": float(loss[0]), "train_loss_last": float(loss[-1]),
                          "holdout_mean_abs_log_error": float(np.abs(pred - y[n:]).mean()),
                          "train_s": time.perf_counter() - t0}))
    else:
        model = SizingModel.load(ctx, a.model)
        ev = evaluate(ctx, model, sweep(a.seed, a.skip + a.count)[a.skip:], log)
        if a.out:
            np.savez_compressed(a.out, **ev)
        print(json.dumps(summarize(ev)))
    return 0


if __name__ == "__main__":
    raise SystemExit(_main())
