"""Python access to the CPU oracle (oracle/oracle.cpp) — test infrastructure.

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; it is the checker, never the product path.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
_lib = None

V = C.c_void_p
U64 = C.c_uint64


def build() -> Path:
    """Compile the oracle (g++, OpenMP, no FMA contraction)."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "oracle.cpp"
    if LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           str(src), "-o", str(LIB)]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stdout)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.oracle_overlap_pairs.restype = C.POINTER(C.c_uint64)
        L.oracle_overlap_pairs.argtypes = [V, V, V, U64, V, V, V, U64, V, V, V, U64, V, V, V, U64,
                                           C.c_int, C.c_int, C.POINTER(U64), C.POINTER(U64)]
        L.oracle_parity_pairs.restype = C.POINTER(C.c_uint64)
        L.oracle_parity_pairs.argtypes = [V, C.c_int32, V, V, V, U64, C.c_int, C.POINTER(U64)]
        L.oracle_parity_crossings.restype = C.POINTER(C.c_uint64)
        L.oracle_parity_crossings.argtypes = [V, C.c_int32, V, V, V, U64, C.POINTER(U64)]
        L.oracle_face_pairs.restype = C.POINTER(C.c_uint64)
        L.oracle_face_pairs.argtypes = [V, V, V, U64, V, V, V, U64, U64, U64, C.POINTER(U64)]
        L.oracle_overlap_pairs_reference.restype = C.POINTER(C.c_uint64)
        L.oracle_overlap_pairs_reference.argtypes = [V, V, V, U64, V, V, V, U64, V, V, V, U64, V, V, V, U64,
                                                     C.c_int, C.c_int, C.POINTER(U64)]
        L.oracle_touch_pairs.restype = C.POINTER(C.c_uint64)
        L.oracle_touch_pairs.argtypes = [V, V, V, U64, V, V, V, U64, C.POINTER(U64), C.POINTER(U64)]
        L.oracle_free.argtypes = [V]
        L.oracle_free.restype = None
        for name in ("oracle_orient3d", "oracle_orient3d_exact"):
            getattr(L, name).argtypes = [V, V, V, V]
            getattr(L, name).restype = C.c_int
        L.oracle_orient2d_xy.argtypes = [V, V, V]
        L.oracle_seg_tri.argtypes = [V, V, V, V, V, C.c_int]
        L.oracle_zray_crosses.argtypes = [V, V, V, V]
        L.oracle_exact_calls.restype = C.c_uint64
        L.oracle_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _take(ptr, n) -> np.ndarray:
    out = np.ctypeslib.as_array(ptr, shape=(max(int(n), 1),))[: int(n)].copy()
    lib().oracle_free(C.cast(ptr, V))
    return out


def keys_to_pairs(keys: np.ndarray) -> np.ndarray:
    """(a << 32 | b) uint64 keys -> (n, 2) uint32 array of (a, b)."""
    keys = np.asarray(keys, dtype=np.uint64)
    return np.stack([(keys >> np.uint64(32)).astype(np.uint32),
                     (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)], axis=1)


def pairs_to_keys(pairs: np.ndarray) -> np.ndarray:
    pairs = np.asarray(pairs).reshape(-1, 2)
    return (pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint64)


def _geom_args(g):
    v = g.vertices
    i = g.indices
    o = g.tri_to_object
    return (v.ctypes.data, i.ctypes.data, o.ctypes.data, i.shape[0]), (v, i, o)


def _edge_args(g):
    s, e, o = g.edge_starts, g.edge_ends, g.edge_src
    return (s.ctypes.data, e.ctypes.data, o.ctypes.data, o.shape[0]), (s, e, o)


def overlap_keys(A, B, direction: int = 0, mode: int = 0):
    """Sorted unique (a<<32|b) keys of the overlap join and the number of
    triangle tests performed.  mode 0 exact, 1 float32 Moller-Trumbore."""
    (ga, ka), (gb, kb) = _geom_args(A), _geom_args(B)
    (ea, kea), (eb, keb) = _edge_args(A), _edge_args(B)
    n, tests = U64(), U64()
    ptr = lib().oracle_overlap_pairs(*ga, *ea, *gb, *eb, direction, mode, C.byref(n), C.byref(tests))
    return _take(ptr, n.value), tests.value


def overlap_keys_reference(A, B, max_iterations: int = 100, direction: int = 0) -> np.ndarray:
    """Overlap keys under the reference's edge-ray semantics: hits at an
    edge's start point and rays in a triangle's plane are not seen, hits at
    one t count once, at most max_iterations hits per edge
    (pierce/query/src/cuda/mesh_overlap_edges.cu:105-176)."""
    (ga, ka), (gb, kb) = _geom_args(A), _geom_args(B)
    (ea, kea), (eb, keb) = _edge_args(A), _edge_args(B)
    n = U64()
    ptr = lib().oracle_overlap_pairs_reference(*ga, *ea, *gb, *eb, direction, max_iterations, C.byref(n))
    return _take(ptr, n.value)


def reference_semantics_diff(A, B, max_iterations: int = 100) -> dict:
    """|exact set Δ reference-semantics set| of the overlap join."""
    exact, _ = overlap_keys(A, B)
    ref = overlap_keys_reference(A, B, max_iterations)
    return {"max_iterations": int(max_iterations), "exact_pairs": int(len(exact)), "reference_pairs": int(len(ref)),
            "only_exact": int(len(np.setdiff1d(exact, ref))), "only_reference": int(len(np.setdiff1d(ref, exact)))}


def parity_keys(first_vertices: np.ndarray, T, swap: int = 0) -> np.ndarray:
    fv = _f32(first_vertices).reshape(-1, 3)
    gt, keep = _geom_args(T)
    n = U64()
    ptr = lib().oracle_parity_pairs(fv.ctypes.data, fv.shape[0], *gt, swap, C.byref(n))
    return _take(ptr, n.value)


def parity_crossings(first_vertices: np.ndarray, T) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(source, target, crossings) of every target object the +Z ray from
    each source first vertex crosses, sorted by (source, target)."""
    fv = _f32(first_vertices).reshape(-1, 3)
    gt, keep = _geom_args(T)
    n = U64()
    ptr = lib().oracle_parity_crossings(fv.ctypes.data, fv.shape[0], *gt, C.byref(n))
    words = _take(ptr, 2 * n.value).reshape(-1, 2)
    keys = words[:, 0]
    return ((keys >> np.uint64(32)).astype(np.int32), (keys & np.uint64(0xFFFFFFFF)).astype(np.int32),
            words[:, 1].astype(np.int64))


def face_keys(A, B, tri_begin: int = 0, tri_end: int | None = None) -> np.ndarray:
    (ga, ka), (gb, kb) = _geom_args(A), _geom_args(B)
    if tri_end is None:
        tri_end = A.num_triangles
    n = U64()
    ptr = lib().oracle_face_pairs(*ga, *gb, tri_begin, tri_end, C.byref(n))
    return _take(ptr, n.value)


def touch_keys(A, B) -> tuple[np.ndarray, int]:
    """TOUCH baseline restated (baselines/face/src/touch_query.cpp): sorted
    unique overlap keys and the number of candidate pairs it refined."""
    (ga, ka), (gb, kb) = _geom_args(A), _geom_args(B)
    n, cand = U64(), U64()
    ptr = lib().oracle_touch_pairs(*ga, *gb, C.byref(n), C.byref(cand))
    return _take(ptr, n.value), cand.value


def intersection_keys(A, B) -> np.ndarray:
    """S_surf U parity(A first vertex in B) U parity(B first vertex in A)."""
    surf, _ = overlap_keys(A, B)
    pa = parity_keys(A.first_vertices(), B, swap=0)
    pb = parity_keys(B.first_vertices(), A, swap=1)
    return np.unique(np.concatenate([surf, pa, pb]))


def containment_keys(A, B) -> np.ndarray:
    """(a, b) with B's first vertex inside A by parity and (a, b) not in S_surf."""
    surf, _ = overlap_keys(A, B)
    pb = parity_keys(B.first_vertices(), A, swap=1)
    return np.setdiff1d(pb, surf, assume_unique=True)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def grid_estimate(cells_a: np.ndarray, cells_b: np.ndarray, cell_size: float, epsilon: float, gamma: float,
                  alpha_correction: bool = True) -> tuple[float, int, int]:
    """Grid selectivity estimate of the reference, restated in numpy:
    (raw sum over matched cells, alpha-corrected estimate, matched cells).

    Cells of B are matched with the cell of A of the same index
    (pierce/query/src/applications/pierce_overlap_main.cpp:376-414); each
    matched pair contributes touchA * touchB * min(1, (sizeA + sizeB + eps)^3
    / cellVolume * sqrt(ratioA * ratioB)^gamma), evaluated in float32 in the
    kernel's order (pierce/query/src/cuda/estimated_overlap.cu:8-41, the
    same in estimated_intersection.cu:8-42).  The raw sum is taken exactly
    here (the reference reduces in float32, in the order of its reduction).
    The estimate divides the float32 sum by alpha = max(1, (effA + effB)^3 /
    cellVolume), eff = touch-weighted mean size * cbrt(touch-weighted mean
    volume ratio) over all cells of a side (pierce_overlap_main.cpp:431-451,
    pierce_intersection_main.cpp:181-211), and truncates."""
    import math
    f = np.float32
    a = np.asarray(cells_a)
    b = np.asarray(cells_b)
    index_a = {(int(c["ix"]), int(c["iy"]), int(c["iz"])): k for k, c in enumerate(a)}
    pairs = [(index_a[(int(c["ix"]), int(c["iy"]), int(c["iz"]))], k) for k, c in enumerate(b)
             if (int(c["ix"]), int(c["iy"]), int(c["iz"])) in index_a]
    vol = f(cell_size) * f(cell_size) * f(cell_size)
    terms = []
    for ka, kb in pairs:
        A, B = a[ka], b[kb]
        if A["touch_count"] == 0 or B["touch_count"] == 0:
            continue
        comb = f(f(A["avg_size_mean"]) + f(B["avg_size_mean"])) + f(epsilon)
        prob = (comb * comb * comb) / vol
        ratio = np.sqrt(f(A["vol_ratio"]) * f(B["vol_ratio"]))
        prob = f(prob * np.power(ratio, f(gamma)))
        prob = min(prob, f(1.0))
        terms.append(float(f(f(A["touch_count"]) * f(B["touch_count"])) * prob))
    raw = math.fsum(terms)

    def avg(c, field, empty):
        t = c["touch_count"].astype(np.float64)
        if t.sum() == 0:
            return f(empty)
        return f(float(np.sum(c[field].astype(np.float64) * t)) / float(t.sum()))

    eff = [avg(c, "avg_size_mean", 0.0) * np.cbrt(avg(c, "vol_ratio", 1.0)) for c in (a, b)]
    comb = f(eff[0] + eff[1])
    vol = max(vol, f(1e-9))
    alpha = f(1.0)
    if alpha_correction:
        alpha = max(f((comb * comb * comb) / vol), f(1.0))
    return raw, int(f(f(raw) / alpha)), len(pairs)
