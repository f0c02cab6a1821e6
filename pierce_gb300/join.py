"""User-facing join API over the CUDA library.

Mirrors the reference's query operations (pierce/query/src/applications/):

* :func:`overlap_join` – ``pierce_overlap`` (hash mode, executeHashQuery)
* :func:`overlap_join_two_pass` – ``pierce_overlap_two_pass``
  (executeTwoPassQueryEdgesOptimized)
* :func:`intersection_join` – ``pierce_intersection``
* :func:`containment_join` – ``pierce_containment``

Each returns the unique (mesh1 object id, mesh2 object id) pairs as an
``(n, 2)`` int32 array sorted by (a, b), plus the join statistics.  All
computation happens in ``libpierce_gb300.so``; there is no other path.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import capi
from .capi import check

PREDICATES = {"overlap": capi.OVERLAP, "intersection": capi.INTERSECTION, "containment": capi.CONTAINMENT}
DIRECTIONS = {"both": capi.BOTH, "mesh1_to_mesh2": capi.MESH1_TO_MESH2, "mesh2_to_mesh1": capi.MESH2_TO_MESH1}
SIZINGS = {"two_pass": capi.SIZING_TWO_PASS, "hash": capi.SIZING_HASH, "fixed": capi.SIZING_FIXED,
           "learned": capi.SIZING_LEARNED}
PRECISIONS = {"exact": capi.EXACT, "fp32": capi.FP32}


class Context:
    """One CUDA device + stream; all datasets and joins of a context run on it."""

    def __init__(self, device: int = 0):
        self._lib = capi.lib()
        h = C.c_void_p()
        check(self._lib.pierce_ctx_create(device, C.byref(h)), "ctx_create")
        self._h = h
        self.device = int(device)
        self._children = weakref.WeakSet()

    def adopt(self, child) -> None:
        """Register an object (dataset, sizing network) released before the context."""
        self._children.add(child)

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(self._lib.pierce_ctx_stream(self._h) or 0)

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.pierce_ctx_kernel_launches(self._h))

    def synchronize(self) -> None:
        check(self._lib.pierce_ctx_synchronize(self._h), "synchronize")

    def release_scratch(self) -> None:
        """Free the join scratch memory the context keeps between joins."""
        check(self._lib.pierce_ctx_release_scratch(self._h), "release_scratch")

    def device_memory(self) -> tuple[int, int]:
        """(free, total) bytes of the context's device."""
        f, t = C.c_uint64(), C.c_uint64()
        check(self._lib.pierce_device_memory(self._h, C.byref(f), C.byref(t)), "device_memory")
        return int(f.value), int(t.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            for child in list(getattr(self, "_children", ())):
                child.close()
            self._lib.pierce_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def default_tuning(**kw) -> capi.Tuning:
    t = capi.Tuning()
    capi.lib().pierce_default_tuning(C.byref(t))
    for k, v in kw.items():
        setattr(t, k, v)
    return t


class Dataset:
    """A dataset resident on the device with its BVH."""

    def __init__(self, ctx: Context, handle, keep=None):
        self.ctx = ctx
        self._h = handle
        self._keep = keep
        self._lib = capi.lib()
        ctx.adopt(self)

    @classmethod
    def from_arrays(cls, ctx: Context, vertices, indices, tri_to_object, edge_starts, edge_ends, edge_src,
                    num_objects: int = -1, tuning: capi.Tuning | None = None,
                    object_offsets=None) -> "Dataset":
        """A dataset from host arrays.  With `object_offsets` (num_objects + 1
        triangle offsets of a mesh stored object by object) the per-triangle
        object ids are written on the device and `tri_to_object` may be None."""
        t2o = np.zeros(0, np.int32) if tri_to_object is None else tri_to_object
        arrs = [np.ascontiguousarray(vertices, np.float32), np.ascontiguousarray(indices, np.uint32),
                np.ascontiguousarray(t2o, np.int32), np.ascontiguousarray(edge_starts, np.float32),
                np.ascontiguousarray(edge_ends, np.float32), np.ascontiguousarray(edge_src, np.int32)]
        v = capi.MeshView()
        v.vertices, v.num_vertices = arrs[0].ctypes.data, arrs[0].size // 3
        v.indices, v.num_triangles = arrs[1].ctypes.data, arrs[1].size // 3
        v.tri_to_object = arrs[2].ctypes.data if tri_to_object is not None else None
        v.edge_starts, v.edge_ends, v.edge_src = arrs[3].ctypes.data, arrs[4].ctypes.data, arrs[5].ctypes.data
        v.num_edges = arrs[5].size
        v.num_objects = num_objects
        if object_offsets is not None:
            off = np.ascontiguousarray(object_offsets, np.int64)
            arrs.append(off)
            v.object_offsets = off.ctypes.data
        h = C.c_void_p()
        t = tuning if tuning is not None else default_tuning()
        check(capi.lib().pierce_dataset_create(ctx.handle, C.byref(v), capi.HOST_MEMORY, C.byref(t), C.byref(h)),
              "dataset_create")
        return cls(ctx, h)

    @classmethod
    def from_geometry(cls, ctx: Context, geom, tuning: capi.Tuning | None = None) -> "Dataset":
        if not geom.has_edges:
            raise ValueError("geometry carries no precomputed edges; run extract_edges() first")
        return cls.from_arrays(ctx, geom.vertices, geom.indices, geom.tri_to_object, geom.edge_starts,
                               geom.edge_ends, geom.edge_src, geom.num_objects, tuning)

    @classmethod
    def from_device(cls, ctx: Context, view: capi.MeshView, tuning: capi.Tuning | None = None) -> "Dataset":
        h = C.c_void_p()
        t = tuning if tuning is not None else default_tuning()
        check(capi.lib().pierce_dataset_create(ctx.handle, C.byref(view), capi.DEVICE_MEMORY, C.byref(t),
                                               C.byref(h)), "dataset_create(device)")
        return cls(ctx, h)

    @classmethod
    def from_instances(cls, ctx: Context, inst: np.ndarray, tuning: capi.Tuning | None = None) -> "Dataset":
        """Expand instanced meshes directly on the device."""
        inst = np.ascontiguousarray(inst, dtype=capi.INSTANCE_DTYPE)
        h = C.c_void_p()
        t = tuning if tuning is not None else default_tuning()
        check(capi.lib().pierce_dataset_create_instanced(ctx.handle, inst.ctypes.data if len(inst) else None,
                                                         len(inst), C.byref(t), C.byref(h)),
              "dataset_create_instanced")
        return cls(ctx, h)

    def build(self, tuning: capi.Tuning | None = None) -> None:
        t = tuning if tuning is not None else default_tuning()
        check(self._lib.pierce_dataset_build(self.ctx.handle, self._h, C.byref(t)), "dataset_build")

    def set_partitions(self, obj_part, num_parts: int) -> None:
        """Partition the objects: joins then pair partition p of A with
        partition p of B only (a batch of independent joins)."""
        part = np.ascontiguousarray(obj_part, np.int32)
        check(self._lib.pierce_dataset_set_partitions(self.ctx.handle, self._h, part.ctypes.data if len(part) else None,
                                                      int(num_parts)), "dataset_set_partitions")

    def download(self) -> dict:
        """The dataset's arrays, copied back to host memory."""
        i = self.info()
        out = {"vertices": np.zeros((i.num_vertices, 3), np.float32),
               "indices": np.zeros((i.num_triangles, 3), np.uint32),
               "tri_to_object": np.zeros(i.num_triangles, np.int32),
               "edge_starts": np.zeros((i.num_edges, 3), np.float32),
               "edge_ends": np.zeros((i.num_edges, 3), np.float32),
               "edge_src": np.zeros(i.num_edges, np.int32)}
        check(self._lib.pierce_dataset_download(self.ctx.handle, self._h, *[a.ctypes.data for a in out.values()]),
              "dataset_download")
        out["num_objects"] = i.num_objects
        return out

    def info(self) -> capi.DatasetInfo:
        i = capi.DatasetInfo()
        check(self._lib.pierce_dataset_info_get(self._h, C.byref(i)), "dataset_info")
        return i

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pierce_dataset_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


@dataclass
class ParityTracking:
    """Parity-ray diagnostics of one direction (source objects against
    target objects), per source object s: ids[s, :] the targets its +Z ray
    crosses an odd number of times (-1 in unused slots), hits[s, :] their
    crossing counts, crossed[s] the targets it crosses at all, overflow[s]
    the odd targets beyond the slots."""
    ids: np.ndarray        # (n, max_targets) int32
    hits: np.ndarray       # (n, max_targets) uint32
    crossed: np.ndarray    # (n,) uint32
    overflow: np.ndarray   # (n,) uint32


def parity_tracking(ctx: Context, src: Dataset, tgt: Dataset, max_targets: int = 256) -> ParityTracking:
    """The parity rays of src's objects against tgt's, as the reference's
    --enable-tracking buffers hold them (pierce_parity_tracking)."""
    n = max(src.info().num_objects, 0)
    ids = np.full((n, max_targets), -1, np.int32)
    hits = np.zeros((n, max_targets), np.uint32)
    crossed = np.zeros(n, np.uint32)
    overflow = np.zeros(n, np.uint32)
    if n:
        check(capi.lib().pierce_parity_tracking(ctx.handle, src.handle, tgt.handle, int(max_targets),
                                                ids.ctypes.data, hits.ctypes.data, crossed.ctypes.data,
                                                overflow.ctypes.data), "parity_tracking")
    return ParityTracking(ids, hits, crossed, overflow)


@dataclass
class JoinResult:
    pairs: np.ndarray          # (n, 2) int32, sorted by (a, b)
    stats: dict
    containment_count: int = 0


def object_offsets(tri_to_object, num_objects: int):
    """Triangle offsets (num_objects + 1, int64) of a mesh stored object by
    object (object ids non-decreasing over the triangles), or None."""
    t2o = np.asarray(tri_to_object)
    if len(t2o) and (np.any(np.diff(t2o) < 0) or t2o[0] < 0 or t2o[-1] >= num_objects):
        return None
    off = np.zeros(num_objects + 1, np.int64)
    np.cumsum(np.bincount(t2o, minlength=num_objects), out=off[1:])
    return off


def make_opts(predicate="overlap", direction="both", sizing="hash", precision="exact", expected_pairs=0,
              hash_table_slots=0, hash_load_factor=0.5, output_safety=1.2, include_overlap_pairs=False,
              max_retries=4, cull_objects=True, defer_exact=True, active_bvh=True,
              sizing_model=None, leaf_size=0, rays_per_warp=0, stack_depth=0,
              traversal="per_ray", edge_source="auto", shard_index=0, shard_count=1) -> capi.JoinOpts:
    o = capi.JoinOpts()
    capi.lib().pierce_default_join_opts(C.byref(o))
    o.predicate = PREDICATES[predicate] if isinstance(predicate, str) else int(predicate)
    o.direction = DIRECTIONS[direction] if isinstance(direction, str) else int(direction)
    o.sizing = SIZINGS[sizing] if isinstance(sizing, str) else int(sizing)
    o.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    o.expected_pairs = int(expected_pairs)
    o.hash_table_slots = int(hash_table_slots)
    o.hash_load_factor = float(hash_load_factor)
    o.output_safety = float(output_safety)
    o.include_overlap_pairs = 1 if include_overlap_pairs else 0
    o.max_retries = int(max_retries)
    o.cull_objects = 1 if cull_objects else 0
    o.defer_exact = 1 if defer_exact else 0
    o.active_bvh = 1 if active_bvh else 0
    o.sizing_model = sizing_model.handle if sizing_model is not None else None
    o.leaf_size, o.rays_per_warp, o.stack_depth = int(leaf_size), int(rays_per_warp), int(stack_depth)
    o.traversal = ({"per_ray": 0, "packets": 1, "per_ray_binary": 2}[traversal] if isinstance(traversal, str)
                   else int(traversal))
    o.edge_source = ({"auto": 0, "dataset": 1, "triangles": 2}[edge_source] if isinstance(edge_source, str)
                     else int(edge_source))
    o.shard_index, o.shard_count = int(shard_index), int(shard_count)
    return o


def autotune(ctx: Context, a: Dataset, b: Dataset, opts: capi.JoinOpts, repeats: int = 2):
    """The library's autotuner: returns (best setting, all trials) as dicts."""
    best = capi.Tuned()
    trials = (capi.Tuned * 64)()
    n = C.c_int32()
    check(capi.lib().pierce_autotune_join(ctx.handle, a.handle, b.handle, C.byref(opts), int(repeats),
                                          C.byref(best), trials, 64, C.byref(n)), "autotune_join")
    as_dict = lambda t: {k: getattr(t, k) for k, _ in t._fields_}
    return as_dict(best), [as_dict(trials[i]) for i in range(min(n.value, 64))]


def tuned_opts(opts: capi.JoinOpts, best: dict) -> capi.JoinOpts:
    o = capi.JoinOpts.from_buffer_copy(opts)
    o.leaf_size, o.rays_per_warp = int(best["leaf_size"]), int(best["rays_per_warp"])
    o.stack_depth, o.hash_load_factor = int(best["stack_depth"]), float(best["hash_load_factor"])
    o.traversal = int(best.get("traversal", 0))
    o.edge_source = int(best.get("edge_source", o.edge_source))
    return o


def run_join(ctx: Context, a: Dataset, b: Dataset, opts: capi.JoinOpts, download: bool = True):
    """Run one join; returns (JoinResult, result handle or None)."""
    L = capi.lib()
    r = C.c_void_p()
    st = capi.Stats()
    check(L.pierce_join(ctx.handle, a.handle, b.handle, C.byref(opts), C.byref(r), C.byref(st)), "join")
    try:
        n = C.c_uint64()
        check(L.pierce_result_count(r, C.byref(n)), "result_count")
        nc = C.c_uint64()
        check(L.pierce_result_containment_count(r, C.byref(nc)), "result_containment_count")
        pairs = np.zeros((n.value, 2), dtype=np.int32)
        if download and n.value:
            check(L.pierce_result_copy(ctx.handle, r, pairs.ctypes.data, n.value), "result_copy")
        return JoinResult(pairs, st.as_dict(), int(nc.value))
    finally:
        L.pierce_result_destroy(r)


class JoinGraph:
    """A join captured as one CUDA graph: planned by an eager run, then
    replayed with one launch per call (same datasets, same result)."""

    def __init__(self, ctx: Context, a: Dataset, b: Dataset, opts: capi.JoinOpts):
        self.ctx, self._a, self._b, self._opts = ctx, a, b, opts
        self._lib = capi.lib()
        h = C.c_void_p()
        st = capi.Stats()
        check(self._lib.pierce_join_graph_create(ctx.handle, a.handle, b.handle, C.byref(opts), C.byref(h),
                                                 C.byref(st)), "join_graph_create")
        self._h = h
        self.plan_stats = st.as_dict()
        ctx.adopt(self)

    def launch(self) -> dict:
        st = capi.Stats()
        check(self._lib.pierce_join_graph_launch(self.ctx.handle, self._h, C.byref(st)), "join_graph_launch")
        return st.as_dict()

    def pairs(self) -> np.ndarray:
        p, n = C.c_void_p(), C.c_uint64()
        check(self._lib.pierce_join_graph_pairs(self._h, C.byref(p), C.byref(n)), "join_graph_pairs")
        out = np.zeros((n.value, 2), np.int32)
        if n.value:
            check(self._lib.pierce_join_graph_copy(self.ctx.handle, self._h, out.ctypes.data, n.value),
                  "join_graph_copy")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pierce_join_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def join(ctx: Context, a: Dataset, b: Dataset, **kw) -> JoinResult:
    return run_join(ctx, a, b, make_opts(**kw))


def overlap_join(ctx, a, b, **kw) -> JoinResult:
    kw.setdefault("sizing", "hash")
    return join(ctx, a, b, predicate="overlap", **kw)


def overlap_join_two_pass(ctx, a, b, **kw) -> JoinResult:
    return join(ctx, a, b, predicate="overlap", sizing="two_pass", **kw)


def intersection_join(ctx, a, b, **kw) -> JoinResult:
    return join(ctx, a, b, predicate="intersection", **kw)


def containment_join(ctx, a, b, **kw) -> JoinResult:
    return join(ctx, a, b, predicate="containment", **kw)


def pairs_to_keys(pairs: np.ndarray) -> np.ndarray:
    p = np.asarray(pairs).reshape(-1, 2)
    return (p[:, 0].astype(np.uint32).astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint32).astype(np.uint64)
