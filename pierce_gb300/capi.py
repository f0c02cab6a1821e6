"""ctypes binding of ``include/pierce_capi.h`` (the CUDA join library).

The structures below mirror the header field for field; the functions are
declared with exact argument types so that a wrong call fails in Python
instead of corrupting memory.  This module is the only place that talks to
``libpierce_gb300.so`` directly; :mod:`pierce_gb300.join` builds the user API
on top of it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native

V = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
U64 = C.c_uint64
D = C.c_double
F = C.c_float

# status codes
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_NO_DEVICE = 4
ERR_HASH_FULL = 5
ERR_STACK_OVERFLOW = 6
ERR_OUTPUT_OVERFLOW = 7
ERR_QUEUE_TIMEOUT = 8
ERR_NOT_BUILT = 9

HOST_MEMORY = 0
DEVICE_MEMORY = 1

OVERLAP, INTERSECTION, CONTAINMENT = 0, 1, 2
EDGES_AUTO, EDGES_DATASET, EDGES_TRIANGLES = 0, 1, 2
BOTH, MESH1_TO_MESH2, MESH2_TO_MESH1 = 0, 1, 2
SIZING_TWO_PASS, SIZING_HASH, SIZING_FIXED, SIZING_LEARNED = 0, 1, 2, 3
EXACT, FP32 = 0, 1
RAYS_COUNT, RAYS_WRITE, RAYS_HASH = 0, 1, 2
NOALLOC_TABLE_SLOTS = 1 << 22
NOALLOC_MAX_PAIRS = 1 << 21


class MeshView(C.Structure):
    _fields_ = [("vertices", V), ("num_vertices", U64), ("indices", V), ("num_triangles", U64),
                ("tri_to_object", V), ("edge_starts", V), ("edge_ends", V), ("edge_src", V),
                ("num_edges", U64), ("num_objects", I32), ("object_offsets", V)]


# pierce_mesh_instance (pierce_instance.h), as a numpy record type.
INSTANCE_DTYPE = np.dtype([("center", "<f8", (3,)), ("axes", "<f8", (3,)), ("rotation", "<f8", (9,)),
                           ("noise_amp", "<f8"), ("noise_offset", "<f8", (3,)), ("noise_seed", "<u8"),
                           ("level", "<i4"), ("group", "<i4")])
assert INSTANCE_DTYPE.itemsize == 168


class Tuning(C.Structure):
    _fields_ = [("leaf_size", I32), ("block_size", I32), ("sort_rays", I32), ("cull_objects", I32),
                ("defer_build", I32), ("skip_edges", I32)]


class JoinOpts(C.Structure):
    _fields_ = [("predicate", I32), ("direction", I32), ("sizing", I32), ("precision", I32),
                ("expected_pairs", U64), ("hash_table_slots", U64), ("hash_load_factor", D),
                ("output_safety", D), ("include_overlap_pairs", I32), ("max_retries", I32),
                ("cull_objects", I32), ("defer_exact", I32), ("active_bvh", I32), ("sizing_model", V),
                ("leaf_size", I32), ("rays_per_warp", I32), ("stack_depth", I32), ("traversal", I32),
                ("edge_source", I32), ("shard_index", I32), ("shard_count", I32), ("reserved", I32)]


class Stats(C.Structure):
    _fields_ = [("ms_total", D), ("ms_edge_rays", D * 2), ("ms_parity", D * 2), ("ms_dedup", D),
                ("rays", U64), ("node_visits", U64), ("tri_tests", U64), ("raw_hits", U64),
                ("fp32_ambiguous", U64), ("fp64_ambiguous", U64), ("parity_rays", U64),
                ("hash_slots", U64), ("result_capacity", U64), ("num_pairs", U64),
                ("overlap_pairs", U64), ("containment_pairs", U64), ("retries", I32),
                ("launches", I32), ("ms_count_pass", D * 2), ("raw_pairs", U64 * 2),
                ("hash_accesses", U64), ("hash_contentions", U64), ("ms_build", D),
                ("active_triangles", U64 * 2), ("predicted_pairs", D), ("ms_sizing", D),
                ("sizing_overflow", I32), ("containment_by_pairs", I32)]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


MLP_INPUTS, MLP_HIDDEN = 32, 64
MLP_PARAMS = MLP_HIDDEN * MLP_INPUTS + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN + 1


class MlpParams(C.Structure):
    _fields_ = [("weights", F * MLP_PARAMS), ("x_mean", F * MLP_INPUTS), ("x_scale", F * MLP_INPUTS),
                ("y_mean", F), ("y_std", F)]


class MlpTrainOpts(C.Structure):
    _fields_ = [("seed", U64), ("epochs", I32), ("fit_normalization", I32), ("lr", F), ("beta1", F),
                ("beta2", F), ("eps", F)]


class Tuned(C.Structure):
    _fields_ = [("leaf_size", I32), ("rays_per_warp", I32), ("stack_depth", I32), ("traversal", I32),
                ("edge_source", I32), ("reserved", I32), ("hash_load_factor", D), ("ms", D)]


class DatasetInfo(C.Structure):
    _fields_ = [("num_vertices", U64), ("num_triangles", U64), ("num_edges", U64),
                ("num_objects", I32), ("built", I32), ("num_nodes", U64), ("device_bytes", U64),
                ("ms_build", D), ("bounds_lo", F * 3), ("bounds_hi", F * 3), ("num_parts", I32),
                ("objects_contiguous", I32), ("reserved", I32)]


# Every symbol the header declares, with its signature.
SIGNATURES = {
    "pierce_last_error": (C.c_char_p, []),
    "pierce_status_string": (C.c_char_p, [C.c_int]),
    "pierce_ctx_create": (C.c_int, [C.c_int, C.POINTER(V)]),
    "pierce_ctx_destroy": (None, [V]),
    "pierce_ctx_synchronize": (C.c_int, [V]),
    "pierce_ctx_stream": (V, [V]),
    "pierce_default_tuning": (None, [C.POINTER(Tuning)]),
    "pierce_default_join_opts": (None, [C.POINTER(JoinOpts)]),
    "pierce_ctx_kernel_launches": (U64, [V]),
    "pierce_device_memory": (C.c_int, [V, C.POINTER(U64), C.POINTER(U64)]),
    "pierce_ctx_release_scratch": (C.c_int, [V]),
    "pierce_dataset_create": (C.c_int, [V, C.POINTER(MeshView), C.c_int, C.POINTER(Tuning), C.POINTER(V)]),
    "pierce_dataset_build": (C.c_int, [V, V, C.POINTER(Tuning)]),
    "pierce_dataset_create_instanced": (C.c_int, [V, V, I32, C.POINTER(Tuning), C.POINTER(V)]),
    "pierce_dataset_download": (C.c_int, [V, V, V, V, V, V, V, V]),
    "pierce_dataset_set_partitions": (C.c_int, [V, V, V, I32]),
    "pierce_dataset_info_get": (C.c_int, [V, C.POINTER(DatasetInfo)]),
    "pierce_dataset_destroy": (None, [V]),
    "pierce_join": (C.c_int, [V, V, V, C.POINTER(JoinOpts), C.POINTER(V), C.POINTER(Stats)]),
    "pierce_result_count": (C.c_int, [V, C.POINTER(U64)]),
    "pierce_result_device_pairs": (V, [V]),
    "pierce_result_copy": (C.c_int, [V, V, V, U64]),
    "pierce_result_containment_count": (C.c_int, [V, C.POINTER(U64)]),
    "pierce_result_destroy": (None, [V]),
    "pierce_autotune_join": (C.c_int, [V, V, V, C.POINTER(JoinOpts), I32, C.POINTER(Tuned), V, I32,
                                       C.POINTER(I32)]),
    "pierce_join_graph_create": (C.c_int, [V, V, V, C.POINTER(JoinOpts), C.POINTER(V), C.POINTER(Stats)]),
    "pierce_join_graph_launch": (C.c_int, [V, V, C.POINTER(Stats)]),
    "pierce_join_graph_pairs": (C.c_int, [V, C.POINTER(V), C.POINTER(U64)]),
    "pierce_join_graph_copy": (C.c_int, [V, V, V, U64]),
    "pierce_join_graph_destroy": (None, [V]),
    "pierce_launch_edge_rays": (C.c_int, [V, V, V, C.c_int, C.c_int, C.c_int, V, V, V, V, U64,
                                          C.POINTER(Stats)]),
    "pierce_launch_parity": (C.c_int, [V, V, V, C.c_int, C.c_int, V, V, U64, C.POINTER(Stats)]),
    "pierce_parity_tracking": (C.c_int, [V, V, V, I32, V, V, V, V]),
    "pierce_exclusive_scan": (C.c_int, [V, V, V, I64, C.POINTER(I64)]),
    "pierce_merge_and_deduplicate_pairs": (C.c_int, [V, V, I64, V, I64, V, C.POINTER(I64)]),
    "pierce_compact_hash_table_pairs": (C.c_int, [V, V, U64, V, U64, C.POINTER(U64)]),
    "pierce_deduplicate_pairs_noalloc": (C.c_int, [V, I64, V, V, V]),
    "pierce_default_mlp_train_opts": (None, [C.POINTER(MlpTrainOpts)]),
    "pierce_mlp_init_params": (C.c_int, [C.POINTER(MlpParams), U64]),
    "pierce_mlp_create": (C.c_int, [V, C.POINTER(MlpParams), C.POINTER(V)]),
    "pierce_mlp_destroy": (None, [V]),
    "pierce_mlp_get": (C.c_int, [V, V, C.POINTER(MlpParams)]),
    "pierce_mlp_train": (C.c_int, [V, V, V, V, I32, C.POINTER(MlpTrainOpts), V]),
    "pierce_mlp_gradient": (C.c_int, [V, V, V, V, I32, V, V]),
    "pierce_mlp_predict": (C.c_int, [V, V, V, I32, V]),
    "pierce_join_features": (C.c_int, [V, V, V, V]),
    "pierce_estimate_pairs": (C.c_int, [V, V, C.c_uint32, V, C.c_uint32, F, F, F, C.c_int,
                                        C.POINTER(D), C.POINTER(I64), C.POINTER(I32)]),
}

_bound = None


def lib() -> C.CDLL:
    """The CUDA library with all signatures declared (raises if unbuilt)."""
    global _bound
    if _bound is None:
        L = native.gpu()
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _bound = L
    return _bound


class PierceError(RuntimeError):
    def __init__(self, status: int, what: str):
        L = lib()
        self.status = status
        msg = L.pierce_last_error().decode(errors="replace")
        super().__init__(f"{what}: {L.pierce_status_string(status).decode()} ({status}): {msg}")


def check(status: int, what: str) -> None:
    if status != OK:
        raise PierceError(status, what)
