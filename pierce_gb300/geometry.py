"""Host-side geometry: `.pre` files, unique edges, grid statistics, generators.

Thin ctypes layer over ``libpierce_host.so`` (``include/pierce_host.h``).
A :class:`Geometry` owns a native ``pierce_geom``; its arrays are exposed as
read-only numpy views (no copies).

Reference counterparts: ``GeometryData`` (pierce/common/include/Geometry.h:42-51),
``readBinaryFile``/``writeBinaryFile`` (pierce/common/include/BinaryIO.h:32-151),
``EdgePreprocessor::extractEdges`` (pierce/preprocess/src/EdgePreprocessor.cpp:44-111).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import native

EDGE_ORDER_MAP = 0      # reference order: keys sorted (start, end, object)
EDGE_ORDER_OBJECT = 1   # same edge set grouped by object


class GeomView(C.Structure):
    _fields_ = [
        ("vertices", C.POINTER(C.c_float)), ("num_vertices", C.c_uint64),
        ("indices", C.POINTER(C.c_uint32)), ("num_triangles", C.c_uint64),
        ("tri_to_object", C.POINTER(C.c_int32)), ("num_mappings", C.c_uint64),
        ("total_triangles", C.c_uint64),
        ("edge_starts", C.POINTER(C.c_float)), ("edge_ends", C.POINTER(C.c_float)),
        ("edge_src", C.POINTER(C.c_int32)), ("num_edges", C.c_uint64),
        ("has_edges", C.c_int32), ("has_grid", C.c_int32),
        ("grid_cell_size", C.c_float), ("num_grid_cells", C.c_uint32),
        ("grid_cells", C.c_void_p), ("num_objects", C.c_int32),
    ]


GRID_DTYPE = np.dtype([("ix", "<i4"), ("iy", "<i4"), ("iz", "<i4"), ("center_count", "<u4"),
                       ("touch_count", "<u4"), ("avg_size_mean", "<f4"), ("vol_ratio", "<f4")])


class HostError(RuntimeError):
    pass


def _check(status: int, what: str) -> None:
    if status != 0:
        msg = native.host().pierce_host_last_error().decode()
        raise HostError(f"{what}: status {status}: {msg}")


def _arr(ptr, n, dtype, shape):
    if n == 0 or not ptr:
        return np.zeros(shape, dtype=dtype)
    a = np.ctypeslib.as_array(ptr, shape=(int(np.prod(shape)),))
    a = a.view(dtype).reshape(shape)
    a.flags.writeable = False
    return a


class Geometry:
    """A triangle-mesh dataset (one `.pre` file's content)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self._lib = native.host()

    # -- construction -----------------------------------------------------------
    @classmethod
    def from_arrays(cls, vertices, indices, tri_to_object) -> "Geometry":
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        t = np.ascontiguousarray(tri_to_object, dtype=np.int32).reshape(-1)
        if t.shape[0] != i.shape[0]:
            raise ValueError("tri_to_object must have one entry per triangle")
        h = C.c_void_p()
        lib = native.host()
        _check(lib.pierce_geom_create(v.ctypes.data, v.shape[0], i.ctypes.data, i.shape[0],
                                      t.ctypes.data, C.byref(h)), "geom_create")
        return cls(h)

    @classmethod
    def read_pre(cls, path) -> "Geometry":
        h = C.c_void_p()
        _check(native.host().pierce_geom_read_pre(str(path).encode(), C.byref(h)), "read_pre")
        return cls(h)

    def write_pre(self, path) -> None:
        _check(self._lib.pierce_geom_write_pre(self._h, str(path).encode()), "write_pre")

    def extract_edges(self, order: int = EDGE_ORDER_MAP, num_threads: int = 0) -> "Geometry":
        _check(self._lib.pierce_geom_extract_edges(self._h, order, num_threads), "extract_edges")
        return self

    def set_edges(self, starts, ends, src) -> None:
        s = np.ascontiguousarray(starts, dtype=np.float32).reshape(-1, 3)
        e = np.ascontiguousarray(ends, dtype=np.float32).reshape(-1, 3)
        o = np.ascontiguousarray(src, dtype=np.int32).reshape(-1)
        _check(self._lib.pierce_geom_set_edges(self._h, s.ctypes.data, e.ctypes.data, o.ctypes.data,
                                               o.shape[0]), "set_edges")

    def grid_stats(self, cell_size: float) -> "Geometry":
        _check(self._lib.pierce_geom_grid_stats(self._h, C.c_float(cell_size)), "grid_stats")
        return self

    def append(self, other: "Geometry") -> "Geometry":
        _check(self._lib.pierce_geom_append(self._h, other._h), "append")
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.pierce_geom_free(h)
            self._h = None

    # -- views --------------------------------------------------------------
    def view(self) -> GeomView:
        v = GeomView()
        _check(self._lib.pierce_geom_get_view(self._h, C.byref(v)), "get_view")
        return v

    @property
    def vertices(self) -> np.ndarray:
        v = self.view()
        return _arr(v.vertices, v.num_vertices, np.float32, (v.num_vertices, 3))

    @property
    def indices(self) -> np.ndarray:
        v = self.view()
        return _arr(v.indices, v.num_triangles, np.uint32, (v.num_triangles, 3))

    @property
    def tri_to_object(self) -> np.ndarray:
        v = self.view()
        return _arr(v.tri_to_object, v.num_mappings, np.int32, (v.num_mappings,))

    @property
    def edge_starts(self) -> np.ndarray:
        v = self.view()
        return _arr(v.edge_starts, v.num_edges, np.float32, (v.num_edges, 3))

    @property
    def edge_ends(self) -> np.ndarray:
        v = self.view()
        return _arr(v.edge_ends, v.num_edges, np.float32, (v.num_edges, 3))

    @property
    def edge_src(self) -> np.ndarray:
        v = self.view()
        return _arr(v.edge_src, v.num_edges, np.int32, (v.num_edges,))

    @property
    def grid_cells(self) -> np.ndarray:
        v = self.view()
        if not v.num_grid_cells:
            return np.zeros(0, dtype=GRID_DTYPE)
        buf = (C.c_char * (28 * v.num_grid_cells)).from_address(v.grid_cells)
        return np.frombuffer(buf, dtype=GRID_DTYPE).copy()

    @property
    def num_objects(self) -> int:
        return int(self.view().num_objects)

    @property
    def num_triangles(self) -> int:
        return int(self.view().num_triangles)

    @property
    def num_edges(self) -> int:
        return int(self.view().num_edges)

    @property
    def has_edges(self) -> bool:
        return bool(self.view().has_edges)

    def first_vertices(self) -> np.ndarray:
        n = self.num_objects
        out = np.zeros((n, 3), dtype=np.float32)
        _check(self._lib.pierce_geom_first_vertices(self._h, out.ctypes.data, n), "first_vertices")
        return out


# -- generators ------------------------------------------------------------------

def icospheres(seed: int, num_meshes: int, level: int = 3, ln_mu: float = float(np.log(1.5)),
               sigma: float = 0.3, lo: float = 0.0, hi: float = 200.0) -> Geometry:
    h = C.c_void_p()
    _check(native.host().pierce_gen_icospheres(C.c_uint64(seed), num_meshes, level, C.c_double(ln_mu),
                                               C.c_double(sigma), C.c_double(lo), C.c_double(hi),
                                               C.byref(h)), "gen_icospheres")
    return Geometry(h)


def ellipsoid_pair(seed_a: int, seed_b: int, num_a: int, num_b: int, level: int = 3,
                   axis_lo: float = 2.0, axis_hi: float = 5.0, noise_amp: float = 0.05,
                   lo: float = 0.0, hi: float = 1000.0, frac_inside: float = 0.2,
                   inside_scale: float = 0.3, frac_contact: float = 0.01):
    ha, hb = C.c_void_p(), C.c_void_p()
    _check(native.host().pierce_gen_ellipsoid_pair(
        C.c_uint64(seed_a), C.c_uint64(seed_b), num_a, num_b, level, C.c_double(axis_lo),
        C.c_double(axis_hi), C.c_double(noise_amp), C.c_double(lo), C.c_double(hi),
        C.c_double(frac_inside), C.c_double(inside_scale), C.c_double(frac_contact),
        C.byref(ha), C.byref(hb)), "gen_ellipsoid_pair")
    return Geometry(ha), Geometry(hb)


def tubes(seed: int, num_meshes: int, target_tris: int = 200_000, step: float = 1.0,
          branch_prob: float = 0.02, r_lo: float = 0.5, r_hi: float = 3.0, n_sides: int = 12,
          lo: float = 0.0, hi: float = 1000.0, first: int | None = None) -> Geometry:
    """Branching tube meshes; with `first`, only tubes 0 .. first-1 of the
    same dataset (identical coordinates and object ids)."""
    h = C.c_void_p()
    if first is None:
        _check(native.host().pierce_gen_tubes(C.c_uint64(seed), num_meshes, C.c_int64(target_tris),
                                              C.c_double(step), C.c_double(branch_prob), C.c_double(r_lo),
                                              C.c_double(r_hi), n_sides, C.c_double(lo), C.c_double(hi),
                                              C.byref(h)), "gen_tubes")
    else:
        _check(native.host().pierce_gen_tubes_head(C.c_uint64(seed), num_meshes, first, C.c_int64(target_tris),
                                                   C.c_double(step), C.c_double(branch_prob), C.c_double(r_lo),
                                                   C.c_double(r_hi), n_sides, C.c_double(lo), C.c_double(hi),
                                                   C.byref(h)), "gen_tubes_head")
    return Geometry(h)


SPHERES, ELLIPSOIDS = 0, 1


def instances(seed: int, num_meshes: int, family: int = SPHERES, level_lo: int = 3, level_hi: int | None = None,
              p0: float | None = None, p1: float | None = None, noise_amp: float = 0.05, lo: float = 0.0,
              hi: float = 200.0) -> np.ndarray:
    """Per-mesh parameters of an instanced dataset (``pierce_instance.h``).

    Spheres: radius exp(p0 + p1 N(0,1)) (defaults ln 1.5, 0.3); ellipsoids:
    semi-axes U[p0, p1] (defaults 2, 5), random rotation, radial value noise.
    Returns a record array of dtype :data:`capi.INSTANCE_DTYPE`."""
    from .capi import INSTANCE_DTYPE
    level_hi = level_lo if level_hi is None else level_hi
    if p0 is None:
        p0 = float(np.log(1.5)) if family == SPHERES else 2.0
    if p1 is None:
        p1 = 0.3 if family == SPHERES else 5.0
    out = np.zeros(num_meshes, dtype=INSTANCE_DTYPE)
    _check(native.host().pierce_gen_instances(C.c_uint64(seed), num_meshes, family, level_lo, level_hi,
                                              C.c_double(p0), C.c_double(p1), C.c_double(noise_amp),
                                              C.c_double(lo), C.c_double(hi), out.ctypes.data), "gen_instances")
    return out


def expand_instances(inst: np.ndarray) -> Geometry:
    """Host expansion of instanced meshes (edges in template order)."""
    from .capi import INSTANCE_DTYPE
    inst = np.ascontiguousarray(inst, dtype=INSTANCE_DTYPE)
    h = C.c_void_p()
    _check(native.host().pierce_expand_instances(inst.ctypes.data, len(inst), C.byref(h)), "expand_instances")
    return Geometry(h)


def write_pre_bytes(geom: Geometry, path: Path) -> bytes:
    geom.write_pre(path)
    return Path(path).read_bytes()
