"""Loading of the in-tree native libraries.

The libraries are built in place by :mod:`pierce_gb300.build` (``__graft_entry__.build()``
calls it).  Loading never falls back to anything: if a library is missing the
caller gets an error naming it, so a missing CUDA build fails loudly instead of
silently running some other code path.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "_lib"
_lock = threading.Lock()
_host = None
_gpu = None

V = C.c_void_p
I32 = C.c_int32
U32 = C.c_uint32
I64 = C.c_int64
U64 = C.c_uint64
D = C.c_double
F = C.c_float


class NativeLibraryMissing(RuntimeError):
    pass


def _load(name: str) -> C.CDLL:
    path = LIB_DIR / name
    if not path.exists():
        raise NativeLibraryMissing(
            f"{path} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` first")
    return C.CDLL(str(path))


def _sig(lib, name, restype, argtypes):
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = argtypes


def host() -> C.CDLL:
    global _host
    with _lock:
        if _host is None:
            lib = _load("libpierce_host.so")
            _sig(lib, "pierce_host_last_error", C.c_char_p, [])
            _sig(lib, "pierce_geom_create", C.c_int, [V, U64, V, U64, V, C.POINTER(V)])
            _sig(lib, "pierce_geom_free", None, [V])
            _sig(lib, "pierce_geom_get_view", C.c_int, [V, V])
            _sig(lib, "pierce_geom_set_edges", C.c_int, [V, V, V, V, U64])
            _sig(lib, "pierce_geom_read_pre", C.c_int, [C.c_char_p, C.POINTER(V)])
            _sig(lib, "pierce_geom_write_pre", C.c_int, [V, C.c_char_p])
            _sig(lib, "pierce_geom_extract_edges", C.c_int, [V, C.c_int, C.c_int])
            _sig(lib, "pierce_geom_grid_stats", C.c_int, [V, F])
            _sig(lib, "pierce_geom_first_vertices", C.c_int, [V, V, I32])
            _sig(lib, "pierce_geom_append", C.c_int, [V, V])
            _sig(lib, "pierce_icosphere_template", C.c_int, [I32, V, V, V, V])
            _sig(lib, "pierce_gen_instances", C.c_int, [U64, I32, I32, I32, I32, D, D, D, D, D, V])
            _sig(lib, "pierce_expand_instances", C.c_int, [V, I32, C.POINTER(V)])
            _sig(lib, "pierce_gen_icospheres", C.c_int, [U64, I32, I32, D, D, D, D, C.POINTER(V)])
            _sig(lib, "pierce_gen_ellipsoid_pair", C.c_int,
                 [U64, U64, I32, I32, I32, D, D, D, D, D, D, D, D, C.POINTER(V), C.POINTER(V)])
            _sig(lib, "pierce_gen_tubes", C.c_int, [U64, I32, I64, D, D, D, D, I32, D, D, C.POINTER(V)])
            _sig(lib, "pierce_gen_tubes_head", C.c_int, [U64, I32, I32, I64, D, D, D, D, I32, D, D, C.POINTER(V)])
            _host = lib
        return _host


def gpu() -> C.CDLL:
    """The CUDA library.  Its signatures are declared by :mod:`pierce_gb300.capi`."""
    global _gpu
    with _lock:
        if _gpu is None:
            _gpu = _load("libpierce_gb300.so")
        return _gpu
