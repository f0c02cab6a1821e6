"""The C-ABI libraries load and export every symbol their headers declare
(CPU only: no compute call is made)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from pierce_gb300 import capi, native

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def declared(header: str) -> set[str]:
    text = (INCLUDE / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(pierce_[a-z0-9_]+)\s*\(", text))
    return {n for n in names if not n.endswith("_t")}


def test_gpu_library_exports_every_declared_symbol():
    L = native.gpu()
    names = declared("pierce_capi.h")
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert names <= set(capi.SIGNATURES), sorted(names - set(capi.SIGNATURES))


def test_host_library_exports_every_declared_symbol():
    L = native.host()
    names = declared("pierce_host.h")
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_and_defaults():
    L = capi.lib()
    assert L.pierce_status_string(capi.ERR_HASH_FULL) == b"hash table full"
    o = capi.JoinOpts()
    L.pierce_default_join_opts(C.byref(o))
    assert o.hash_load_factor == 0.5 and o.output_safety == pytest.approx(1.2) and o.sizing == capi.SIZING_HASH
    t = capi.Tuning()
    L.pierce_default_tuning(C.byref(t))
    assert t.leaf_size == 1 and t.block_size == 128


def test_invalid_arguments_are_reported_without_a_device():
    L = capi.lib()
    assert L.pierce_join(None, None, None, None, None, None) == capi.ERR_INVALID_ARGUMENT
    assert b"null" in L.pierce_last_error()
    assert L.pierce_dataset_info_get(None, None) == capi.ERR_INVALID_ARGUMENT
    d = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.pierce_deduplicate_pairs_noalloc(d, capi.NOALLOC_MAX_PAIRS + 1, d, d, None) == \
        capi.ERR_INVALID_ARGUMENT
