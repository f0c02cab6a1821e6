"""The C-ABI libraries load and export every symbol their headers declare
(CPU only: no compute call is made)."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
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
    assert L.pierce_parity_tracking(None, None, None, 256, None, None, None, None) == capi.ERR_INVALID_ARGUMENT
    assert b"parity_tracking" in L.pierce_last_error()
    d = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.pierce_deduplicate_pairs_noalloc(d, capi.NOALLOC_MAX_PAIRS + 1, d, d, None) == \
        capi.ERR_INVALID_ARGUMENT


def _c_layout(header: str, structs: dict[str, list[str]], tmp_path: Path) -> dict[str, dict]:
    """sizeof and offsetof of each struct field as gcc lays them out from the header."""
    lines = [f'#include "{header}"', "#include <stddef.h>", "#include <stdio.h>", "int main(void) {"]
    for s, fields in structs.items():
        lines.append(f'printf("{s} size %zu\\n", sizeof({s}));')
        for f in fields:
            lines.append(f'printf("{s} {f} %zu\\n", offsetof({s}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    exe = tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", str(INCLUDE), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout: dict[str, dict] = {s: {} for s in structs}
    for line in out.splitlines():
        s, key, val = line.split()
        layout[s][key] = int(val)
    return layout


def _py_layout(t) -> dict:
    if isinstance(t, np.dtype):
        out = {name: t.fields[name][1] for name in t.names}
        out["size"] = t.itemsize
        return out
    out = {name: getattr(t, name).offset for name, _ in t._fields_}
    out["size"] = C.sizeof(t)
    return out


def _names(t) -> list[str]:
    return list(t.names) if isinstance(t, np.dtype) else [name for name, _ in t._fields_]


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_python_mirrors_match_the_c_struct_layouts(tmp_path):
    from pierce_gb300 import geometry
    mirrors = {
        "pierce_capi.h": {
            "pierce_mesh_view": capi.MeshView, "pierce_tuning": capi.Tuning,
            "pierce_join_opts": capi.JoinOpts, "pierce_stats": capi.Stats,
            "pierce_mlp_params": capi.MlpParams, "pierce_mlp_train_opts": capi.MlpTrainOpts,
            "pierce_tuned": capi.Tuned, "pierce_dataset_info": capi.DatasetInfo,
            "pierce_mesh_instance": capi.INSTANCE_DTYPE,
        },
        "pierce_host.h": {"pierce_geom_view": geometry.GeomView, "pierce_grid_entry": geometry.GRID_DTYPE},
    }
    for header, types in mirrors.items():
        layout = _c_layout(header, {s: _names(t) for s, t in types.items()}, tmp_path)
        for s, t in types.items():
            assert _py_layout(t) == layout[s], s


def test_object_offsets_of_meshes_stored_object_by_object():
    """Triangle offsets for pierce_mesh_view.object_offsets: only for object
    ids that never decrease over the triangles; empty objects give equal
    offsets."""
    from pierce_gb300 import join as J
    off = J.object_offsets(np.array([0, 0, 1, 1, 1, 3], np.int32), 4)
    assert off.dtype == np.int64 and off.tolist() == [0, 2, 5, 5, 6]
    assert J.object_offsets(np.array([0, 1, 0], np.int32), 2) is None
    assert J.object_offsets(np.array([0, 2], np.int32), 2) is None  # id past the object count
    assert J.object_offsets(np.zeros(0, np.int32), 3).tolist() == [0, 0, 0, 0]

