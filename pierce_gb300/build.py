"""In-tree build of the native parts of pierce_gb300.

Produces, under ``pierce_gb300/_lib/``:

* ``libpierce_host.so``  – C++ host library: `.pre` I/O, edge extraction,
  grid statistics, seeded generators (``include/pierce_host.h``);
* ``libpierce_gb300.so`` – CUDA kernels for sm_103a plus the C ABI
  (``include/pierce_capi.h``);
* ``pierce_overlap``, ``pierce_overlap_two_pass``, ``pierce_intersection``,
  ``pierce_containment``, ``pierce_preprocess`` – the drop-in executables.

Every translation unit is compiled in parallel; nothing is built outside the
repository.  No cmake: plain ``g++``/``nvcc`` command lines.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
LIB = PKG / "_lib"
OBJ = PKG / "_lib" / "obj"
INCLUDE = ROOT / "include"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["pre_io.cpp", "edges.cpp", "generators.cpp", "host_capi.cpp"]
CUDA_SOURCES = ["lbvh.cu", "join.cu", "sortscan.cu", "capi.cu", "instanced.cu", "sizing.cu", "noalloc.cu"]
APP_COMMON = ["cli.cpp", "timer.cpp", "app_common.cpp", "tracking_csv.cpp"]
APPS = ["pierce_overlap", "pierce_overlap_two_pass", "pierce_intersection",
        "pierce_containment", "pierce_preprocess"]

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
            "-Wall", "-Wno-unused-function", f"-I{INCLUDE}"]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def _headers(directory: Path) -> list[Path]:
    return (sorted(directory.glob("*.h")) + sorted(directory.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
            + sorted((PKG / "host").glob("*.h")))


def _compile_host(src: Path) -> Path:
    obj = OBJ / (src.stem + ".host.o")
    if not _newer(obj, [src] + _headers(src.parent)):
        _run(["g++", *CXXFLAGS, "-c", str(src), "-o", str(obj)])
    return obj


def _compile_cuda(src: Path) -> Path:
    obj = OBJ / (src.stem + ".cu.o")
    if not _newer(obj, [src] + _headers(src.parent)):
        _run([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)])
    return obj


def build(verbose: bool = True) -> None:
    """Compile every native component (in parallel) into pierce_gb300/_lib."""
    LIB.mkdir(parents=True, exist_ok=True)
    OBJ.mkdir(parents=True, exist_ok=True)
    host_src = [PKG / "host" / s for s in HOST_SOURCES]
    cuda_src = [PKG / "csrc" / s for s in CUDA_SOURCES if (PKG / "csrc" / s).exists()]
    app_common = [PKG / "apps" / s for s in APP_COMMON if (PKG / "apps" / s).exists()]
    with cf.ThreadPoolExecutor(max_workers=max(4, os.cpu_count() or 4)) as ex:
        host_objs = list(ex.map(_compile_host, host_src))
        cuda_futs = [ex.submit(_compile_cuda, s) for s in cuda_src]
        app_common_objs = list(ex.map(_compile_host, app_common))
        cuda_objs = [f.result() for f in cuda_futs]

    host_so = LIB / "libpierce_host.so"
    if not _newer(host_so, host_objs):
        _run(["g++", "-shared", "-fopenmp", "-o", str(host_so), *map(str, host_objs)])
    gpu_so = LIB / "libpierce_gb300.so"
    if cuda_objs and not _newer(gpu_so, cuda_objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(gpu_so), *map(str, cuda_objs),
              "-lcudart_static", "-Xcompiler", "-fPIC"])

    # Applications link both libraries with an rpath to _lib.
    apps_dir = PKG / "apps"
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=max(4, os.cpu_count() or 4)) as ex:
        for app in APPS:
            src = apps_dir / f"{app}.cpp"
            if not src.exists() or not gpu_so.exists():
                continue
            out = LIB / app
            deps = [src, host_so, gpu_so, *app_common_objs] + _headers(apps_dir)
            if _newer(out, deps):
                continue
            cmd = ["g++", *CXXFLAGS, str(src), *map(str, app_common_objs), "-o", str(out),
                   f"-L{LIB}", "-lpierce_gb300", "-lpierce_host", f"-Wl,-rpath,{LIB}"]
            jobs.append(ex.submit(_run, cmd))
        for j in jobs:
            j.result()
    if verbose:
        print(f"pierce_gb300: native build complete in {LIB}", file=sys.stderr)


def clean() -> None:
    shutil.rmtree(LIB, ignore_errors=True)


if __name__ == "__main__":
    build()
