"""Build libgbflow.so in-tree with nvcc for sm_103a (no cmake, no torch).

Each translation unit is compiled in parallel, then linked into
_build/libgbflow.so next to this file. Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = PKG.parent / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]
# Per-file extra flags. The one-kernel-per-function path rounds every
# multiply and add separately like the CPU reference; so does the host field
# generator (the same fields on x86 and Arm, and porosity bit-identical to
# the device generator).
EXTRA = {"gbf_eager.cu": ["-fmad=false"], "gbf_fields.cpp": ["-Xcompiler", "-ffp-contract=off"]}
SOURCES = ["gbf_host.cpp", "gbf_fields.cpp", "gbf_tma.cpp", "gbf_checkpoint.cpp", "gbf_plots.cpp", "gbf_defines.cpp", "gbf_fields_gpu.cu", "gbf_eager.cu", "gbf_f64.cu", "gbf_split.cu", "gbf_domain.cu", "gbf_dropin.cu",
           "gbf_ensemble.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbflow")
    return exe


def _deps(src: pathlib.Path):
    return [src] + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _compile(src: pathlib.Path) -> pathlib.Path:
    obj = BUILD / (src.name + ".o")
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in _deps(src)):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *EXTRA.get(src.name, []), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), *COMMON, *EXTRA.get(src.name, []), "-x", "c++", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    lib = BUILD / "libgbflow.so"
    if not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-cudart", "static",
               "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(verbose=True)
