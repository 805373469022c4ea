"""Build libgomcore.so (CUDA, sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel and linked into one shared library with a plain C
ABI (include/gom_core.h); nothing here depends on PyTorch.  ``-fmad=false`` keeps every FP64
multiply and add separately rounded, as in the CPU restatement of the reference.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
SOURCES = ["gom_core.cu", "k_hydro.cu", "k_surface.cu", "k_transport.cu", "k_forcing.cu", "gom_noalloc.cu",
           "gom_measure.cu", "k_geometry.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_core(verbose: bool = False, extra: list[str] | None = None) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    nv = nvcc()
    extra = extra or []
    headers = [CSRC / h for h in ("gom_device.cuh", "gom_launch.h", "gom_pcg.cuh")] + [PKG.parent / "include" / "gom_core.h"]
    hdr_mtime = max(h.stat().st_mtime for h in headers)

    def compile_one(src):
        obj = OUT / (Path(src).stem + ".o")
        srcp = CSRC / src
        if obj.exists() and obj.stat().st_mtime > max(srcp.stat().st_mtime, hdr_mtime) and not extra:
            return ""
        cmd = [nv, *ARCH, *NVCC_FLAGS, *extra, "-c", str(srcp), "-o", str(obj)]
        return _run(cmd)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        logs = list(ex.map(compile_one, SOURCES))
    if verbose:
        for l in logs:
            if l:
                print(l)
    so = OUT / "libgomcore.so"
    tmp = OUT / "libgomcore.so.tmp"
    objs = [str(OUT / (Path(s).stem + ".o")) for s in SOURCES]
    _run([nv, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"])
    os.replace(tmp, so)
    return so


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else None
    print(build_core(verbose=v or bool(extra), extra=extra))
