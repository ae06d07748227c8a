"""In-tree build of libmarie_gb300.so for sm_103a (nvcc, no cmake).

Each translation unit is compiled in parallel, then linked into a shared
library beside this file (``lib/libmarie_gb300.so``).  A stamp of the source
hashes avoids rebuilding when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libmarie_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmarie_gb300")
    return cand


# Sources compiled more than once with different macros: one object each.
# The float-float z-pass kernels are split by NB = n3/16 so that the eight
# objects compile in parallel (together they take many minutes).
VARIANTS = {"fast_ff_z.cu": [(f"fast_ff_z{nb}", [f"-DMARIE_FF_NB={nb}"]) for nb in range(1, 9)]}


def _sources():
    """(source, object stem, extra flags) of every object in the library."""
    out = []
    for src in sorted(CSRC.glob("*.cu")):
        for stem, extra in VARIANTS.get(src.name, [(src.stem, [])]):
            out.append((src, stem, extra))
    return out


def _stamp() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA source and link the shared library; return its path."""
    LIBDIR.mkdir(exist_ok=True)
    stamp_file = LIBDIR / "build.stamp"
    stamp = _stamp()
    if not force and LIB.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    nvcc = _nvcc()
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)

    def compile_one(item) -> Path:
        src, stem, extra = item
        obj = objdir / (stem + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, *extra, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        # the four-step kernel units are the slowest: start them first
        order = sorted(srcs, key=lambda it: (not it[1].startswith("fast"), it[1]))
        objs = list(ex.map(compile_one, order))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lcublas"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
