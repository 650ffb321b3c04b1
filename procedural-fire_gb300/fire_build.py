"""Builds libfiresim.so (the CUDA sm_103a kernels + the C ABI of include/fire_sim.h) in-tree.

Every translation unit is compiled in parallel with nvcc for sm_103a only, then linked into one shared
library next to this file.  The tables/geometry unit is compiled with -fmad=false so that its results
are bit-identical to the CPU oracle; the hot-path units keep FMA contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "libfiresim.so"
OBJ = HERE / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "fire_tables.cu": ["-fmad=false"],
    "fire_step.cu": [],
    "fire_mg.cu": [],
    "fire_stats.cu": [],
    "fire_api.cu": [],
    "fire_noalloc.cu": [],
    "fire_poisson.cu": [],
    "fire_sparks.cu": [],
    "fire_volume.cu": [],
    "fire_adjoint.cu": [],
    "fire_blackbody.cpp": [],
    "fire_scene.cpp": [],
    "fire_timeline.cpp": [],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise RuntimeError("nvcc not found")
    return p


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "fire_sim.h"]
    cc = nvcc()
    base = [cc, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
            *ARCH, "-I", str(HERE.parent / "include")]

    def one(item):
        src, extra = item
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        if force or _stale(o, [s, *headers, Path(__file__)]):
            cmd = base + extra + ["-c", str(s), "-o", str(o)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            if verbose:
                print(" ".join(cmd))
        return o

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, SOURCES.items()))
    if force or _stale(OUT, objs):
        cmd = [cc, "-shared", *ARCH, "-o", str(OUT), *map(str, objs), "-cudart", "shared"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
