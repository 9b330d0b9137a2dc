"""Build libgpunb.so in-tree with nvcc for sm_103a (no cmake, no torch).

    python -m nbody6ppgpu_gb300.build        # or __graft_entry__.build()

Translation units are compiled in parallel, then linked into
nbody6ppgpu_gb300/libgpunb.so.  Objects go to nbody6ppgpu_gb300/_build/.
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
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libgpunb.so"
SOURCES = ["regf_kernels.cu", "pot_kernels.cu", "order_kernels.cu", "engine.cu", "noalloc.cu",
           "rsmlp.cu", "irr.cu", "peak.cu", "regcor.cu"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgpunb.so")


def _flags() -> list[str]:
    return [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O3",
            f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def _compile(src: str) -> Path:
    out = OBJ / (Path(src).stem + ".o")
    cmd = [nvcc(), *_flags(), "-c", str(CSRC / src), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return out


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list((ROOT / "include").glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libgpunb.so if any source is newer than the library."""
    if not force and not _stale():
        return LIB
    OBJ.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), GENCODE, "-shared", "-o", str(tmp), *map(str, objs),
           "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
