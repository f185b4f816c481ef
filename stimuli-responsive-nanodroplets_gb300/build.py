"""Build the in-tree shared library ``libscft_gb300.so`` (CUDA for sm_103a + host C).

Every translation unit is compiled in parallel into ``_build/`` and linked with
nvcc. The library is placed next to this file so that loading it never depends
on an installed copy.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libscft_gb300.so"
HOST_EXE = PKG / "scft"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]
CC_FLAGS = ["-O2", "-std=gnu11", "-fPIC", "-Wall", "-Wno-unused-result", f"-I{ROOT / 'include'}"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append([_nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("scft_*.c")):
        if src.name == "scft_main.c":
            continue
        obj = BUILD / (src.stem + ".c.o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append(["gcc", *CC_FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        _run([_nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lm"])
    return LIB


def build_host(params_dir: str | os.PathLike, out: str | os.PathLike | None = None) -> Path:
    """Compile the drop-in C host against a directory holding parameters.h.

    The host (csrc/scft_main.c) is the replacement for SCFT.c's main(): same
    compile-time parameters.h, same input and output files in the working
    directory, with the hot path on the GPU through libscft_gb300.so.
    """
    build()
    out = Path(out) if out else Path(params_dir) / "scft_gb300"
    _run(["gcc", *CC_FLAGS, f"-I{Path(params_dir).resolve()}", str(CSRC / "scft_main.c"), "-o", str(out),
          f"-L{PKG}", "-lscft_gb300", f"-Wl,-rpath,{PKG}", "-lm"])
    return out


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
