"""Build recipes for the oracle (TEST INFRASTRUCTURE).

build_oracle()    -> oracle/_build/liboracle.so: the C restatement
                     (scft_oracle.c) + the project FFT shim. Built on any
                     machine; the GPU machine builds it through __graft_entry__.build().
build_reference() -> oracle/_ref/<case>/: the reference SCFT.c compiled from
                     where it lies (read on stdin so that the parameters.h next
                     to the build directory is the one it includes), linked with
                     the FFT shim. Needs the reference source tree, so it only
                     runs where that tree exists; outputs never leave oracle/_ref/.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
BUILD = ORACLE / "_build"
REF_OUT = ORACLE / "_ref"
SHIM = ORACLE / "fftw_shim"
#: the reference source tree comes only from the environment (SCFT_REFERENCE_DIR)
REFERENCE_DIR = os.environ.get("SCFT_REFERENCE_DIR")
REFERENCE_SRC = Path(REFERENCE_DIR) / "SCFT.c" if REFERENCE_DIR else None
LIB = BUILD / "liboracle.so"

CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-fno-fast-math", f"-I{SHIM}"]


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [ORACLE / "scft_oracle.c", SHIM / "fft_shim.c", SHIM / "fftw3.h"]
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in srcs):
        _run(["gcc", *CFLAGS, "-shared", "-o", str(LIB), str(ORACLE / "scft_oracle.c"), str(SHIM / "fft_shim.c"),
              "-lm"])
    return LIB


def reference_available() -> bool:
    return REFERENCE_SRC is not None and REFERENCE_SRC.exists()


def build_reference(case_dir: Path, parameters_h: str, full_precision: bool = True, shared: bool = False) -> Path:
    if not reference_available():
        raise RuntimeError("the reference source tree is not available: set SCFT_REFERENCE_DIR to the directory "
                           "holding SCFT.c")
    """Compile the unmodified SCFT.c against ``parameters_h`` inside case_dir.

    full_precision appends the fprintf redirect (ref_support/precise_fprintf.c)
    so every floating output is printed with %.17g. shared builds a .so with
    main renamed, so single functions can be called (per-function checks)."""
    case_dir = Path(case_dir)
    case_dir.mkdir(parents=True, exist_ok=True)
    hdr = parameters_h
    if full_precision:
        hdr += "\n#include <stdio.h>\nint oracle_fprintf(FILE *f, const char *fmt, ...);\n#define fprintf oracle_fprintf\n"
    (case_dir / "parameters.h").write_text(hdr)
    out = case_dir / ("libscftref.so" if shared else "scft_ref")
    cmd = ["gcc", *CFLAGS, "-w", "-x", "c", "-"]
    cmd += ["-x", "none", str(SHIM / "fft_shim.c")]
    if full_precision:
        cmd.append(str(ORACLE / "ref_support" / "precise_fprintf.c"))
    if shared:
        cmd = cmd[:1] + ["-Dmain=scft_ref_main", "-shared"] + cmd[1:]
    cmd += ["-o", str(out), "-lm"]
    with open(REFERENCE_SRC, "rb") as src:
        r = subprocess.run(cmd, stdin=src, capture_output=True, cwd=case_dir)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stderr.decode()}")
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
