"""Build the engine's native libraries in-tree (nvcc for sm_103a, g++ for the host emulation).

``build()`` compiles every CUDA translation unit of ``csrc/`` in parallel, links
``_lib/libspi_engine.so`` and builds ``_lib/libspi_hostemu.so``. A stamp of the
sources, flags and machine keeps repeated calls cheap.
"""
from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
LIB_DIR = PKG / "_lib"
ENGINE_SO = LIB_DIR / "libspi_engine.so"
HOSTEMU_SO = LIB_DIR / "libspi_hostemu.so"

CU_SOURCES = ("engine.cu", "items.cu", "cem.cu", "server.cu", "sensitivity.cu", "step.cu", "probe.cu", "noalloc.cu", "fd_fisher.cu", "search.cu", "adjoint.cu")
ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")
NVCC_FLAGS = ARCH + ("-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-prec-div=false", "-prec-sqrt=false",
                     "-Xcompiler", "-fPIC",
                     f"-I{INCLUDE}", f"-I{CSRC}")
CXX_FLAGS = ("-O2", "-std=c++17", "-shared", "-fPIC", "-Wall", "-Wno-unknown-pragmas",
             f"-I{INCLUDE}", f"-I{CSRC}")


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or add CUDA to PATH)")


def _stamp():
    h = hashlib.sha256()
    for p in sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h")):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    LIB_DIR.mkdir(exist_ok=True)
    stamp_file = LIB_DIR / ".stamp"
    stamp = _stamp()
    if (not force and ENGINE_SO.exists() and HOSTEMU_SO.exists() and stamp_file.exists()
            and stamp_file.read_text() == stamp):
        return ENGINE_SO
    nvcc = _nvcc()
    objs = [LIB_DIR / (Path(s).stem + ".o") for s in CU_SOURCES]
    cmds = [[nvcc, *NVCC_FLAGS, "-c", str(CSRC / s), "-o", str(o)] for s, o in zip(CU_SOURCES, objs)]
    cxx = os.environ.get("CXX", "g++")
    emu = [cxx, *CXX_FLAGS, str(CSRC / "hostemu.cpp"), "-o", str(HOSTEMU_SO) + ".tmp"]
    with ThreadPoolExecutor(max_workers=len(cmds) + 1) as ex:
        futs = [ex.submit(_run, c, verbose) for c in cmds] + [ex.submit(_run, emu, verbose)]
        for f in futs:
            f.result()
    tmp = str(ENGINE_SO) + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *map(str, objs)], verbose)
    os.replace(tmp, ENGINE_SO)
    os.replace(str(HOSTEMU_SO) + ".tmp", HOSTEMU_SO)
    for o in objs:
        o.unlink(missing_ok=True)
    stamp_file.write_text(stamp)
    return ENGINE_SO
