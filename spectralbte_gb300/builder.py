"""Build libspectral_gb300.so in place with nvcc for sm_103a.

Each translation unit compiles in parallel to an object under _build/; the
objects then link into spectralbte_gb300/libspectral_gb300.so.  The
benchmark's FP32 FMA-rate probe (calib/fma_probe.cu) links into a library of
its own, libspectral_calib.so, so the collision library carries no
calibration code.  No CMake is involved, and building needs no GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libspectral_gb300.so")

SOURCES = ["fft3d.cu", "conv.cu", "conv_ws.cu", "conserve.cu", "weights.cu", "transport.cu",
           "capi.cu", "noalloc.cu", "fno.cu"]
CALIB_SRC = os.path.join(HERE, "calib", "fma_probe.cu")
CALIB_LIB = os.path.join(HERE, "libspectral_calib.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-fvisibility=default"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str]) -> str:
    path = src if os.path.isabs(src) else os.path.join(CSRC, src)
    obj = os.path.join(OUT, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale(objs: list[str]) -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CALIB_LIB):
        return True
    if os.path.getmtime(CALIB_SRC) > os.path.getmtime(CALIB_LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "spectral_bte.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    extra = list(extra or [])
    os.makedirs(OUT, exist_ok=True)
    if not force and not _stale([]):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES + [CALIB_SRC]))
    for lib, parts in ((LIB, objs[:-1]), (CALIB_LIB, objs[-1:])):
        tmp = lib + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *parts, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=[a for a in sys.argv[1:] if a != "--force"])
