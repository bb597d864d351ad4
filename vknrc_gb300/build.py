"""Builds libnrc.so (the C-ABI library) in-tree with nvcc for sm_103a.

    python -m vknrc_gb300.build        # or vknrc_gb300.build.build()

Translation units compile in parallel; the library lands in vknrc_gb300/_lib/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libnrc.so")
SOURCES = ["nrc_api.cu", "nrc_infer.cu", "nrc_train.cu", "nrc_encode.cu", "nrc_noalloc.cu", "nrc_server.cu", "nrc_server_loop.cu", "nrc_screen.cu", "nrc_unpack.cu", "nrc_fp8.cu", "nrc_trace.cu", "nrc_optimize.cu"]
# per-file flags: the path tracer keeps every multiply and add separate (its CPU
# oracle repeats the same IEEE operations)
FILE_FLAGS = {"nrc_trace.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnrc.so")
    return path


def _compile(src: str, obj: str, verbose: bool) -> str:
    cmd = [nvcc(), *ARCH, *FLAGS, *FILE_FLAGS.get(src, []), "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "nrc.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link libnrc.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    objs = [os.path.join(OUT_DIR, "obj", s.replace(".cu", ".o")) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        logs = list(ex.map(lambda so: _compile(so[0], so[1], verbose), zip(SOURCES, objs)))
    if verbose:
        for s, log in zip(SOURCES, logs):
            sys.stderr.write(f"== {s}\n{log}")
    tmp = LIB + ".tmp"
    link = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
