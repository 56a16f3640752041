"""Compiles the CUDA / C++ sources of the engine into the in-tree shared
library rtm_gpu_gb300/_lib/librtm_gb300.so (sm_103a only)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "librtm_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "177"]
SOURCES = ["rtm_dropin.cu", "rtm_engine.cu", "rtm_host.cpp", "rtm_coeffs.cu", "rtm_noalloc.cu", "rtm_mlp.cu",
           "rtm_io.cu", "rtm_post.cu"]
# sources compiled without multiply-add contraction (FP64 parity with the host)
NOFMA = {"rtm_coeffs.cu"}
HEADERS = ["rtm_common.cuh", "rtm_engine_kernels.cuh"]
# the reference-style executable (rtm_run_config on the run file in the cwd)
CLI = os.path.join(LIBDIR, "rtm_gb300_run")
CLI_SRC = "rtm_cli_main.cpp"


def _newest_input() -> float:
    paths = [os.path.join(CSRC, f) for f in SOURCES + HEADERS + [CLI_SRC]]
    paths.append(os.path.join(HERE, "..", "include", "rtm_gb300.h"))
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _compile(src: str) -> str:
    out = os.path.join(LIBDIR, os.path.splitext(src)[0] + ".o")
    extra = ["-fmad=false"] if src in NOFMA else []
    cmd = [NVCC, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return out


def build(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    if (not force and os.path.exists(LIB) and os.path.exists(CLI)
            and os.path.getmtime(LIB) >= _newest_input()):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    cmd = [NVCC, *ARCH, "-O2", "-std=c++17", "-o", CLI + ".tmp", os.path.join(CSRC, CLI_SRC),
           "-L" + LIBDIR, "-lrtm_gb300", "-Xlinker", "-rpath=$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("executable link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv))
