"""Build recipe for the CPU oracle and for the reference's own CPU code.

TEST INFRASTRUCTURE ONLY.  Products:

* ``oracle/_build/liboracle.so`` -- the C restatement (rtm_oracle.c,
  lsm_oracle.c, resample_oracle.c, poststack_oracle.c), FP32 + FP64, OpenMP.
* ``oracle/_ref/libref_rtm.so`` -- the reference's kernel bodies
  (caixh90/RTM_GPU kernel.cu:15-517) and Ricker function (kernel.cu:1261-1266)
  run on the CPU through ``ref_shim.cpp``.  The two source fragments are copied
  verbatim from a reference checkout into ``oracle/_ref/`` (git-ignored; the
  repository never holds reference source).  Once copied, the fragments let
  the library be rebuilt on a machine without the checkout.
* ``oracle/_ref/libref_host.so`` -- LSMOrCon_rec_2D.cpp,
  GPU_velocity_real.cpp and Resample.cpp compiled in place from the checkout
  (only where the checkout exists; used to generate the golden fixtures).
* ``oracle/_ref/libref_post.so`` -- DisToTimeAndTimeToDis1D.cpp and
  phase_correction_ricker_decon.cpp, likewise (the post-stack chain).
* ``oracle/_ref/libref_gpu.so`` -- the same kernel fragment compiled by nvcc
  for the GPU (sm_103a) under ``ref_gpu_shim.cu``, which restates the
  reference's per-shot launch sequence: the reference's own GPU code as a
  yardstick and parity target (built wherever nvcc is present).

The reference checkout is the directory named by the RTM_REFERENCE_CHECKOUT
environment variable or the --checkout argument (default: the checkout this
recipe was written against).

Everything is compiled with ``-ffp-contract=off`` so that neither x86-64 nor
aarch64 fuses multiply-adds: the FP32 oracle then reproduces the reference's
rounding sequence exactly.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
DEFAULT_CHECKOUT = os.environ.get("RTM_REFERENCE_CHECKOUT", "/root/reference")
NVCC = os.environ.get("NVCC", "nvcc")

CFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in
            ("rtm_oracle.c", "lsm_oracle.c", "resample_oracle.c", "poststack_oracle.c",
             "rtm_oracle_body.h", "rtm_driver_body.h", "rtm_oracle.h")]
    if force or _stale(out, srcs):
        _run(["gcc", *CFLAGS, "-std=gnu11", "-o", out + ".tmp", *srcs[:4], "-lm"])
        os.replace(out + ".tmp", out)
    return out


def extract_fragments(checkout: str = DEFAULT_CHECKOUT) -> bool:
    """Copy the kernel block and the Ricker function of kernel.cu into
    oracle/_ref/ (verbatim).  Returns False when no checkout is present."""
    src = os.path.join(checkout, "kernel.cu")
    if not os.path.exists(src):
        return False
    text = open(src, "r", encoding="latin-1").read().splitlines(keepends=True)
    start = next(i for i, l in enumerate(text) if l.startswith("#define BLOCKSIZE"))
    stop = next(i for i, l in enumerate(text) if l.startswith("float f(float t1,float f0);"))
    fdef = next(i for i, l in enumerate(text) if l.startswith("float f(float t1,float f0)")
                and not l.rstrip().endswith(";") and "//" not in l)
    os.makedirs(REF_OUT, exist_ok=True)
    with open(os.path.join(REF_OUT, "ref_kernels.inc"), "w", encoding="latin-1") as fh:
        fh.writelines(text[start:stop])
    with open(os.path.join(REF_OUT, "ref_ricker.inc"), "w", encoding="latin-1") as fh:
        fh.write("#ifndef pi\n#define pi 3.1415926535898\n#endif\n")
        fh.writelines(text[fdef:])
    return True


def build_ref(checkout: str = DEFAULT_CHECKOUT, force: bool = False) -> dict:
    """Build what can be built of the reference; returns {name: path}."""
    got = {}
    have_checkout = extract_fragments(checkout)
    kin = os.path.join(REF_OUT, "ref_kernels.inc")
    if os.path.exists(kin):
        out = os.path.join(REF_OUT, "libref_rtm.so")
        srcs = [os.path.join(HERE, "ref_shim.cpp"), kin, os.path.join(REF_OUT, "ref_ricker.inc"),
                os.path.join(HERE, "rtm_driver_body.h"), os.path.join(HERE, "rtm_oracle.h")]
        if force or _stale(out, srcs):
            _run(["g++", *CFLAGS, "-w", "-I", REF_OUT, "-I", HERE, "-o", out + ".tmp", srcs[0]])
            os.replace(out + ".tmp", out)
        got["kernels"] = out
    if have_checkout:
        out = os.path.join(REF_OUT, "libref_host.so")
        srcs = [os.path.join(HERE, "ref_host_shim.cpp"),
                os.path.join(checkout, "LSMOrCon_rec_2D.cpp"),
                os.path.join(checkout, "GPU_velocity_real.cpp"),
                os.path.join(checkout, "Resample.cpp")]
        if force or _stale(out, srcs):
            _run(["g++", *CFLAGS, "-w", "-I", checkout, "-o", out + ".tmp", srcs[0]])
            os.replace(out + ".tmp", out)
        got["host"] = out
        out = os.path.join(REF_OUT, "libref_post.so")
        srcs = [os.path.join(HERE, "ref_post_shim.cpp"),
                os.path.join(checkout, "DisToTimeAndTimeToDis1D.cpp"),
                os.path.join(checkout, "phase_correction_ricker_decon.cpp")]
        if force or _stale(out, srcs):
            _run(["g++", *CFLAGS, "-w", "-I", checkout, "-o", out + ".tmp", srcs[0]])
            os.replace(out + ".tmp", out)
        got["post"] = out
    return got


def build_ref_gpu(force: bool = False) -> str:
    """oracle/_ref/libref_gpu.so: the reference's kernels (the verbatim
    fragment in oracle/_ref/) under ref_gpu_shim.cu, for sm_103a, with
    nvcc's default optimisation and contraction as the reference's own build
    line (README.md:5) uses them.  Raises when the fragment or nvcc is
    missing."""
    kin = os.path.join(REF_OUT, "ref_kernels.inc")
    if not os.path.exists(kin):
        raise RuntimeError("reference kernel fragment unavailable (no checkout, no oracle/_ref)")
    out = os.path.join(REF_OUT, "libref_gpu.so")
    srcs = [os.path.join(HERE, "ref_gpu_shim.cu"), kin, os.path.join(HERE, "rtm_oracle.h")]
    if force or _stale(out, srcs):
        _run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC", "-shared",
              "-w", "-I", REF_OUT, "-I", HERE, "-o", out + ".tmp", srcs[0]])
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    args = sys.argv[1:]
    force = "--force" in args
    checkout = DEFAULT_CHECKOUT
    if "--checkout" in args:
        checkout = args[args.index("--checkout") + 1]
    print(build_oracle(force=force))
    print(build_ref(checkout, force=force))
    print(build_ref_gpu(force=force))
