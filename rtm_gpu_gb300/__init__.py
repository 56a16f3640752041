"""GB300 (sm_103a) engine for the 2-D acoustic reverse-time-migration path of
caixh90/RTM_GPU: hand-written CUDA kernels behind a C ABI
(include/rtm_gb300.h), with this package as a thin Python front end.

    from rtm_gpu_gb300 import build_problem, Engine
"""
from .capi import lib, lib_path, KERNEL_NAMES  # noqa: F401
from .engine import Engine  # noqa: F401
from .problem import Problem, build_problem, prep_taylor, prep_wavelet  # noqa: F401

__all__ = ["lib", "lib_path", "Engine", "Problem", "build_problem", "prep_taylor", "prep_wavelet",
           "KERNEL_NAMES"]
