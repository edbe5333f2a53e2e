"""marshmallow: GB300 cloud raymarch pass of Project-Marshmallow behind the C ABI of include/mm.h.

Python side of the library: a ctypes binding of libmm.so (lib), the scene set-up of the benchmark
configurations (scene), texture/frame helpers over CUDA device memory (render) and the error
metrics of the parity gates (metrics).  All device work runs in libmm.so's CUDA kernels.
"""
from . import build, lib, metrics, render, scene  # noqa: F401
from .lib import load  # noqa: F401
