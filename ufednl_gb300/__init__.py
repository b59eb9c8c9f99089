"""GB300-native (sm_103a) engine for the FedNL round hot path of u-FedNL (dopt).

The compute path is the native library ``_build/libfednl_gpu.so`` (CUDA kernels behind the C ABI
declared in include/fednl_gpu.h); ``fednl`` is its Python host API and ``datagen`` builds the seeded
synthetic workloads.
"""
from . import datagen  # noqa: F401

__all__ = ["datagen", "fednl", "build"]
