"""GB300-native progressive-refinement hemicube radiosity solver.

The product is the CUDA shared library radiosity_gb300/libradiosity_gb300.so
(C ABI in include/radiosity.h); this package builds it in-tree and binds it
with ctypes.  Scene generators for the synthetic benchmark workloads live in
``radiosity_gb300.scenes``.
"""
from ._lib import (  # noqa: F401
    EXPORTS, MLP, MODE_PHYS, MODE_REF, Multi, MultiGather, RadConfig, RadError, RadGatherStats, RadStats, RadTuning, Solver, bf16_gemm,
    default_config, derived, load, obj_scene, plan_shooters, reference_neighbours,
    reference_scene, rr_read, rr_write, selftest_bounded_wait,
)
from .build import LIB as LIB_PATH  # noqa: F401
from .build import build  # noqa: F401
