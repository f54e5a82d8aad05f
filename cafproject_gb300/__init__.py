"""GB300-native implementation of CUBE's per-step gravity/update path.

The product is ``libcube_gb300.so`` (CUDA for sm_103a behind the C ABI in
include/cube_gpu.h); ``cube.CubeGPU`` mirrors the reference's subroutine
surface over that ABI.
"""
from .params import CubeParams, cdm64, cdm512, small  # noqa: F401
