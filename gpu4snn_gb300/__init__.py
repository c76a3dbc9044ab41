"""GB300-native simulation step of GPU4SNN (pulse-coupled Izhikevich networks).

The compute path is libgpu4snn.so (hand-written sm_103a CUDA behind a C ABI,
include/gpu4snn.h); this package is its Python host side.
"""
from ._lib import (ALG_AB, ALG_AP, ALG_AUTO, ALG_N, ALG_NAMES, ALG_S, ALG_SKL, CONN_GLIBC, CONN_PHILOX,
                   G4SError, load)
from .network import Network, Stats, conn_glibc, row_stride, run_batch, run_protocol

__all__ = ["Network", "Stats", "G4SError", "conn_glibc", "row_stride", "run_batch", "run_protocol", "load",
           "ALG_AP", "ALG_N", "ALG_S", "ALG_AB", "ALG_SKL", "ALG_AUTO", "ALG_NAMES", "CONN_PHILOX", "CONN_GLIBC"]
