"""GB300-native (sm_103a, FP64) Smolyak type-4 H.psi for ElVibRot-style SG4 bases.

The compute path is libevrsg4.so (CUDA kernels behind the C ABI declared in
include/evr_sg4.h); this package is its host-side mirror of the reference's
operator interface (sub_TabOpPsi / sub_OpPsi / sub_scaledOpPsi).
"""
from .sg4 import (EVRError, MultiOp, ParamOp, Polynomial, SG4Basis, SG4Tables, fp64_peak_tflops, fp64_pipes_tflops,
                  hpsi_multi, lib, sub_OpPsi, sub_scaledOpPsi, sub_TabOpPsi)

__all__ = ["EVRError", "MultiOp", "ParamOp", "Polynomial", "SG4Basis", "SG4Tables", "fp64_peak_tflops",
           "fp64_pipes_tflops", "hpsi_multi", "lib", "sub_OpPsi", "sub_scaledOpPsi", "sub_TabOpPsi"]
