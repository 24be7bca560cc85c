"""qflex_gb300 — a GB300-native engine for qFlex grid tensor-network
contraction of random quantum circuits.

Public surface:
  * ``simulate(options)``: drop-in for the reference's pybind ``qflex.simulate``.
  * ``Context``: the C-ABI engine context (evaluate, evaluate_many, tensor ops).
  * ``Tensor``, ``multiply``: named-index device tensors with the reference's
    Tensor semantics (reorder / bundle / project / multiply).
  * ``rqc``: seeded random-circuit, grid and ordering generators for the
    benchmark workloads.
"""
from ._lib import (BF16X3, FP16X3, FP32, FP64, FP64_FF, TF32X3, Context, QflexGb300Error,  # noqa: F401
                   load_library)
from .qflex import simulate  # noqa: F401

__all__ = ["Context", "QflexGb300Error", "load_library", "simulate", "FP32", "TF32X3", "BF16X3", "FP16X3", "FP64",
           "FP64_FF"]
