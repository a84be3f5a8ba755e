"""GB300-native (sm_103a) position-based-fluid step of Lustrine.

The compute path is liblustrine_gb300.so (hand-written CUDA kernels behind a
C ABI, include/lustrine_gb300.h); this package is its Python host side.
"""
from ._lib import LISTS_COLUMN, LISTS_COMPACT, LustrineError, load
from .pbf import (MODE_PBF, MODE_REFERENCE, MODE_SAND, PRECISION_FP32, PRECISION_MIXED, PRECISION_MIXED_SCENE,
                  PbfParams, PbfSim,
                  pbf_params, reference_params, rest_lattice_mass, sand_params)

__all__ = ["LustrineError", "load", "PbfSim", "PbfParams", "pbf_params", "reference_params", "rest_lattice_mass", "sand_params",
           "MODE_PBF", "MODE_REFERENCE", "MODE_SAND", "PRECISION_FP32", "PRECISION_MIXED",
           "PRECISION_MIXED_SCENE", "LISTS_COLUMN", "LISTS_COMPACT"]
