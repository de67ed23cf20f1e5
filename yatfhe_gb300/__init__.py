"""GB300-native TFHE programmable bootstrapping (GINX / MP21 path of the yatfhe library).

The compute path is the CUDA library built from yatfhe_gb300/csrc (see build.py) and
reached through the C ABI in include/yatfhe_gb300.h; this package is a thin Python view
of that ABI plus the parameter sets.
"""
from .params import PARAM_SETS, T32_N1024, T56_N2048, PbsParams, small  # noqa: F401

__all__ = ["PbsParams", "T32_N1024", "T56_N2048", "PARAM_SETS", "small"]
