"""GB300-native molecular-dynamics hot path for MolTwister's `moldyn run` (sm_103a CUDA behind a C ABI).

The compute path is libmtgpu.so (moltwister_gb300/csrc, C ABI in include/mtgpu.h); this package is the
host-side Python binding and the system/configuration description it consumes.
"""
from .system import (MDConfig, MDSystem, NonBondedTerm, BondTerm, AngleTerm, DihedralTerm)  # noqa: F401
