"""GB300-native erosion stage for Cartogenesis.

The product is libcg_erosion.so (hand-written sm_103a CUDA behind the C ABI of
include/cg_erosion.h). This package loads it and mirrors the reference's own entry points
(ErosionStage.apply, ErosionAccelerator.erode, FlowRouting.*, SeaLevelStage.percentileCut) on
top of it. There is no CPU fallback: if the library or the device is missing, calls raise.
"""
from .runtime import (CgError, Context, library, load_library)  # noqa: F401
from .api import (BeltErosion, BeltReplay, BeltWindow, ErosionStage, ErosionConfig, GaussianBlur,  # noqa: F401
                  GpuErosionAccelerator, FlowRouting, HydraulicErosion, Isostasy, SeaLevelStage, StageRounds,
                  ThermalLimits)
