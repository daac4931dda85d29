"""Loads libcg_erosion.so and wraps its context. Fails loudly when the library is missing."""
import ctypes as C
import os
import threading

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcg_erosion.so")

# Every symbol include/cg_erosion.h declares; the CPU tests check the library exports them all.
EXPORTS = [
    "cg_default_params", "cg_thermal_limits_for", "cg_create", "cg_destroy", "cg_cancel", "cg_last_error",
    "cg_stream", "cg_kernel_launches", "cg_probe_fp64_rate",
    "cg_thermal_sweeps", "cg_thermal_sweeps_noalloc", "cg_erode_stage", "cg_erode_stage_dev", "cg_erode_batch", "cg_percentile_cut", "cg_fill_depressions", "cg_flow_directions",
    "cg_drainage_order", "cg_accumulate", "cg_spillways", "cg_breach",
    "cg_stage_begin", "cg_erode_rounds", "cg_stage_height", "cg_stage_finish", "cg_sea_level_cut",
    "cg_flexure_deflection", "cg_sequential_sum", "cg_sequential_sum_f64", "cg_belt_replay", "cg_gaussian_blur",
    "cg_stage_replay_belts", "cg_route_cut",
]


class CgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None
_lock = threading.Lock()


def load_library(path=LIB_PATH):
    """Load the library and declare its signatures. Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise CgError(abi.CG_CUDA, f"{path} is missing: build it with cartogenesis_gb300.build.build()")
        L = C.CDLL(path)
        vp, i32, i64, f32, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_float, C.c_double
        PP = C.POINTER(abi.ErosionParams)
        L.cg_default_params.argtypes = [PP, i32, i32, i64]
        L.cg_default_params.restype = None
        L.cg_thermal_limits_for.argtypes = [PP, C.POINTER(abi.ThermalLimits), C.POINTER(i32)]
        L.cg_create.argtypes = [C.POINTER(vp), i32]
        L.cg_destroy.argtypes = [vp]
        L.cg_destroy.restype = None
        L.cg_cancel.argtypes = [vp]
        L.cg_cancel.restype = None
        L.cg_last_error.argtypes = [vp]
        L.cg_last_error.restype = C.c_char_p
        L.cg_stream.argtypes = [vp]
        L.cg_stream.restype = vp
        L.cg_kernel_launches.argtypes = [vp]
        L.cg_kernel_launches.restype = i64
        L.cg_probe_fp64_rate.argtypes = [vp, C.POINTER(f64)]
        L.cg_thermal_sweeps.argtypes = [vp, i32, i32, vp, vp, abi.ThermalLimits, i32, f32]
        L.cg_thermal_sweeps_noalloc.argtypes = [vp, vp, i32, i32, abi.ThermalLimits, i32, f32, vp]
        if hasattr(L, "cg_erode_stage"):
            L.cg_erode_stage.argtypes = [vp, PP, C.POINTER(abi.Inputs), C.POINTER(abi.Outputs), vp]
            L.cg_erode_stage_dev.argtypes = [vp, PP, C.POINTER(abi.Inputs), vp, vp, C.POINTER(i32)]
            L.cg_percentile_cut.argtypes = [vp, i32, i32, vp, f32, f32, f32, f32, C.POINTER(f32), vp, vp,
                                            C.POINTER(i32)]
            L.cg_fill_depressions.argtypes = [vp, i32, i32, vp, vp, vp, C.POINTER(i64), C.POINTER(i64)]
            L.cg_flow_directions.argtypes = [vp, i32, i32, vp, vp, vp, i64, f64, i32, i32, i32, vp, vp, vp]
            L.cg_drainage_order.argtypes = [vp, i32, i32, vp, vp, i32, vp]
            L.cg_accumulate.argtypes = [vp, i32, i32, vp, vp, i32, vp, vp]
            L.cg_spillways.argtypes = [vp, i32, i32, vp, vp, vp, vp, f32, vp, C.POINTER(abi.Basins)]
            L.cg_erode_batch.argtypes = [vp, i32, C.POINTER(abi.World), vp]
            L.cg_breach.argtypes = [vp, PP, vp, vp, vp, vp, vp, f32, f32, vp, C.POINTER(i32)]
            L.cg_stage_begin.argtypes = [vp, PP, C.POINTER(abi.Inputs)]
            L.cg_erode_rounds.argtypes = [vp, i32, i32, C.POINTER(abi.Weather), vp]
            L.cg_stage_height.argtypes = [vp, vp]
            L.cg_stage_finish.argtypes = [vp, C.POINTER(abi.Outputs)]
            L.cg_sea_level_cut.argtypes = [vp, PP, vp, f64, i32, C.POINTER(f32), vp, vp, C.POINTER(i32),
                                           C.POINTER(i32)]
            L.cg_flexure_deflection.argtypes = [vp, PP, vp, vp, C.POINTER(f64), C.POINTER(f64)]
            L.cg_sequential_sum.argtypes = [vp, vp, vp, i32, C.c_int64, C.POINTER(f64), vp]
            L.cg_sequential_sum_f64.argtypes = [vp, vp, C.c_int64, C.POINTER(f64)]
            L.cg_belt_replay.argtypes = [vp, PP, vp, C.POINTER(abi.BeltWindow), C.POINTER(abi.BeltInputs), vp,
                                         C.POINTER(abi.BeltBooks)]
            L.cg_gaussian_blur.argtypes = [vp, i32, i32, vp, f64, f64]
            L.cg_route_cut.argtypes = [vp, PP, vp, vp, i32, vp, vp, vp, vp, vp]
            L.cg_stage_replay_belts.argtypes = [vp, C.POINTER(abi.BeltWindow), C.POINTER(abi.Weather), i32, f64, vp,
                                                C.POINTER(abi.BeltBooks)]
        _lib = L
        return _lib


def library():
    return load_library()


class Context:
    """One cg_ctx on one device. Calls on a context are serialised by a lock."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.cg_create(C.byref(h), device)
        if st != abi.CG_OK:
            raise CgError(st, f"cg_create(device={device}) failed (no CUDA device?)")
        self.handle = h
        self.lock = threading.Lock()

    def check(self, status):
        if status != abi.CG_OK:
            raise CgError(status, self.lib.cg_last_error(self.handle).decode(errors="replace"))

    def cancel(self):
        self.lib.cg_cancel(self.handle)

    @property
    def stream(self):
        """The cudaStream_t (as an int) every kernel of this context runs on."""
        return self.lib.cg_stream(self.handle)

    @property
    def kernel_launches(self):
        return self.lib.cg_kernel_launches(self.handle)

    def close(self):
        if self.handle:
            self.lib.cg_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
