"""The thermal sweeps on the GPU against the oracle, bit for bit (ErosionStage.thermalSweep,
P/ErosionStage.kt:235-403), through the ErosionAccelerator seam's C entry point."""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def accel():
    from cartogenesis_gb300 import GpuErosionAccelerator
    return GpuErosionAccelerator()


@pytest.mark.parametrize("W,H,passes", [
    (16, 16, 1), (16, 16, 7), (32, 16, 13), (64, 32, 8), (128, 64, 3), (512, 256, 24), (2048, 1024, 96),
    (256, 256, 1500),
])
def test_thermal_sweeps_bit_exact(accel, W, H, passes):
    from cartogenesis_gb300 import ErosionConfig
    h, up, _ = synthetic.world(W, H, seed=W + H + passes)
    h = np.clip(h + up * 0.02, 0, None).astype(np.float32)
    cfg = ErosionConfig(W, H, 5)
    lim, _ = cfg.thermal_limits()
    got = accel.erode(W, H, h, lim, passes, 0.25)
    olim, _ = oracle.thermal_limits(oracle.default_params(W, H, 5))
    want = oracle.thermal_sweep(h, olim, passes, 0.25, skip=True)
    assert got.dtype == np.float32
    diff = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
    assert diff.size == 0, f"{diff.size} cells differ, first {diff[:5]}"


def test_thermal_mesa_12000km(accel):
    """The ThermalAspect mesa (T/ThermalAspectTest.kt) on the device, bit-exact to the oracle."""
    from cartogenesis_gb300 import ErosionConfig
    W = H = 256
    cfg = ErosionConfig(W, H, 1, world_width_km=12000.0)
    lim, _ = cfg.thermal_limits()
    cw, ch = 12000.0 / W, 6000.0 / H
    cols, rows = np.meshgrid(np.arange(W), np.arange(H))
    on = np.sqrt(((cols - W // 2) * cw) ** 2 + ((rows - H // 2) * ch) ** 2) < 1200.0
    mesa = (np.where(on, 15000.0, 9000.0).astype(np.float32) / np.float32(16000.0)).astype(np.float32)
    got = accel.erode(W, H, mesa, lim, 1500, 0.25)
    want = oracle.thermal_sweep(mesa, oracle.thermal_limits(oracle.default_params(W, H, 1,
                                                                                  world_width_km=12000.0))[0], 1500)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_thermal_zero_passes_is_a_copy(accel):
    from cartogenesis_gb300 import ErosionConfig
    h = synthetic.heights_field(64, 32, seed=3)
    lim, _ = ErosionConfig(64, 32, 1).thermal_limits()
    got = accel.erode(64, 32, h, lim, 0, 0.25)
    assert np.array_equal(got, h) and got is not h


def test_thermal_rejects_bad_grid(accel):
    from cartogenesis_gb300 import CgError, ErosionConfig
    lim, _ = ErosionConfig(64, 32, 1).thermal_limits()
    with pytest.raises(CgError):
        accel.erode(48, 32, np.zeros((32, 48), np.float32), lim, 1, 0.25)
