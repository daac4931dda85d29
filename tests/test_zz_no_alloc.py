"""cg_thermal_sweeps_noalloc, the entry point for callers that cannot allocate device memory (a JVM
in a memory-accounted container lending its own buffers, a renderer that owns every allocation on
its device, replay of a graph captured elsewhere): the sweeps with their scratch field in a fixed
device array instead of a context buffer.

Checked through the C ABI against cg_thermal_sweeps on the same input, bit for bit (the tolerance
of the thermal tests: none), on two calls in a row, so the second call also shows that what the
first left in the shared array does not leak into it. The cases cover no sweep (a plain copy), one
sweep (a single launch straight into the output), odd and even counts, a grid exactly at the
array's 2^20-cell limit, and a stream other than the one torch is using. Kept in its own file,
collected last."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("side_stream", [False, True])
def test_noalloc_sweeps_match_the_allocating_entry_point(side_stream):
    import torch

    from cartogenesis_gb300 import ErosionConfig, GpuErosionAccelerator, abi, synthetic
    from cartogenesis_gb300.runtime import load_library

    lib = load_library()
    accel = GpuErosionAccelerator()
    s = torch.cuda.Stream() if side_stream else torch.cuda.current_stream()
    cases = ((512, 256, 24, 3), (1024, 512, 13, 4), (256, 128, 0, 5), (256, 128, 1, 6), (1024, 1024, 7, 7))
    for W, H, passes, seed in cases:
        h, up, _ = synthetic.world(W, H, seed)
        h = np.clip(h + up * 0.02, 0, None).astype(np.float32)
        lim, _ = ErosionConfig(W, H, seed).thermal_limits()
        want = accel.erode(W, H, h, lim, passes, 0.25) if passes > 0 else h.copy()
        d_in = torch.from_numpy(h).cuda()
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        st = lib.cg_thermal_sweeps_noalloc(d_in.data_ptr(), d_out.data_ptr(), W, H, lim.to_c(), passes, 0.25,
                                           s.cuda_stream)
        assert st == abi.CG_OK
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (W, H, passes)
        assert np.array_equal(d_in.cpu().numpy(), h)   # the input is only read


def test_noalloc_rejects_what_it_cannot_hold():
    import torch

    from cartogenesis_gb300 import ErosionConfig, abi
    from cartogenesis_gb300.runtime import load_library

    lib = load_library()
    lim, _ = ErosionConfig(64, 32, 1).thermal_limits()
    a = torch.zeros(32, 64, device="cuda")
    b = torch.zeros(32, 64, device="cuda")
    big = torch.zeros(2 * 32 * 64, device="cuda")
    # 2048 x 1024 is twice the array's 2^20 cells; checked before anything touches the device.
    assert lib.cg_thermal_sweeps_noalloc(a.data_ptr(), b.data_ptr(), 2048, 1024, lim.to_c(), 4, 0.25,
                                         None) == abi.CG_BAD_ARG
    assert lib.cg_thermal_sweeps_noalloc(a.data_ptr(), a.data_ptr(), 64, 32, lim.to_c(), 4, 0.25,
                                         None) == abi.CG_BAD_ARG
    # Partly overlapping input and output: the output starts one cell into the input.
    assert lib.cg_thermal_sweeps_noalloc(big.data_ptr(), big.data_ptr() + 4, 64, 32, lim.to_c(), 4, 0.25,
                                         None) == abi.CG_BAD_ARG
    assert lib.cg_thermal_sweeps_noalloc(big.data_ptr() + 4, big.data_ptr(), 64, 32, lim.to_c(), 0, 0.25,
                                         None) == abi.CG_BAD_ARG
    assert lib.cg_thermal_sweeps_noalloc(a.data_ptr(), b.data_ptr(), 48, 32, lim.to_c(), 4, 0.25,
                                         None) == abi.CG_BAD_ARG
    assert lib.cg_thermal_sweeps_noalloc(a.data_ptr(), b.data_ptr(), 64, 32, lim.to_c(), -1, 0.25,
                                         None) == abi.CG_BAD_ARG
