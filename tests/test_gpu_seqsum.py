"""The reference's sequential double sums (`s += v[c]` in cell order: normaliseOverLand's rain mean and
shieldingOverLand's cover mean, HydraulicErosion.kt:476-486, 557-567; deflectionMetres' load mean,
Isostasy.kt:337-339) on the device, bit for bit against numpy's running sum (np.cumsum adds in order),
over the cases that stress the parallel form: ties to even, sign changes, binade crossings, values
that dwarf the sum, masks, infinities; and a check that smooth fields go the parallel way."""
import numpy as np
import pytest

from cartogenesis_gb300.api import sequential_sum

pytestmark = pytest.mark.gpu


def want(x, mask=None, mode=0):
    v = np.asarray(x, np.float32)
    if mode == 1:
        v = (np.float32(1.0) - np.float32(0.5) * v).astype(np.float32)
    if mask is not None:
        v = v[np.asarray(mask, bool)]
    v = v.astype(np.float64)
    return float(np.cumsum(v)[-1]) if v.size else 0.0


def same(a, b):
    return np.float64(a).view(np.uint64) == np.float64(b).view(np.uint64) or (a != a and b != b)


rng = np.random.default_rng(7)
N = 1 << 21
CASES = {
    "normal": rng.normal(0.0, 1e6, N),
    "positive": rng.uniform(0.0, 1e3, N),
    "rain": rng.uniform(150.0, 2500.0, N),
    "mixed_scales": rng.normal(0.0, 1.0, N) * 10.0 ** rng.integers(-8, 9, N),
    "ties": np.concatenate([[2.0 ** 40], np.full(N // 2, 2.0 ** -13), np.full(N // 2, 3 * 2.0 ** -13)]),
    "ties_negative": np.concatenate([[-(2.0 ** 40)], np.tile([2.0 ** -13, -(2.0 ** -13), 5 * 2.0 ** -13], N // 3)]),
    "boundary": np.concatenate([[2.0 ** 30 - 1], rng.choice([1.0, -1.0, 0.5, -0.5, 0.25], N)]),
    "spikes": np.where(rng.random(N) < 1e-4, 1e30, rng.normal(0.0, 1.0, N)),
    "denormal": rng.normal(0.0, 1.0, N) * 1e-40,
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("masked", [False, True])
def test_sum_is_the_sequential_one(name, masked):
    x = CASES[name].astype(np.float32)
    mask = (rng.random(x.size) < 0.6).astype(np.uint8) if masked else None
    got, counts = sequential_sum(x, mask)
    assert same(got, want(x, mask)), (got, want(x, mask), counts)


@pytest.mark.parametrize("n", [0, 1, 7, 1023, 1024, 8191, 8192, 8193, 3 * 8192 + 5])
def test_sizes(n):
    x = rng.normal(5.0, 3.0, n).astype(np.float32)
    got, _ = sequential_sum(x)
    assert same(got, want(x))


def test_cover_factor_mode():
    veg = rng.uniform(0.0, 1.0, N).astype(np.float32)
    land = (rng.random(N) < 0.4).astype(np.uint8)
    got, _ = sequential_sum(veg, land, mode=1)
    assert same(got, want(veg, land, 1))


def test_infinities_and_nan():
    x = rng.normal(0.0, 1.0, 50000).astype(np.float32)
    x[12345] = np.inf
    got, _ = sequential_sum(x)
    assert same(got, want(x))
    x[23456] = -np.inf
    got, _ = sequential_sum(x)
    assert got != got


def test_smooth_fields_take_the_parallel_way():
    """A rain field (positive, the reference's range) is summed almost wholly by blocks."""
    x = CASES["rain"].astype(np.float32)
    got, counts = sequential_sum(x)
    assert same(got, want(x))
    blocks = (x.size + 8191) // 8192
    assert counts[0] >= 0.9 * blocks, counts
    assert counts[2] <= 16, counts
