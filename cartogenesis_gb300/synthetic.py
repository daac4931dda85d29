"""Seeded synthetic worlds standing in for the reference's terrain and plate stages.

The reference's benchmark worlds come out of TerrainStage + PlateStage for a seed; those stages
cannot run without a JVM, so worlds here are project-written and fully determined by their seed
(numpy's PCG64):

- heights: fBm with spectral exponent beta (power ~ k^-beta), rescaled to [-10000, 6000] m and
  mapped to the height field's units, (m + 10000) / 16000 (WorldScale.fieldAtAltitude);
- uplift: millimetres a year, >= 0, in 100-300 km bands along plate boundaries (a seeded
  Voronoi partition of the sphere), or Gaussian ridges along great-circle segments;
- rock erodibility: a smooth lognormal factor, median 1, log-sigma 0.5;
- the belts' exposure-window history: thickening, wear and onset under the active uplift bands.
"""
import numpy as np

EARTH_KM = 40075.0


def _rng(seed, salt):
    return np.random.Generator(np.random.PCG64([int(seed) & 0xFFFFFFFF, salt]))


def fbm(width, height, beta=2.0, seed=1, salt=0):
    """Zero-mean, unit-variance fBm on a width x height grid, periodic in x."""
    rng = _rng(seed, 1000 + salt)
    ky = np.fft.fftfreq(height)[:, None]
    kx = np.fft.rfftfreq(width)[None, :] * (width / height) * 0.5  # cells are 2:1 on the ground
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    amp = k ** (-beta / 2.0)
    amp[0, 0] = 0.0
    phase = rng.uniform(0.0, 2.0 * np.pi, size=amp.shape)
    mag = rng.standard_normal(size=amp.shape)
    spec = amp * mag * np.exp(1j * phase)
    field = np.fft.irfft2(spec, s=(height, width))
    field -= field.mean()
    sd = field.std()
    return (field / sd if sd > 0 else field).astype(np.float64)


def heights_field(width, height, seed=1, beta=2.0, lo_m=-10000.0, hi_m=6000.0):
    """fBm heights rescaled to [lo_m, hi_m] metres, in field units (float32)."""
    f = fbm(width, height, beta, seed)
    m = lo_m + (f - f.min()) / (f.max() - f.min()) * (hi_m - lo_m)
    return ((m + 10000.0) / 16000.0).astype(np.float32)


def _lonlat(width, height):
    lon = (np.arange(width) + 0.5) / width * 2.0 * np.pi
    lat = np.pi / 2 - (np.arange(height) + 0.5) / height * np.pi
    return np.meshgrid(lon, lat)


def _unit(lon, lat):
    return np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], axis=-1)


def uplift_bands(width, height, seed=1, plates=12, world_km=EARTH_KM, lo_mm=0.5, hi_mm=3.0):
    """Uplift in mm/yr in 100-300 km bands along the boundaries of a seeded spherical Voronoi."""
    rng = _rng(seed, 2000)
    lon, lat = _lonlat(width, height)
    p = _unit(lon, lat)
    centres = rng.standard_normal((plates, 3))
    centres /= np.linalg.norm(centres, axis=1, keepdims=True)
    radius_km = world_km / (2.0 * np.pi)
    dots = np.einsum("hwk,pk->hwp", p, centres)
    ang = np.arccos(np.clip(dots, -1.0, 1.0))
    part = np.partition(ang, 1, axis=-1)
    gap_km = (part[..., 1] - part[..., 0]) * radius_km * 0.5   # distance to the nearest boundary
    first = np.argmin(ang, axis=-1)
    band_km = rng.uniform(100.0, 300.0, size=plates)[first]
    peak = rng.uniform(lo_mm, hi_mm, size=plates)[first]
    active = rng.uniform(size=plates)[first] < 0.6
    up = np.where((gap_km < band_km) & active, peak * np.cos(0.5 * np.pi * gap_km / band_km) ** 2, 0.0)
    return up.astype(np.float32)


def uplift_ridges(width, height, seed=1, ridges=15, world_km=EARTH_KM, lo_m_per_myr=50.0, hi_m_per_myr=4000.0):
    """Uplift in mm/yr: Gaussian ridges of 50-4000 m/Myr along random great-circle segments."""
    rng = _rng(seed, 3000)
    lon, lat = _lonlat(width, height)
    p = _unit(lon, lat)
    radius_km = world_km / (2.0 * np.pi)
    up = np.zeros((height, width))
    for _ in range(ridges):
        a = rng.standard_normal(3)
        a /= np.linalg.norm(a)
        t = rng.standard_normal(3)
        t -= t.dot(a) * a
        t /= np.linalg.norm(t)
        n = np.cross(a, t)                      # pole of the great circle through a along t
        length = rng.uniform(0.05, 0.35) * np.pi
        width_km = rng.uniform(100.0, 300.0)
        rate = rng.uniform(lo_m_per_myr, hi_m_per_myr) / 1000.0   # m/Myr -> mm/yr
        off = np.arcsin(np.clip(p @ n, -1.0, 1.0)) * radius_km   # distance off the circle
        along = np.arctan2(p @ t, p @ a)
        inside = (along >= 0.0) & (along <= length)
        up = np.maximum(up, np.where(inside, rate * np.exp(-0.5 * (off / (0.5 * width_km)) ** 2), 0.0))
    return up.astype(np.float32)


def rock_erodibility(width, height, seed=1, sigma=0.5):
    """A smooth lognormal factor with median 1 and log-standard-deviation sigma."""
    z = fbm(width, height, beta=3.0, seed=seed, salt=7)
    return np.exp(sigma * z).astype(np.float32)


def world(width, height, seed=1, uplift="bands"):
    """One synthetic world: (height, uplift_mm_per_year, rock_erodibility), float32 [H, W]."""
    h = heights_field(width, height, seed)
    up = uplift_bands(width, height, seed) if uplift == "bands" else uplift_ridges(width, height, seed)
    rk = rock_erodibility(width, height, seed)
    return h, up, rk


def belt_window(width, height, seed=1, window_myr=40.0, threshold_mm=0.05):
    """A seeded stand-in for the plate stage's exposure-window history (BeltWindow): the cells under
    uplift_bands' active bands thickened by 40 km per mm/yr of today's uplift (so the window's rise
    outruns the rounds' share of today's rate, as a young belt's does), worn by 20-50% of that,
    beginning 40-100% of the window ago (a smooth field); -1 onset, no thickening and no wear
    elsewhere. Returns (tectonic_km, wear_km, onset_myr_ago, window_myr), float32 [H, W] and a float."""
    up = uplift_bands(width, height, seed)
    belt = up > threshold_mm
    wear_share = 0.2 + 0.3 * (0.5 + 0.5 * np.tanh(fbm(width, height, beta=3.0, seed=seed, salt=11)))
    start = 0.4 + 0.6 * (0.5 + 0.5 * np.tanh(fbm(width, height, beta=3.0, seed=seed, salt=12)))
    tectonic = np.where(belt, 40.0 * up, 0.0).astype(np.float32)
    wear = np.where(belt, tectonic * wear_share, 0.0).astype(np.float32)
    onset = np.where(belt, window_myr * start, -1.0).astype(np.float32)
    return tectonic, wear, onset, float(window_myr)


def batch_shapes(n, seed=1, max_rows=2048):
    """The batched workload's world shapes: n planets of radius r ~ U(0.25, 2.0) Earth radii, each
    grid 2R x R cells with R the power of two nearest 1024 r (WorldGenConfig wants powers of two),
    in {256, ..., max_rows}. Returns [(width, height, seed_i, radius)]; seed_i = seed * 1000 + i."""
    rng = _rng(seed, 4000)
    out = []
    for i in range(n):
        r = float(rng.uniform(0.25, 2.0))
        rows = int(2 ** np.round(np.log2(1024.0 * r)))
        rows = int(min(max(rows, 256), max_rows))
        out.append((2 * rows, rows, seed * 1000 + i, r))
    return out
