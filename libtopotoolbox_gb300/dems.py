"""Seeded synthetic DEMs for the D8 flow pipeline workloads.

All grids are returned as float32 numpy arrays of shape (nrows, ncols) in
Fortran (column-major) order, the memory layout of libtopotoolbox
(include/topotoolbox.h:284-290: dims = {nrows, ncols}, fastest dimension
first).  Boundary-condition grids are uint8 with the same layout.

The generators stand in for real DEMs (the reference's snapshot DEMs are not
available); they reproduce the shapes, sizes and value distributions of the
five workloads:

* ``plain_512``      512 x 512 fractal (Hurst 0.7, 200 m relief) + U[0,0.5) m noise
* ``plain_4096``     4096 x 4096 fractal (Hurst 0.8, 1000 m relief), 200 inverted
                     Gaussian pits, rounded to 1 m (extensive flats)
* ``plain_16384``    16384 x 16384 fractal (Hurst 0.75, 2000 m relief), 5 % NaN
                     nodata disks, 1000 closed depressions
* ``batch_tiles``    512 tiles, side log-uniform in [128, 2048], aspect 0.5-2
* ``grad_8192``      8192 x 8192 fractal (Hurst 0.7, 800 m relief) + lognormal
                     runoff weights

``pcg4d_dem`` reproduces the random DEM of the reference's property tests
(test/grid.c:136-168 with the hash of test/utils.c:6-28).
"""
from __future__ import annotations

import math

import numpy as np

try:  # scipy's FFT is multithreaded and supports float32
    import scipy.fft as _fft

    def _irfft2(a, shape):
        return _fft.irfft2(a, s=shape, workers=-1)

except Exception:  # pragma: no cover - numpy fallback for the generator only
    def _irfft2(a, shape):
        return np.fft.irfft2(a, s=shape)


def fractal_surface(shape, hurst, relief, seed):
    """Spectral-synthesis fractal surface.

    Power spectrum proportional to |k|^-(2H+2); the surface is rescaled to
    span [0, relief] metres.  Returned as float32 (nrows, ncols), F-order.
    """
    nr, nc = int(shape[0]), int(shape[1])
    rng = np.random.default_rng(seed)
    # Spectrum laid out for irfft2 over axes (ncols, nrows): generating the
    # transposed C-ordered array gives an F-ordered (nrows, ncols) result.
    ky = np.fft.fftfreq(nc).astype(np.float32)[:, None]
    kx = np.fft.rfftfreq(nr).astype(np.float32)[None, :]
    k2 = ky * ky + kx * kx
    k2[0, 0] = 1.0
    amp = k2 ** np.float32(-(hurst + 1.0) / 2.0)
    amp[0, 0] = 0.0
    spec = (rng.standard_normal(amp.shape, dtype=np.float32)
            + 1j * rng.standard_normal(amp.shape, dtype=np.float32)).astype(np.complex64)
    spec *= amp
    del amp, k2
    z = _irfft2(spec, (nc, nr)).astype(np.float32, copy=False)
    del spec
    zmin, zmax = float(z.min()), float(z.max())
    z -= np.float32(zmin)
    z *= np.float32(relief / max(zmax - zmin, 1e-30))
    return z.T  # (nrows, ncols) view, Fortran-contiguous


def border_bc(shape):
    """bc = 1 on the outer ring, 0 inside (test/random_dem.cpp:640-647)."""
    bc = np.zeros(shape, dtype=np.uint8, order="F")
    bc[0, :] = 1
    bc[-1, :] = 1
    bc[:, 0] = 1
    bc[:, -1] = 1
    return bc


def _gaussian_pits(z, count, depth_range, sigma_range, rng):
    nr, nc = z.shape
    for _ in range(count):
        ci = rng.uniform(0, nr)
        cj = rng.uniform(0, nc)
        depth = rng.uniform(*depth_range)
        sigma = rng.uniform(*sigma_range)
        r = int(math.ceil(4 * sigma))
        i0, i1 = max(0, int(ci) - r), min(nr, int(ci) + r + 1)
        j0, j1 = max(0, int(cj) - r), min(nc, int(cj) + r + 1)
        gi = np.exp(-((np.arange(i0, i1, dtype=np.float32) - ci) ** 2) / (2 * sigma * sigma))
        gj = np.exp(-((np.arange(j0, j1, dtype=np.float32) - cj) ** 2) / (2 * sigma * sigma))
        z[i0:i1, j0:j1] -= np.float32(depth) * np.outer(gi, gj).astype(np.float32)


def nan_to_outlets(dem, bc):
    """The NaN convention of the reference's callers (test/grid.c:505-515,
    test/snapshot.cpp:365-380): NaN cells become -INF with bc = 1.  Returns
    (dem_for_fill, bc, nanmask)."""
    nanmask = np.isnan(dem)
    d = np.array(dem, dtype=np.float32, order="F", copy=True)
    b = np.array(bc, dtype=np.uint8, order="F", copy=True)
    d[nanmask] = -np.inf
    b[nanmask] = 1
    return d, b, nanmask


def plain_512(seed=1, size=512):
    """Workload 1: fractal H=0.7, 200 m relief + U[0, 0.5) m pits, cellsize 30."""
    rng = np.random.default_rng(seed + 1000)
    z = np.asfortranarray(fractal_surface((size, size), 0.7, 200.0, seed))
    z += rng.uniform(0.0, 0.5, size=z.shape).astype(np.float32)
    return np.asfortranarray(z, dtype=np.float32), border_bc(z.shape), 30.0


def plain_4096(seed=2, size=4096):
    """Workload 2: fractal H=0.8, 1000 m relief, 200 inverted Gaussian pits
    (depth 5-50 m, sigma 10-200 cells), rounded to 1 m; border bc."""
    rng = np.random.default_rng(seed + 2000)
    z = np.array(fractal_surface((size, size), 0.8, 1000.0, seed), order="F")
    scale = size / 4096.0
    _gaussian_pits(z, 200, (5.0, 50.0), (10.0 * scale, 200.0 * scale), rng)
    z = np.round(z).astype(np.float32)
    return np.asfortranarray(z), border_bc(z.shape), 30.0


def plain_16384(seed=3, size=16384):
    """Workload 3: fractal H=0.75, 2000 m relief, 5 % NaN nodata disks
    (radius 20-400 cells), 1000 closed depressions up to 100 m deep.
    Returns the raw DEM (with NaN) and the border bc; apply
    ``nan_to_outlets`` for the reference's NaN convention."""
    rng = np.random.default_rng(seed + 3000)
    z = np.array(fractal_surface((size, size), 0.75, 2000.0, seed), order="F")
    scale = size / 16384.0
    _gaussian_pits(z, 1000, (1.0, 100.0), (5.0 * scale + 2, 60.0 * scale + 3), rng)
    nr, nc = z.shape
    target = 0.05 * nr * nc
    covered = 0
    mask = np.zeros(z.shape, dtype=bool, order="F")
    rmin, rmax = max(2.0, 20.0 * scale), max(3.0, 400.0 * scale)
    while covered < target:
        ci, cj = rng.uniform(0, nr), rng.uniform(0, nc)
        rad = rng.uniform(rmin, rmax)
        i0, i1 = max(0, int(ci - rad)), min(nr, int(ci + rad) + 1)
        j0, j1 = max(0, int(cj - rad)), min(nc, int(cj + rad) + 1)
        ii = (np.arange(i0, i1) - ci)[:, None]
        jj = (np.arange(j0, j1) - cj)[None, :]
        disk = ii * ii + jj * jj <= rad * rad
        sub = mask[i0:i1, j0:j1]
        covered += int(np.count_nonzero(disk & ~sub))
        sub |= disk
    z[mask] = np.nan
    return np.asfortranarray(z, dtype=np.float32), border_bc(z.shape), 30.0


def _batch_params(seed, count, side_range):
    """(index, nrows, ncols, hurst, relief) of every tile of workload 4."""
    rng = np.random.default_rng(seed + 4000)
    lo, hi = math.log(side_range[0]), math.log(side_range[1])
    for t in range(count):
        s = math.exp(rng.uniform(lo, hi))
        a = rng.uniform(0.5, 2.0)
        nr = max(8, int(round(s * math.sqrt(a))))
        nc = max(8, int(round(s / math.sqrt(a))))
        h = rng.uniform(0.6, 0.9)
        relief = rng.uniform(50.0, 1500.0)
        yield t, nr, nc, h, relief


def batch_tile_shapes(seed=4, count=512, side_range=(128, 2048)):
    """The (nrows, ncols) of every tile of `batch_tiles`, without building
    the tiles."""
    return [(nr, nc) for _, nr, nc, _, _ in _batch_params(seed, count, side_range)]


def batch_tiles(seed=4, count=512, side_range=(128, 2048), only=None):
    """Workload 4: `count` independent tiles, side log-uniform in side_range,
    aspect ratio U[0.5, 2], Hurst U[0.6, 0.9], relief U[50, 1500] m,
    quantised to 0.1 m.  Returns a list of (dem, bc) pairs; with `only` (a
    collection of tile indices), just those tiles, in index order."""
    out = []
    for t, nr, nc, h, relief in _batch_params(seed, count, side_range):
        if only is not None and t not in only:
            continue
        z = fractal_surface((nr, nc), h, relief, seed * 100003 + t)
        z = (np.round(np.asarray(z, dtype=np.float64) * 10.0) / 10.0).astype(np.float32)
        out.append((np.asfortranarray(z), border_bc((nr, nc))))
    return out


def grad_8192(seed=5, size=8192):
    """Workload 5: fractal H=0.7, 800 m relief; lognormal(0, 0.5) weights."""
    rng = np.random.default_rng(seed + 5000)
    z = np.asfortranarray(fractal_surface((size, size), 0.7, 800.0, seed), dtype=np.float32)
    w = np.asfortranarray(rng.lognormal(0.0, 0.5, size=z.shape).astype(np.float32))
    return z, border_bc(z.shape), w, 30.0


def pcg4d_dem(dims, seed):
    """100 * pcg4d(i, j, seed_hi, seed_lo), the random DEM of the reference's
    property tests (test/grid.c:136-168, hash test/utils.c:6-28)."""
    nr, nc = int(dims[0]), int(dims[1])
    with np.errstate(over="ignore"):
        i = np.arange(nr, dtype=np.uint32)[:, None] * np.ones((1, nc), dtype=np.uint32)
        j = np.ones((nr, 1), dtype=np.uint32) * np.arange(nc, dtype=np.uint32)[None, :]
        c = np.uint32((seed >> 32) & 0xFFFFFFFF)
        d = np.uint32(seed & 0xFFFFFFFF)
        m1, a1 = np.uint32(1664525), np.uint32(1013904223)
        x = i * m1 + a1
        y = j * m1 + a1
        zc = np.full_like(x, c) * m1 + a1
        w = np.full_like(x, d) * m1 + a1
        x = x + y * w
        y = y + zc * x
        zc = zc + x * y
        w = w + y * zc
        x ^= x >> np.uint32(16)
        y ^= y >> np.uint32(16)
        zc ^= zc >> np.uint32(16)
        w ^= w >> np.uint32(16)
        x = x + y * w
        y = y + zc * x
        zc = zc + x * y
        w = w + y * zc
    v = (w >> np.uint32(8)).astype(np.float32) / np.float32(1 << 24)
    return np.asfortranarray(np.float32(100.0) * v)
