"""Seeded synthetic inputs for the multi-spline workloads.

Everything is derived from a splitmix64 counter stream so that the same seed
gives the same numbers with numpy on any machine and with the library's
device-side generator (``einspline_gb300_fill_uniform``), which uses the
identical formula.  Uniform draws are ``lo + (hi - lo) * u`` with
``u = (z >> 11) * 2**-53`` in double precision.

Workloads (no public dataset is involved; these stand in for the shapes and
value distributions the benchmark names):
  * grid data i.i.d. uniform in [-1, 1];
  * sums of random periodic plane waves plus 1e-2 uniform noise;
  * points uniform in the box, or walkers of uneven point counts.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """Elements offset..offset+n-1 of the splitmix64 stream for ``seed``:
    z_i = mix(seed + (i + 1) * golden)."""
    i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, n: int, lo: float = 0.0, hi: float = 1.0, offset: int = 0) -> np.ndarray:
    u = (splitmix64(seed, n, offset) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return lo + (hi - lo) * u


def grid_data_uniform(seed: int, M: tuple, num_splines: int, dtype=np.float32, complex_: bool = False):
    """Data for ``num_splines`` splines on an Mx x My x Mz grid, i.i.d.
    uniform in [-1, 1].  Spline s uses stream offset s * (values per spline).
    Returns shape (num_splines, Mx, My, Mz) (complex: trailing axis 2)."""
    per = int(np.prod(M)) * (2 if complex_ else 1)
    out = uniform(seed, per * num_splines, -1.0, 1.0).astype(dtype)
    shape = (num_splines,) + tuple(M) + ((2,) if complex_ else ())
    return out.reshape(shape)


def grid_data_planewaves(seed: int, M: tuple, num_splines: int, waves: int = 8, kmax: int = 4,
                         noise: float = 1e-2, dtype=np.float64):
    """Each spline: the real part of a sum of ``waves`` periodic plane waves
    exp(2 pi i k.r) with integer k (|k_a| <= kmax) and random complex
    amplitude of modulus <= 1, plus ``noise`` * U[-1, 1], on the unit-cube grid
    r = (ix/Mx, iy/My, iz/Mz).  Returns (num_splines, Mx, My, Mz) and the wave
    parameters (k: [S, W, 3] ints, amp: [S, W] complex) for analytic checks."""
    Mx, My, Mz = M
    nparam = num_splines * waves
    ku = uniform(seed, 3 * nparam, 0.0, 1.0).reshape(num_splines, waves, 3)
    k = np.floor(ku * (2 * kmax + 1)).astype(np.int64) - kmax
    au = uniform(seed + 1, 2 * nparam, -1.0, 1.0).reshape(num_splines, waves, 2)
    amp = (au[..., 0] + 1j * au[..., 1]) / np.sqrt(2.0)
    xs = [np.arange(m) / m for m in (Mx, My, Mz)]
    out = np.empty((num_splines, Mx, My, Mz), dtype=dtype)
    noise_vals = uniform(seed + 2, num_splines * Mx * My * Mz, -1.0, 1.0).reshape(out.shape)
    for s in range(num_splines):
        acc = np.zeros((Mx, My, Mz), dtype=np.complex128)
        for w in range(waves):
            ex = np.exp(2j * np.pi * k[s, w, 0] * xs[0])
            ey = np.exp(2j * np.pi * k[s, w, 1] * xs[1])
            ez = np.exp(2j * np.pi * k[s, w, 2] * xs[2])
            acc += amp[s, w] * ex[:, None, None] * ey[None, :, None] * ez[None, None, :]
        out[s] = acc.real + noise * noise_vals[s]
    return out, k, amp


def points_uniform(seed: int, npts: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)) -> np.ndarray:
    """npts points uniform in the box [lo, hi), shape (npts, len(lo)) float64
    (3 coordinates by default; 1 or 2 for the 1D/2D multi-splines)."""
    dims = len(lo)
    u = uniform(seed, dims * npts, 0.0, 1.0).reshape(npts, dims)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    p = lo + (hi - lo) * u
    return np.minimum(p, np.nextafter(hi, lo))


def walker_sizes(seed: int, nwalkers: int, lo: int = 32, hi: int = 512) -> np.ndarray:
    """Uneven per-walker point counts, uniform in {lo..hi}."""
    u = uniform(seed, nwalkers, 0.0, 1.0)
    return (lo + np.floor(u * (hi - lo + 1))).astype(np.int64)


def poisson_arrivals(seed: int, n: int, rate_hz: float) -> np.ndarray:
    """Arrival times (seconds) of a Poisson stream with the given rate."""
    u = uniform(seed, n, 0.0, 1.0)
    gaps = -np.log1p(-u) / rate_hz
    return np.cumsum(gaps)


def uniform_at(seed: int, idx: np.ndarray, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    """Elements of the uniform stream at arbitrary indices idx (int64 array)."""
    i = np.asarray(idx, dtype=np.uint64) + np.uint64(1)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return lo + (hi - lo) * u
