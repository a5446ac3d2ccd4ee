"""CPU checks of the screened kernels' analytic bounds (bsf_screen.cuh).

OCTAVE3_ABS_MAX bounds |value| of one legacy 3D Perlin octave
(NoiseGeneratorPerlin173.java:172-285): a trilinear blend, with fade weights,
of gradient terms +-a +-b over two distinct components of each corner's offset.
The y offset comes from the cell's first sample while y's weight comes from the
sample's own fraction, so |dy| < 1 is all that is known about it.
"""
import re
from pathlib import Path

import numpy as np

HEADER = Path(__file__).resolve().parents[1] / "betaseedfinder_gb300" / "csrc" / "bsf_screen.cuh"


def octave3_abs_max():
    m = re.search(r"constexpr float OCTAVE3_ABS_MAX = ([0-9.]+)f;", HEADER.read_text())
    assert m, "OCTAVE3_ABS_MAX not found"
    return float(m.group(1))


def fade(t):
    return t ** 3 * (t * (t * 6 - 15) + 10)


def corner_bound(x, z):
    """F(x, z): the fade-weighted sum of 1 + max(|dx|, |dz|) over the 4 (x, z) corners."""
    wx, wz = (1 - fade(x), fade(x)), (1 - fade(z), fade(z))
    return sum(wx[cx] * wz[cz] * (1 + np.maximum(abs(x - cx), abs(z - cz))) for cx in (0, 1) for cz in (0, 1))


def test_octave_bound_covers_the_corner_model():
    n = 2001
    g = np.linspace(0.0, 1.0, n)
    X, Z = np.meshgrid(g, g)
    grid_max = corner_bound(X, Z).max()
    # |dF/dx|, |dF/dz| <= 2 * max fade' (1.875) + 1: any point lies within h/2 of a
    # grid point in each coordinate
    h = 1.0 / (n - 1)
    assert grid_max + 4.75 * h <= octave3_abs_max()


def grad3(h, x, y, z):
    h &= 15
    u = np.where(h < 8, x, y)
    v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
    return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)


def test_random_legacy_octave_values_stay_inside_the_bound():
    rng = np.random.default_rng(7)
    n = 200_000
    x, z = rng.random(n), rng.random(n)
    cell = rng.random(n)   # the cell's first-sample fraction: the y offset
    own = rng.random(n)    # the sample's own fraction: the y weight
    hashes = rng.integers(0, 256, size=(n, 8))
    fx, fy, fz = fade(x), fade(own), fade(z)
    value = np.zeros(n)
    for k in range(8):
        cx, cy, cz = k & 1, (k >> 1) & 1, (k >> 2) & 1
        w = (fx if cx else 1 - fx) * (fy if cy else 1 - fy) * (fz if cz else 1 - fz)
        value += w * grad3(hashes[:, k], x - cx, cell - cy, z - cz)
    assert (np.abs(value) <= corner_bound(x, z) + 1e-12).all()
    assert np.abs(value).max() <= octave3_abs_max()


def test_oracle_legacy_octaves_stay_inside_the_bound():
    """The oracle's FP64 legacy 3D octave column (17 Y samples with the cell
    reuse of NoiseGeneratorPerlin173.java:172-285) on real generator states and
    random lattice coordinates and Y scales: every sample is inside the bound."""
    import ctypes
    from oracle import pyoracle as po
    rng = np.random.default_rng(11)
    out = np.zeros(17)
    worst = 0.0
    for s in range(12):
        seed = int(rng.integers(-2 ** 62, 2 ** 62))
        for state in (0, 5, 15, 16, 27, 33, 39):  # noise2, noise3 and noise1 generators
            perm, abc = po.world_state(seed, state)
            for _ in range(60):
                xs, zs = rng.uniform(-5e3, 5e3, 2)
                sy = float(rng.choice([684.412 / 2 ** k for k in range(16)] + [4.27757 / 2 ** k for k in range(8)]))
                po.lib().or_perlin_column17_test(perm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                                 abc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                 float(xs), sy, float(zs), 0,
                                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
                worst = max(worst, float(np.abs(out).max()))
    assert worst <= octave3_abs_max()
