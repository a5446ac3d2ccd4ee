"""CPU: two steps of the screen's error model, checked numerically.

1. The screened exact fill (bsf_exact.cu k_chunks_screen) runs the reference's
   incremental trilinear fill (BetaTerrain173.java:582-665) in FP32 on corner
   densities that are within emax of the FP64 ones, and accepts a block's sign
   only when |value| > 2 (emax + 32 u M) + 1e-6, M bounding |corner| + emax. The
   claim behind it: every FP32 block value lies within emax + 16 u M of the FP64
   fill's. Checked here on random cells, many of them crossing zero, with
   corners perturbed by up to emax.
2. The per-octave constants (bsf_screen.cuh): a lerp a + t (b - a) with t in
   [0, 1] adds at most 4 e_t + 6u to its operands' error (convex blend), so a 3D
   octave's FP32 value is within 2.12e-6 of its FP64 one given inputs within
   e_in and fades within e_f. numpy has no fused multiply-add, so the FP32 lerp
   here rounds its product too; that adds u |t (b - a)| <= 4u per level, and the
   check uses 4 e_f + 10u per level.
"""
import numpy as np

U = 2.0 ** -24


def fill(c, dtype):
    """Incremental fill of one cell per row: c[:, 0:4] corners at the lower
    level ((x, z), (x, z + 1), (x + 1, z), (x + 1, z + 1)), c[:, 4:8] the upper."""
    c = c.astype(dtype)
    d1, d2, d3, d4 = (c[:, k].copy() for k in range(4))
    q = dtype(0.125)
    d5, d6, d7, d8 = ((c[:, 4 + k] - c[:, k]) * q for k in range(4))
    out = []
    quarter = dtype(0.25)
    for _ in range(8):
        d10, d11 = d1.copy(), d2.copy()
        d12 = (d3 - d1) * quarter
        d13 = (d4 - d2) * quarter
        for _ in range(4):
            d15 = d10.copy()
            d16 = (d11 - d10) * quarter
            for _ in range(4):
                out.append(d15.copy())
                d15 = d15 + d16
            d10 = d10 + d12
            d11 = d11 + d13
        d1 = d1 + d5
        d2 = d2 + d6
        d3 = d3 + d7
        d4 = d4 + d8
    return np.stack(out, axis=1)


def test_fp32_fill_within_corner_bound_plus_rounding():
    rng = np.random.default_rng(17)
    n = 40000
    scale = np.where(rng.random((n, 1)) < 0.5, 3.0, 150.0)  # near the surface and far from it
    c64 = (rng.standard_normal((n, 8)) * scale + rng.standard_normal((n, 1)) * scale * 0.5)
    emax = np.abs(c64).max(axis=1) * 1e-4 * rng.random(n)  # the corners' own bounds
    c32_in = c64 + (rng.random((n, 8)) * 2 - 1) * emax[:, None]  # screened corners within emax
    c32_in = c32_in.astype(np.float32).astype(np.float64)
    emax = np.maximum(emax, np.abs(c32_in - c64).max(axis=1))  # rounding to FP32 included
    v64 = fill(c64, np.float64)
    v32 = fill(c32_in, np.float32).astype(np.float64)
    m = np.abs(c32_in).max(axis=1) + emax
    err = np.abs(v32 - v64).max(axis=1)
    claim = emax + 16 * U * m
    assert (err <= claim).all(), float((err / claim).max())
    # the test's margin: the kernel takes 32 u M and doubles the whole
    assert (2 * (emax + 32 * U * m) + 1e-6 > err).all()


def grad(h, x, y, z):
    u = np.where(h < 8, x, y)
    v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
    return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)


def lerp(t, a, b):
    return a + t * (b - a)


def fade(t):
    return t * t * t * (t * (t * 6 - 15) + 10)


def test_octave3_value_within_e_oct3_derivation():
    rng = np.random.default_rng(23)
    n = 200000
    fx, fy, fz = (rng.random(n) for _ in range(3))
    h = rng.integers(0, 16, (n, 8))
    ux, uy, uz = fade(fx), fade(fy), fade(fz)

    def value(dtype, x, y, z, x1, y1, z1, tx, ty, tz):
        g = [grad(h[:, 0], x, y, z), grad(h[:, 1], x1, y, z), grad(h[:, 2], x, y1, z), grad(h[:, 3], x1, y1, z),
             grad(h[:, 4], x, y, z1), grad(h[:, 5], x1, y, z1), grad(h[:, 6], x, y1, z1), grad(h[:, 7], x1, y1, z1)]
        g = [gi.astype(dtype) for gi in g]
        c00, c10 = lerp(tx, g[0], g[1]), lerp(tx, g[2], g[3])
        c01, c11 = lerp(tx, g[4], g[5]), lerp(tx, g[6], g[7])
        return lerp(tz, lerp(ty, c00, c10), lerp(ty, c01, c11))

    v64 = value(np.float64, fx, fy, fz, fx - 1, fy - 1, fz - 1, ux, uy, uz)
    f32 = np.float32
    v32 = value(f32, fx.astype(f32), fy.astype(f32), fz.astype(f32), fx.astype(f32) - f32(1), fy.astype(f32) - f32(1),
                fz.astype(f32) - f32(1), ux.astype(f32), uy.astype(f32), uz.astype(f32)).astype(np.float64)
    e_in = U + 2.0 ** -25 + 2.0 ** -30
    e_f = U + 2.0 ** -30
    per_level = 4 * e_f + 10 * U  # 6u for the fma form, + 4u for numpy's separate product rounding
    bound = (2 * e_in + 2 * U) + 3 * per_level
    err = np.abs(v32 - v64).max()
    assert err <= bound, (err, bound)
    assert bound < 3.0e-6 + 3 * 4 * U  # the E_OCT3 in use, plus numpy's extra rounding
