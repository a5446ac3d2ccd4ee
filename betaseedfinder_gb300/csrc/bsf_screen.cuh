// FP32 screening of lattice density signs with rigorous error bounds.
//
// GB300's FP64 pipe issues about 1.75 operations per clock per SM against 128
// for FP32, and every output of this path is a function of density *signs*
// (stage masks, coarse cells, block bitmaps). So the octave arithmetic runs in
// FP32 from exact FP64 lattice coordinates, each result carries an upper bound
// of its distance to the FP64 value the reference computes, and a sign is
// accepted only when |value| exceeds that bound. Columns with any point inside
// its bound are recomputed with the exact FP64 path (bsf_device.cuh), so the
// decisions are bit-identical to the reference by construction.
//
// Error model (u = 2^-24, FP32 round-to-nearest, products with FMA rounded
// once), against the FP64 value of the same expression. Inputs: lattice
// fractions (and fraction - 1) within e_in = u + 2^-25 + 2^-30 < 1.0e-7 of
// the FP64 ones (rounded, the subtraction of 1 rounded, the double-float
// axis term), fades within e_f = u + 2^-30 < 6.1e-8. A gradient is +-a +- b
// of two inputs: e_g <= 2 e_in + 2u (|g| <= 2) = 3.2e-7. A lerp
// fma(t, b - a, a) with t in [0, 1] is the convex blend (1 - t) a + t b of its
// operands up to the rounding of b - a (<= 4u, times t <= 1) and of the fma
// (<= 2u, |value| <= 2), and t's error enters times |b - a| <= 4, so each
// level adds at most 4 e_f + 6u = 6.0e-7 to its operands' error. One 3D
// octave value (gradients, then x, y and z lerps): 3.2e-7 + 3 * 6.0e-7 =
// 2.12e-6 -> E_OCT3 = 3e-6. One 2D octave (two lerp levels): 1.52e-6 ->
// E_OCT2 = 2.5e-6. (The products of two errors are below 1e-13; the FP64
// side's own rounding below 1e-14.) bsf_screen_probe measures both on the GPU.
// Octave sums add w_o * E plus the running-sum rounding u * 2 * sum(w).
// Everything after the octave sums is tracked per value with (value, bound)
// pairs (struct Fe) whose operations add the propagated and rounding terms;
// piecewise branches add their jump or mark the column ambiguous. The final
// bound is doubled and gets an absolute 1e-6 for the FP64 side's own rounding.
#pragma once

#include "bsf_device.cuh"

namespace bsf {
namespace screen {

constexpr float U = 5.9604645e-8f;  // 2^-24
constexpr float E_OCT3 = 3.0e-6f;
constexpr float E_OCT2 = 2.5e-6f;

// Value with an upper bound of its absolute error against the FP64 reference.
struct Fe {
    float v, e;
};

__device__ __forceinline__ Fe fe_exact(double x) {
    const float f = static_cast<float>(x);
    return Fe{f, fabsf(f) * U};
}
__device__ __forceinline__ Fe fe_add(Fe a, Fe b) {
    const float v = a.v + b.v;
    return Fe{v, a.e + b.e + fabsf(v) * U};
}
__device__ __forceinline__ Fe fe_sub(Fe a, Fe b) {
    const float v = a.v - b.v;
    return Fe{v, a.e + b.e + fabsf(v) * U};
}
__device__ __forceinline__ Fe fe_mul(Fe a, Fe b) {
    const float v = a.v * b.v;
    return Fe{v, fabsf(a.v) * b.e + fabsf(b.v) * a.e + a.e * b.e + fabsf(v) * U};
}
__device__ __forceinline__ Fe fe_scale(Fe a, float c) {  // c exact in FP32
    const float v = a.v * c;
    return Fe{v, a.e * fabsf(c) + fabsf(v) * U};
}
// a / b for b bounded away from zero (b.e < |b.v|); returns a huge bound otherwise.
__device__ __forceinline__ Fe fe_div(Fe a, Fe b) {
    const float v = a.v / b.v;
    const float den = fabsf(b.v) - b.e;
    if (!(den > 0.0f)) return Fe{v, 3.0e38f};
    return Fe{v, (a.e + fabsf(v) * b.e) / den + 2.0f * fabsf(v) * U};
}
__device__ __forceinline__ Fe fe_clamp_hi(Fe a, float hi) { return Fe{a.v > hi ? hi : a.v, a.e}; }
__device__ __forceinline__ Fe fe_clamp_lo(Fe a, float lo) { return Fe{a.v < lo ? lo : a.v, a.e}; }

// ---- lattice axis entries --------------------------------------------------
// One coordinate of one octave: exact FP64 lattice index and fraction, stored
// as FP32 fraction, FP32 (fraction - 1) and FP32 fade, each the rounding of the
// exact FP64 value.
struct AxisF {
    float f, f1, fd;
    int i;
};

// Axis entry for the FP32 tables: the exact lattice index and fraction of the
// FP64 coordinate (floor and the subtraction are exact), and the fade rounded
// to FP32. The fade is evaluated with FMAs, which moves its FP64 value by about
// 1e-16 before the rounding to FP32 (within the inputs' u|x| model). This runs
// for every table entry of every staged world, on GB300's narrow FP64 pipe.
__device__ __forceinline__ AxisF make_axis(double scaled, double offset) {
    double v = scaled + offset;
    const double fl = floor(v);
    v -= fl;
    AxisF a;
    a.i = static_cast<int>(fl) & 255;
    a.f = static_cast<float>(v);
    a.f1 = a.f - 1.0f;
    const double t2 = v * v;
    a.fd = static_cast<float>(t2 * v * fma(v, fma(v, 6.0, -15.0), 10.0));
    return a;
}

// Y axis entry of one 3D octave in FP32: the cell-start fraction (and minus 1),
// own fade, cell ordinal and lattice index.
struct YF {
    float cf, cf1, fd;
    unsigned char yi, cell, pad0, pad1;
};

__device__ __forceinline__ void build_yf(const YEntry* y64, YF* out) {
    for (int y = 0; y < 17; ++y) {
        out[y].cf = static_cast<float>(y64[y].cellFrac);
        out[y].cf1 = static_cast<float>(y64[y].cellFrac - 1.0);
        out[y].fd = static_cast<float>(y64[y].fade);
        out[y].yi = static_cast<unsigned char>(y64[y].yi);
        out[y].cell = static_cast<unsigned char>(y64[y].cell);
        out[y].pad0 = out[y].pad1 = 0;
    }
}

__device__ __forceinline__ float grad3f(int hash, float x, float y, float z) {
    const int h = hash & 15;
    const float u = h < 8 ? x : y;
    const float v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}

__device__ __forceinline__ float lerpf(float t, float a, float b) { return __fmaf_rn(t, b - a, a); }

// FP32 3D octave over levels [Y0, Y0+N): acc[k] (+)= w * value.
template <int Y0, int N>
__device__ __forceinline__ void octave3f(const std::uint8_t* p, const AxisF& ax, const AxisF& az, const YF* yt,
                                         float w, float* acc, bool first) {
    const int xp0 = P(p, ax.i);
    const int xp1 = P(p, ax.i + 1);
    int active = -1;
    float c00 = 0.f, c01 = 0.f, c10 = 0.f, c11 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const YF e = yt[Y0 + k];
        if (e.cell != active) {
            active = e.cell;
            const int p0 = xp0 + e.yi;
            const int p00 = P(p, p0) + az.i;
            const int p01 = P(p, p0 + 1) + az.i;
            const int p1 = xp1 + e.yi;
            const int p10 = P(p, p1) + az.i;
            const int p11 = P(p, p1 + 1) + az.i;
            c00 = lerpf(ax.fd, grad3f(P(p, p00), ax.f, e.cf, az.f), grad3f(P(p, p10), ax.f1, e.cf, az.f));
            c01 = lerpf(ax.fd, grad3f(P(p, p01), ax.f, e.cf1, az.f), grad3f(P(p, p11), ax.f1, e.cf1, az.f));
            c10 = lerpf(ax.fd, grad3f(P(p, p00 + 1), ax.f, e.cf, az.f1), grad3f(P(p, p10 + 1), ax.f1, e.cf, az.f1));
            c11 = lerpf(ax.fd, grad3f(P(p, p01 + 1), ax.f, e.cf1, az.f1), grad3f(P(p, p11 + 1), ax.f1, e.cf1, az.f1));
        }
        const float v = lerpf(az.fd, lerpf(e.fd, c00, c01), lerpf(e.fd, c10, c11)) * w;
        acc[k] = first ? v : acc[k] + v;
    }
}

// octave3f with the first level y0 at run time (one instantiation serves every level
// range of a kernel, which keeps its loop code in the instruction cache). Levels
// past 16 are clamped to 16: their values are computed but never read.
template <int N>
__device__ __forceinline__ void octave3f_y(const std::uint8_t* p, const AxisF& ax, const AxisF& az, const YF* yt,
                                           int y0, float w, float* acc) {
    const int xp0 = P(p, ax.i);
    const int xp1 = P(p, ax.i + 1);
    int active = -1;
    float c00 = 0.f, c01 = 0.f, c10 = 0.f, c11 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const YF e = yt[min(y0 + k, 16)];
        if (e.cell != active) {
            active = e.cell;
            const int p0 = xp0 + e.yi;
            const int p00 = P(p, p0) + az.i;
            const int p01 = P(p, p0 + 1) + az.i;
            const int p1 = xp1 + e.yi;
            const int p10 = P(p, p1) + az.i;
            const int p11 = P(p, p1 + 1) + az.i;
            c00 = lerpf(ax.fd, grad3f(P(p, p00), ax.f, e.cf, az.f), grad3f(P(p, p10), ax.f1, e.cf, az.f));
            c01 = lerpf(ax.fd, grad3f(P(p, p01), ax.f, e.cf1, az.f), grad3f(P(p, p11), ax.f1, e.cf1, az.f));
            c10 = lerpf(ax.fd, grad3f(P(p, p00 + 1), ax.f, e.cf, az.f1), grad3f(P(p, p10 + 1), ax.f1, e.cf, az.f1));
            c11 = lerpf(ax.fd, grad3f(P(p, p01 + 1), ax.f, e.cf1, az.f1), grad3f(P(p, p11 + 1), ax.f1, e.cf1, az.f1));
        }
        acc[k] = lerpf(az.fd, lerpf(e.fd, c00, c01), lerpf(e.fd, c10, c11)) * w;
    }
}

// FP32 2D octave value (legacy 2D sampler, NoiseGeneratorPerlin173.java:188-223).
__device__ __forceinline__ float octave2f(const std::uint8_t* p, const AxisF& ax, const AxisF& az) {
    const int a0 = P(p, ax.i);
    const int a1 = P(p, a0) + az.i;
    const int b0 = P(p, ax.i + 1);
    const int b1 = P(p, b0) + az.i;
    // grad2_legacy in FP32: the signed-zero terms cannot change a value beyond its bound.
    const int h = P(p, a1) & 15;
    float g0;
    switch (h) {
        case 0: case 2: g0 = ax.f; break;
        case 1: case 3: g0 = -ax.f; break;
        case 4: g0 = ax.f + az.f; break;
        case 5: g0 = -ax.f + az.f; break;
        case 6: g0 = ax.f - az.f; break;
        case 7: g0 = -ax.f - az.f; break;
        case 8: case 9: case 13: g0 = az.f; break;
        case 12: g0 = ax.f; break;
        case 14: g0 = -ax.f; break;
        default: g0 = -az.f; break;
    }
    const float q0 = lerpf(ax.fd, g0, grad3f(P(p, b1), ax.f1, 0.0f, az.f));
    const float q1 = lerpf(ax.fd, grad3f(P(p, a1 + 1), ax.f, 0.0f, az.f1), grad3f(P(p, b1 + 1), ax.f1, 0.0f, az.f1));
    return lerpf(az.fd, q0, q1);
}

// Bound of an octave sum: weights 2^0..2^(n-1), per-octave bound e, running
// sum |S_k| <= 2 * (2^(k+1) - 1) rounded once per add.
__host__ __device__ constexpr float octave_sum_bound(int n, float e) {
    return static_cast<float>((1 << n) - 1) * e + U * 2.0f * static_cast<float>(1 << (n + 1));
}
constexpr float E_N1 = octave_sum_bound(8, E_OCT3);   // noise1
constexpr float E_N4 = octave_sum_bound(10, E_OCT2);  // noise4
constexpr float E_N5 = octave_sum_bound(16, E_OCT2);  // noise5

// Bound of a 16-octave sum taken from the largest weight down (2^15 first): the
// per-octave terms as above, and each of the 16 adds rounds a partial sum no
// larger than 2 * (2^16 - 1).
__host__ __device__ constexpr float octave_sum_bound_desc(int n, float e) {
    return static_cast<float>((1 << n) - 1) * e + U * static_cast<float>(n) * 2.0f * static_cast<float>(1 << n);
}
constexpr float E_N2_DESC = octave_sum_bound_desc(16, E_OCT3);

// Largest |value| of one legacy 3D octave. The value is the trilinear blend,
// weights fade(x) fade(y) fade(z) over the 8 cell corners, of gradient terms
// +-a +- b, where a and b are two distinct components of the corner offset
// (dx, dy, dz). |dy| < 1 (the legacy cell reuse decouples y's offset from its
// fade), so a corner's term is at most 1 + max(|dx|, |dz|), and the value is at
// most F(x, z) = sum over the 4 (x, z) corners of wx wz (1 + max(|dx|, |dz|)).
// F's maximum over [0, 1]^2 is 1.5353 (on a 2001^2 grid; F is 4.75-Lipschitz
// in each coordinate, so the true maximum is below 1.538). tests/ recheck it.
constexpr float OCTAVE3_ABS_MAX = 1.55f;

// Simplex sample with exact FP64 lattice geometry and an FP32 kernel: the
// offsets d11..d16 are FP64 (they cancel large coordinates), the falloff and
// gradients are FP32 tracked with bounds. Returns 70*(n0+n1+n2) with its bound.
// One simplex corner, n = t^4 * (g . (x, z)) with t = 0.5 - x^2 - z^2 (0 when
// t < 0), in FP32 with a first-order error bound (NoiseGenerator2173.java:
// 111-174, simplexGrad2 :61-75). Inputs x, z lie within dx = u|x| + eg, dz =
// u|z| + eg of the reference's FP64 offsets.
//   t:  |t - t*| <= et = (2|x| + dx) dx + (2|z| + dz) dz + u (x^2 + z^2 + |c| + |t|),
//       c = 0.5 - x^2, the four roundings of t's evaluation included;
//   g:  the gradient picks (gx, gz) in {-1, 0, 1}^2, so d = gx x + gz z has
//       |d - d*| <= egd = dx + dz + u |d|;
//   n:  with tp = t + et >= max(t, t*): |t^4 - t*^4| <= 4 tp^3 et, so
//       |n - n*| <= 4 tp^3 et (|d| + egd) + tp^4 egd + 4u tp^4 |d|, the last term
//       for the roundings of t^2, t^4 and the product.
// When |t| <= et the reference may or may not add the corner: it returns 0 and
// adds the largest contribution, (|t| + et)^4 * 2, to the bound. Written without
// branches on the gradient (lanes of a warp hold different corners).
// The first-order terms leave out products of errors, and measured errors came
// within 0.74 of them (bsf_screen_probe), so et and the returned term are taken
// twice: every tracked bound downstream (climate, column shape) then keeps a
// margin of two over its measured error, and the intermediate branch decisions
// that use a bound undoubled (the corner sign here, the d6 branch, the noise
// selector) inherit it.
__device__ __forceinline__ float simplex_corner(float x, float z, int g, float& err, float eg = 0.0f) {
    const float ax = fabsf(x), az = fabsf(z);
    const float dx = ax * U + eg, dz = az * U + eg;
    const float xx = x * x, zz = z * z;
    const float c = 0.5f - xx;
    const float t = c - zz;
    const float et = 2.0f * ((2.0f * ax + dx) * dx + (2.0f * az + dz) * dz + U * (xx + zz + fabsf(c) + fabsf(t)));
    // simplexGrad2: g 0..3 (+-x +-z), 4..7 (+-x), 8..11 (+-z)
    const float gx = g < 8 ? ((g & 1) ? -1.0f : 1.0f) : 0.0f;
    const float gz = g < 4 ? ((g & 2) ? -1.0f : 1.0f) : (g < 8 ? 0.0f : ((g & 1) ? -1.0f : 1.0f));
    const float d = gx * x + gz * z;
    const float ad = fabsf(d);
    const float egd = dx + dz + U * ad;
    const float tp = fabsf(t) + et;
    const float tp2 = tp * tp, tp4 = tp2 * tp2;
    if (t <= et) {  // t* < 0 (nothing added) or its sign is undecided
        if (t >= -et) err += tp4 * 2.0f;
        return 0.0f;
    }
    err += 2.0f * (4.0f * tp2 * tp * et * (ad + egd) + tp4 * (egd + 4.0f * U * ad));
    const float t2 = t * t;
    return (t2 * t2) * d;
}

// Out of line: the climate's ten octaves would otherwise inline ten copies.
static __device__ __noinline__ Fe simplex2f(const Gen& s, double xs, double zs) {
    constexpr double F = 0.3660254037844386;
    constexpr double G = 0.21132486540518713;
    const double d5 = xs + s.a;
    const double d6 = zs + s.b;
    const double d7 = (d5 + d6) * F;
    const int j1 = simplex_floor(d5 + d7);
    const int k1 = simplex_floor(d6 + d7);
    const double d8 = static_cast<double>(j1 + k1) * G;
    const double d11 = d5 - (static_cast<double>(j1) - d8);
    const double d12 = d6 - (static_cast<double>(k1) - d8);
    const int b0 = d11 > d12 ? 1 : 0;
    const int b1 = d11 > d12 ? 0 : 1;
    const double d13 = d11 - static_cast<double>(b0) + G;
    const double d14 = d12 - static_cast<double>(b1) + G;
    const double d15 = d11 - 1.0 + 2.0 * G;
    const double d16 = d12 - 1.0 + 2.0 * G;
    const int l1 = j1 & 255;
    const int i2 = k1 & 255;
    const int g0 = P(s.p, l1 + P(s.p, i2)) % 12;
    const int g1 = P(s.p, l1 + b0 + P(s.p, i2 + b1)) % 12;
    const int g2 = P(s.p, l1 + 1 + P(s.p, i2 + 1)) % 12;
    float err = 0.0f;
    const float n0 = simplex_corner(static_cast<float>(d11), static_cast<float>(d12), g0, err);
    const float n1 = simplex_corner(static_cast<float>(d13), static_cast<float>(d14), g1, err);
    const float n2 = simplex_corner(static_cast<float>(d15), static_cast<float>(d16), g2, err);
    const float sum = n0 + n1 + n2;
    const float v = 70.0f * sum;
    return Fe{v, 70.0f * (err + 2.0f * fabsf(sum) * U) + fabsf(v) * U};
}

// ---- simplex lattice geometry in double-float --------------------------------
// The geometry of a simplex sample (skew, cell floors, the corner order and the
// corner offsets) decides which gradients are read, so the reference's FP64
// values must pick the same cell. GB300's FP64 pipe is 1/64 of its FP32 rate and
// the climate's ten octaves per column are the screened kernels' main FP64 load,
// so the geometry runs here on pairs of floats (h + l, ~48 bits): exact products
// by FMA, error-free sums (Knuth's two-sum, Dekker's fast two-sum), after
// Dekker (1971) and the double-double algorithms of Hida, Li and Bailey (2001).
// Every value it yields is within 2^-32 of the real value of the reference
// expression for |values| < 2^10 (about ten pair operations of relative error
// 2^-46 each, inputs split at 2^-48), and the reference's FP64 values are
// within 2^-40 of it. A floor
// or the corner-order comparison whose argument lies within SIMPLEX_EPS = 2^-28
// of its decision point is left to the FP64 path; every other decision equals
// the FP64 one. The offsets, rounded to FP32, then carry u|x| + 2^-28.
constexpr float SIMPLEX_EPS = 3.7252903e-9f;  // 2^-28

struct DF {
    float h, l;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return DF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    DF s = two_sum(a.h, b.h);
    const DF t = two_sum(a.l, b.l);
    s.l = s.l + t.h;
    s = fast_two_sum(s.h, s.l);
    s.l = s.l + t.l;
    return fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF df_mul_f(float a, DF b) {  // a * (b.h + b.l)
    const float p = a * b.h;
    float e = __fmaf_rn(a, b.h, -p);
    e = __fmaf_rn(a, b.l, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = a.h * b.h;
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ DF df_of(double x) {  // split of an FP64 value (2^-48 relative)
    const float h = __double2float_rn(x);
    return DF{h, __double2float_rn(x - static_cast<double>(h))};
}
// The reference's simplex floor (v > 0 ? (int)v : (int)v - 1) of a pair value;
// false when the value is within SIMPLEX_EPS of an integer, where that floor and
// the FP64 rounding could disagree. n = floor(v.h); v lies in [n - |v.l|, n + 1),
// and its distances to n and n + 1 are taken with exact two-sums, so they are
// accurate to far below SIMPLEX_EPS however close to an integer v is.
__device__ __forceinline__ bool df_floor(DF v, int& out) {
    const float n = floorf(v.h);
    const DF a = two_sum(v.h, -n);
    const DF b = two_sum(v.h, -(n + 1.0f));
    const float to_n = a.h + (a.l + v.l);     // v - n
    const float to_n1 = b.h + (b.l + v.l);    // v - (n + 1)
    out = static_cast<int>(n) + (to_n < 0.0f ? -1 : 0) + (to_n1 >= 0.0f ? 1 : 0);
    return fabsf(to_n) > SIMPLEX_EPS && fabsf(to_n1) > SIMPLEX_EPS;
}

// Axis entry (as make_axis) from double-float inputs: `coord` an integer
// lattice coordinate, sc the octave's FP64 scale and off the generator's FP64
// offset, both split into float pairs. coord * sc + off (|.| < 2^17), its floor
// and fraction and the fraction's fade are taken in double-float: within 2^-32
// of the real values, and the reference's FP64 sum is within 2^-36 of its real
// value. Rounded to FP32, the fraction and fade then carry u|x| plus at most
// 2^-30 (the fade's slope is below 2) against the FP64 entry: the e_in and
// e_f of the error model above count it. false when the sum is within
// SIMPLEX_EPS of an integer: the FP64 floor decides that entry.
__device__ __forceinline__ bool make_axis_df(int coord, DF sc, DF off, AxisF& a) {
    const DF v = df_add(df_mul_f(static_cast<float>(coord), sc), off);
    const float n = floorf(v.h);
    const DF lo = two_sum(v.h, -n);
    DF fr = fast_two_sum(lo.h, lo.l + v.l);  // v - n, exact to the pair's precision
    float base = n;
    if (fr.h < 0.0f) {
        fr = df_add(fr, DF{1.0f, 0.0f});
        base -= 1.0f;
    } else if (fr.h >= 1.0f) {
        fr = df_add(fr, DF{-1.0f, 0.0f});
        base += 1.0f;
    }
    if (!(fr.h > SIMPLEX_EPS && fr.h < 1.0f - SIMPLEX_EPS)) return false;
    a.i = static_cast<int>(base) & 255;
    a.f = fr.h + fr.l;
    a.f1 = a.f - 1.0f;
    // fade = t^3 (t (6t - 15) + 10), the reference's expression
    const DF inner = df_add(df_mul(fr, df_add(df_mul_f(6.0f, fr), DF{-15.0f, 0.0f})), DF{10.0f, 0.0f});
    const DF t3 = df_mul(df_mul(fr, fr), fr);
    const DF fd = df_mul(t3, inner);
    a.fd = fd.h + fd.l;
    return true;
}

// The ten climate generators' FP64 offsets a and b as float pairs (a.h, a.l,
// b.h, b.l), split once per staged world: climate_split(off of state ST_TEMP + i).
__device__ __forceinline__ float4 climate_split(const double* abc) {
    const DF a = df_of(abc[0]), b = df_of(abc[1]);
    return make_float4(a.h, a.l, b.h, b.l);
}

// simplex2f with the geometry in double-float (xs = X * sx, zs = Z * sx for the
// integer block coordinates X, Z; ab = climate_split of the generator); false
// when a decision is too close to call, in which case the caller takes the FP64
// geometry.
static __device__ __noinline__ bool simplex2f_df(const Gen& s, float4 ab, int bx, int bz, double sx, Fe& out) {
    constexpr double F = 0.3660254037844386;
    constexpr double G = 0.21132486540518713;
    constexpr float FH = static_cast<float>(F), FL = static_cast<float>(F - static_cast<double>(FH));
    constexpr float GH = static_cast<float>(G), GL = static_cast<float>(G - static_cast<double>(GH));
    constexpr double G1 = G - 1.0, G2 = 2.0 * G - 1.0;  // corner offsets' constants, split like G
    constexpr float G1H = static_cast<float>(G1), G1L = static_cast<float>(G1 - static_cast<double>(G1H));
    constexpr float G2H = static_cast<float>(G2), G2L = static_cast<float>(G2 - static_cast<double>(G2H));
    const DF sxd = df_of(sx);
    const DF d5 = df_add(df_mul_f(static_cast<float>(bx), sxd), DF{ab.x, ab.y});
    const DF d6 = df_add(df_mul_f(static_cast<float>(bz), sxd), DF{ab.z, ab.w});
    const DF d7 = df_mul(df_add(d5, d6), DF{FH, FL});
    int j1, k1;
    if (!df_floor(df_add(d5, d7), j1) || !df_floor(df_add(d6, d7), k1)) return false;
    const DF d8 = df_mul_f(static_cast<float>(j1 + k1), DF{GH, GL});
    const DF d11 = df_add(d5, df_add(DF{-static_cast<float>(j1), 0.0f}, d8));
    const DF d12 = df_add(d6, df_add(DF{-static_cast<float>(k1), 0.0f}, d8));
    const DF diff = df_add(d11, df_neg(d12));
    if (fabsf(diff.h) <= SIMPLEX_EPS) return false;
    const int b0 = diff.h > 0.0f ? 1 : 0;
    const int b1 = 1 - b0;
    const DF d13 = df_add(d11, b0 ? DF{G1H, G1L} : DF{GH, GL});
    const DF d14 = df_add(d12, b1 ? DF{G1H, G1L} : DF{GH, GL});
    const DF d15 = df_add(d11, DF{G2H, G2L});
    const DF d16 = df_add(d12, DF{G2H, G2L});
    const int l1 = j1 & 255;
    const int i2 = k1 & 255;
    const int g0 = P(s.p, l1 + P(s.p, i2)) % 12;
    const int g1 = P(s.p, l1 + b0 + P(s.p, i2 + b1)) % 12;
    const int g2 = P(s.p, l1 + 1 + P(s.p, i2 + 1)) % 12;
    float err = 0.0f;
    const float n0 = simplex_corner(d11.h + d11.l, d12.h + d12.l, g0, err, SIMPLEX_EPS);
    const float n1 = simplex_corner(d13.h + d13.l, d14.h + d14.l, g1, err, SIMPLEX_EPS);
    const float n2 = simplex_corner(d15.h + d15.l, d16.h + d16.l, g2, err, SIMPLEX_EPS);
    const float sum = n0 + n1 + n2;
    const float v = 70.0f * sum;
    out = Fe{v, 70.0f * (err + 2.0f * fabsf(sum) * U) + fabsf(v) * U};
    return true;
}

// Climate (temperature, rain) with bounds (WorldChunkManager173.java:95-126);
// clim[i] = climate_split of climate generator i.
__device__ __forceinline__ void climate_f(const GenTable& t, const float4* clim, int bx, int bz, Fe& temperature,
                                          Fe& rain) {
    const double X = static_cast<double>(bx);
    const double Z = static_cast<double>(bz);
    Fe raw[3];
    const int base[3] = {0, 4, 8};
    const int count[3] = {4, 4, 2};
    const double scale[3] = {0.02500000037252903, 0.05000000074505806, 0.25};
    const double octScale[3] = {0.25, 0.3333333333333333, 0.5882352941176471};
#pragma unroll
    for (int grp = 0; grp < 3; ++grp) {
        const double d2 = scale[grp] / 1.5;
        double d6 = 1.0;
        double d7 = 1.0;
        Fe acc{0.0f, 0.0f};
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            if (o < count[grp]) {
                const double sx = d2 * d7;
                const float w = static_cast<float>(0.55 / d6);  // 0.55 * 2^k: FP32 rounding of w tracked below
                const Gen g = t(ST_TEMP + base[grp] + o);
                Fe s;
                if (!simplex2f_df(g, clim[base[grp] + o], bx, bz, sx, s)) s = simplex2f(g, X * sx, Z * sx);
                const Fe term{s.v * w, s.e * w + fabsf(s.v * w) * 2.0f * U};
                acc = fe_add(acc, term);
                d7 *= octScale[grp];
                d6 *= 0.5;
            }
        }
        raw[grp] = acc;
    }
    // Decimal constants are not exact in FP32: each carries its own rounding bound.
    const Fe c11{1.1f, 1.1f * U}, c015{0.15f, 0.15f * U};
    const Fe d0 = fe_add(fe_mul(raw[2], c11), Fe{0.5f, 0.0f});
    Fe d3 = fe_add(fe_mul(fe_add(fe_mul(raw[0], c015), Fe{0.7f, 0.7f * U}), Fe{0.99f, 0.99f * U}),
                   fe_mul(d0, Fe{0.01f, 0.01f * U}));
    Fe d4 = fe_add(fe_mul(fe_add(fe_mul(raw[1], c015), Fe{0.5f, 0.0f}), Fe{0.998f, 0.998f * U}),
                   fe_mul(d0, Fe{0.002f, 0.002f * U}));
    const Fe om = fe_sub(Fe{1.0f, 0.0f}, d3);
    d3 = fe_sub(Fe{1.0f, 0.0f}, fe_mul(om, om));
    d3 = fe_clamp_hi(fe_clamp_lo(d3, 0.0f), 1.0f);
    d4 = fe_clamp_hi(fe_clamp_lo(d4, 0.0f), 1.0f);
    temperature = d3;
    rain = d4;
}

// d6 / d7 half of the column shape (BetaTerrain173.java:778-804) from noise5
// alone. zeroD5 reports the d6 < 0 branch, in which the reference sets d5 to 0
// before `d5 += 0.5`, so temperature, rain and noise4 cannot change the column
// there (about 70% of Stage0 columns). Returns false when the branch cannot be
// decided within the bound.
__device__ __forceinline__ bool shape_d7_f(Fe n5, Fe& d7out, bool& zeroD5) {
    Fe d6 = fe_div(n5, Fe{8000.0f, 0.0f});
    if (fabsf(d6.v) <= d6.e) {
        d6 = Fe{fabsf(d6.v), d6.e};  // -d6*0.3 and d6 agree at 0: Lipschitz 1
    } else if (d6.v < 0.0f) {
        d6 = fe_scale(Fe{-d6.v, d6.e}, 1.0f);
        d6 = fe_mul(d6, Fe{0.3f, 0.3f * U});
    }
    d6 = fe_sub(fe_scale(d6, 3.0f), Fe{2.0f, 0.0f});
    if (fabsf(d6.v) <= d6.e) return false;  // d5 = 0 branch undecidable
    zeroD5 = d6.v < 0.0f;
    if (zeroD5) {
        d6 = fe_scale(d6, 0.5f);
        d6 = fe_clamp_lo(d6, -1.0f);
        d6 = fe_div(d6, Fe{1.4f, 1.4f * U});
        d6 = fe_scale(d6, 0.5f);
    } else {
        d6 = fe_clamp_hi(d6, 1.0f);
        d6 = fe_scale(d6, 0.125f);
    }
    d6 = fe_scale(fe_scale(d6, 17.0f), 1.0f / 16.0f);
    d7out = fe_add(Fe{8.5f, 0.0f}, fe_scale(d6, 4.0f));
    return true;
}

// d5 of the d6 >= 0 branch (BetaTerrain173.java:753-777, 801-802): the climate
// and noise4 term, clamped to [0, 1], plus 0.5.
__device__ __forceinline__ Fe shape_d5_f(Fe temp, Fe rain, Fe n4) {
    const Fe d3 = fe_mul(rain, temp);
    Fe d4 = fe_sub(Fe{1.0f, 0.0f}, d3);
    d4 = fe_mul(d4, d4);
    d4 = fe_mul(d4, d4);
    d4 = fe_sub(Fe{1.0f, 0.0f}, d4);
    Fe d5 = fe_scale(fe_add(n4, Fe{256.0f, 0.0f}), 1.0f / 512.0f);
    d5 = fe_clamp_hi(fe_mul(d5, d4), 1.0f);
    d5 = fe_clamp_lo(d5, 0.0f);
    return fe_add(d5, Fe{0.5f, 0.0f});
}

// Whole column shape with bounds (BetaTerrain173.java:753-804); false when the
// d6 < 0 branch cannot be decided within the bound.
__device__ __forceinline__ bool column_shape_f(Fe temp, Fe rain, Fe n4, Fe n5, Fe& d5out, Fe& d7out) {
    bool zeroD5 = false;
    if (!shape_d7_f(n5, d7out, zeroD5)) return false;
    d5out = zeroD5 ? Fe{0.5f, 0.0f} : shape_d5_f(temp, rain, n4);
    return true;
}

// Level 16 of a 17-level column is air everywhere: the top fade of
// BetaTerrain173.java:808-830 has d13 = (float)(16 - 13) / 3.0F = 1.0 there, so
// the density is d8 * 0.0 + -10.0 * 1.0 = -10.0 for any finite d8 (d5 >= 0.5
// keeps d9, and so d8, finite). The screened kernels therefore evaluate levels
// up to 15 and leave bit 16 clear.
constexpr int TOP_SOLID_LEVEL = 15;

// A level's density test (BetaTerrain173.java:808-830) as two thresholds on d8.
// The density is T(d8 - d9), where d9 = (y - d7) * 12 / d5 (times 4 when
// negative) depends on the column shape alone and T is the top fade: the
// identity up to level 13, above it T(x) = x (1 - d13) - 10 d13 with
// d13 = (float)(y - 13) / 3F, increasing, zero at x = c_y = 10 d13 / (1 - d13)
// (5.00000022 at level 14, 20.0000018 at level 15; level 16 is air). So the
// density is positive when d8 - d9 > c_y and negative when below, and a test
// with bounds compares our FP32 d8 with d9 + c_y give or take a margin:
//   - d8's own error against the reference: at most E8MAX for d10 and d11
//     (the descending sum bound and the 1/512 scaling of |sum| <= 1.55 * 65535),
//     so for any blend of them, plus |d11 - d10| te for the selector's bound;
//   - d9's bound, the model terms doubled (as elsewhere in this file) plus an
//     absolute 1e-6 for the reference's own FP64 rounding of the blend, the
//     subtraction and T (below 1e-12 for these magnitudes);
//   - 8u (|d9| + 420) for the FP32 roundings of the test itself (the blend,
//     |d8| <= 199 and t |d11 - d10| <= 398; the thresholds; d8 -+ the rest
//     term), which together stay below u (2 |d9| + 1040);
//   - the unsummed octaves: rest / 512 on d8 (1 + 2^-10 for its own rounding),
//     not doubled, as it is an exact bound.
// The selector d12 = (n1/10 + 1)/2 picks d10 (noise2, sel bit 0) below 0, d11
// (noise3, bit 1) above 1, else the lerp d10 + (d11 - d10) d12; the test keeps
// t = d12 clamped to [0, 1] and its bound te (t = 0 or 1 and te = 0 when the
// selection is certain).
struct LevelTerms {
    float thrPos, thrNeg;  // d8 beyond these (with rest and blend margins) decides the sign
    float t, te;
    unsigned sel;
};
constexpr float E8MAX = (E_N2_DESC + OCTAVE3_ABS_MAX * 65535.0f * U) / 512.0f;

// d9 = (y - d7) * 12 / d5, times 4 when negative: the shape alone.
__device__ __forceinline__ Fe level_d9(int y, Fe d5, Fe d7) {
    Fe d9 = fe_div(fe_scale(fe_sub(Fe{static_cast<float>(y), 0.0f}, d7), 12.0f), d5);
    if (d9.v < 0.0f || fabsf(d9.v) <= d9.e) d9 = Fe{d9.v < 0.0f ? d9.v * 4.0f : d9.v, d9.e * 4.0f};
    return d9;
}
__device__ __forceinline__ void level_thresholds(int y, Fe d5, Fe d7, LevelTerms& lt) {
    const Fe d9 = level_d9(y, d5, d7);
    // nearest floats to c_14 and c_15 (errors 2.3e-7 and 1.2e-7, inside the margin)
    const float c = y <= 13 ? 0.0f : (y == 14 ? 5.0f : (y == 15 ? 20.000002f : INFINITY));
    const float margin = 2.0f * (d9.e + E8MAX) + 1.0e-6f + 8.0f * U * (fabsf(d9.v) + 420.0f);
    lt.thrPos = d9.v + c + margin;
    lt.thrNeg = d9.v + c - margin;
    lt.t = 0.0f;
    lt.te = 0.0f;
    lt.sel = 3u;
}
// The selector from the complete noise1 sum.
__device__ __forceinline__ void level_select(float n1, LevelTerms& lt) {
    const Fe d12 = fe_scale(fe_add(fe_div(Fe{n1, E_N1}, Fe{10.0f, 0.0f}), Fe{1.0f, 0.0f}), 0.5f);
    // below 0 only d10 is read, above 1 only d11; in between (or at a clamp
    // edge) the lerp with t clamped to [0, 1] covers both sides
    lt.sel = d12.v + d12.e < 0.0f ? 1u : (d12.v - d12.e > 1.0f ? 2u : 3u);
    lt.t = lt.sel == 1u ? 0.0f : (lt.sel == 2u ? 1.0f : fminf(fmaxf(d12.v, 0.0f), 1.0f));
    lt.te = lt.sel == 3u ? d12.e : 0.0f;
}

// Octave pairs the screened loops sum before noise1 at most (see progressive_signs).
#ifndef BSF_HULL_PAIRS
#define BSF_HULL_PAIRS 16
#endif
constexpr int HULL_PAIRS = BSF_HULL_PAIRS;

// Screened signs of one column's levels [y0, y0+n), n <= N. noise2 and noise3
// are summed from the largest octave (weight 2^15) down. Octave o contributes
// at most OCTAVE3_ABS_MAX * 2^o, so after octaves 15..o the unsummed rest is
// at most OCTAVE3_ABS_MAX * (2^o - 1), which the sign tests carry beside the
// sums' FP32 bounds. Three phases, each warp-uniform:
//   0. noise2 and noise3 octave o together, each level tested at both ends of
//      the hull of d10 and d11, which needs no noise1: d8 is d10, d11 or their
//      lerp with d12 in [0, 1], so it lies between them (the reference's FP64
//      lerp up to three roundings, below 2^-43 for |d8| < 512 and far inside
//      the bound's absolute 1e-6), and the density is non-decreasing in d8
//      (the top fade's slope 1 - d13 is >= 0), so a sign both ends share is
//      the density's sign. Most levels of the Stage0 and coarse tasks lie far
//      enough above or below the terrain surface to be decided here. The
//      phase ends when the warp's levels are all decided, when a level's ends
//      have opposite certain signs (only noise1 can decide it), or after
//      HULL_PAIRS pairs;
//   1. the 8 noise1 octaves (the reference's order, 0.0 + first term being
//      exact), then the selectors and a test at the depth reached;
//   2. the remaining octaves, skipping a sum that no open level of the
//      converged lanes reads (LevelTerms::sel), with a test after each pair.
// A level closed in any phase keeps its sign: a later interval may straddle 0
// again. The warp stops once all its lanes' levels are decided; an undecided
// level after octave 0 returns false (the exact FP64 path decides).
// oct(state, o, v) writes octave o of generator state `state`, weight 2^o, for
// N levels from y0 into v (a level past n costs its octave work but is never
// read). Every step goes through one loop body with one octave evaluation in
// it: the unrolled octave code is large, and a body holding several copies
// misses the instruction cache on every iteration. The 16 pairs and the 8
// noise1 octaves are 40 steps.
template <int N, typename OctFn>
__device__ __forceinline__ bool progressive_signs(int y0, int n, Fe d5, Fe d7, OctFn oct, unsigned& bits) {
    float a1[N], a2[N], a3[N];
    LevelTerms lt[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        a1[k] = a2[k] = a3[k] = 0.0f;  // a skipped sum is read by no open level
        level_thresholds(y0 + k, d5, d7, lt[k]);
    }
    unsigned open = (1u << n) - 1u, pos = 0;
    int phase = HULL_PAIRS > 0 ? 0 : 1, o = 15, i1 = 0, pairs = 0;
    bool third = false;
#pragma unroll 1
    for (int j = 0; j < 40; ++j) {
        bool run = true;
        if (phase == 2) {
            unsigned need = 0;
#pragma unroll
            for (int k = 0; k < N; ++k) need |= ((open >> k) & 1u) ? lt[k].sel : 0u;
            // Any superset of this lane's own need is correct, so the converged
            // lanes' union serves them all and keeps the octave loads warp-uniform.
            need = __reduce_or_sync(__activemask(), need);
            run = (need & (third ? 2u : 1u)) != 0;
        }
        if (run) {  // the one octave evaluation of the loop body
            float v[N];
            const bool n1 = phase == 1;
            oct(n1 ? ST_N1 + i1 : (third ? ST_N3 : ST_N2) + o, n1 ? i1 : o, v);
#pragma unroll
            for (int k = 0; k < N; ++k) {
                if (phase == 1) a1[k] = a1[k] + v[k];
                else if (third) a3[k] = a3[k] + v[k];
                else a2[k] = a2[k] + v[k];
            }
        }
        if (phase == 1) {
            if (++i1 < 8) continue;
#pragma unroll
            for (int k = 0; k < N; ++k) level_select(a1[k], lt[k]);
            phase = 2;
        } else {
            if (!third) {
                third = true;
                continue;
            }
            third = false;
            --o;
            ++pairs;
        }
        // both sums now hold octaves 15..o+1
        const float rest = OCTAVE3_ABS_MAX * static_cast<float>((1 << (o + 1)) - 1);
        const float rs = rest * (1.0f / 512.0f) * (1.0f + 1.0f / 1024.0f);
        const bool hull = phase == 0;
        bool conflict = false;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float d10 = a2[k] * (1.0f / 512.0f), d11 = a3[k] * (1.0f / 512.0f);
            const float diff = d11 - d10;
            const float d8 = __fmaf_rn(lt[k].t, diff, d10);
            const float em = 2.0f * fabsf(diff) * lt[k].te;
            // phase 0: the hull's ends; then the selected d8 with its blend bound
            const float lo = hull ? fminf(d10, d11) : d8 - em;
            const float hi = hull ? fmaxf(d10, d11) : d8 + em;
            const int sg = (lo - rs > lt[k].thrPos ? 1 : 0) - (hi + rs < lt[k].thrNeg ? 1 : 0);
            const bool was = (open >> k) & 1u;
            conflict |= hull && was && hi - rs > lt[k].thrPos && lo + rs < lt[k].thrNeg;
            pos |= (was && sg > 0) ? 1u << (y0 + k) : 0u;
            open &= sg != 0 ? ~(1u << k) : ~0u;
        }
        // The converged lanes leave together: a lane that ran ahead into its
        // next task would split the warp into two instruction streams.
        if (__all_sync(__activemask(), open == 0)) break;
        if (phase == 0) {
            if (o < 0 || pairs >= HULL_PAIRS || __any_sync(__activemask(), conflict)) phase = 1;
        } else if (o < 0) {
            break;
        }
    }
    if (open) return false;
    bits = pos;
    return true;
}


}  // namespace screen
}  // namespace bsf
