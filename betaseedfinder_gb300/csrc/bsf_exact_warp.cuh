// Exact FP64 column evaluated by one warp, for the screened kernels' fallbacks.
//
// A screened column task that its error bound cannot decide is recomputed in
// FP64. Done by one thread, that is ~40 dependent 3D octaves plus the shape:
// hundreds of microseconds on GB300's FP64 pipe, while the rest of the CTA
// waits at the next barrier. Every octave term, though, is independent of the
// others: here each lane computes one or two of them (the 36 shape terms, then
// the 40 3D octave columns), and the terms are added with warp shuffles in the
// reference's order (acc = 0.0 + t0, then acc + t1, ...), so every sum, and so
// every bit, is that of the serial loop (BetaTerrain173.java:739-831,
// NoiseGeneratorOctaves173.java, NoiseGeneratorOctaves2173.java:66-104).
//
// S is the kernel's shared-memory layout; it provides perm and off (the world's
// generators). The FP64 Y axis of each octave is rebuilt here with the same
// build_yaxis call the kernels' staging uses, so it is the same bit for bit.
#pragma once

#include "bsf_device.cuh"

namespace bsf {
namespace exactwarp {

__device__ __forceinline__ double lane_value(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// The reference's octave accumulation over lanes [first, first + count).
__device__ __forceinline__ double ordered_sum(double v, int first, int count) {
    double acc = 0.0 + lane_value(v, first);
#pragma unroll 1
    for (int o = 1; o < count; ++o) acc = acc + lane_value(v, first + o);
    return acc;
}

// Shape term i of the column: 0..9 the climate simplex octaves (temperature 4,
// rain 4, blend 2, each with its weight), 10..19 noise4, 20..35 noise5. Out of
// line, like the steps below, to keep the rarely run fallback code small.
static __device__ __noinline__ double shape_term(const GenTable& t, int i, double X, double Z, double BX, double BZ) {
    if (i < 10) {
        const int grp = i < 4 ? 0 : (i < 8 ? 1 : 2);
        const int o = i - (grp == 0 ? 0 : (grp == 1 ? 4 : 8));
        const double scale = grp == 0 ? 0.02500000037252903 : (grp == 1 ? 0.05000000074505806 : 0.25);
        const double octScale = grp == 0 ? 0.25 : (grp == 1 ? 0.3333333333333333 : 0.5882352941176471);
        const double d2 = scale / 1.5;
        double d6 = 1.0, d7 = 1.0;
        for (int q = 0; q < o; ++q) {  // the serial loop's running products
            d7 *= octScale;
            d6 *= 0.5;
        }
        const double sx = d2 * d7;
        const double w = 0.55 / d6;
        return simplex2(t(ST_TEMP + i), BX * sx, BZ * sx) * w;
    }
    const bool n4 = i < 20;
    const int o = n4 ? i - 10 : i - 20;
    const double amp = exp2_neg(o);  // exact, as amp /= 2.0 per octave
    const double sc = (n4 ? 1.121 : 200.0) * amp;
    return octave2(t((n4 ? ST_N4 : ST_N5) + o), X * sc, Z * sc) * static_cast<double>(1 << o);  // 1 / amp
}

// FP64 Y axis of 3D octave state (0..39): the legacy per-cell Y entries of
// its 17 levels (noise2/3: y scale 684.412 / 2^k; noise1: 684.412 / 160 / 2^k).
template <typename S>
__device__ __forceinline__ void y_entries(const S& s, int state, YEntry* ya) {
    const int k = state < 16 ? state : (state < 32 ? state - 16 : state - 32);
    const double amp = exp2_neg(k);
    const double sy = state < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
    build_yaxis(sy, s.off[state][1], ya);
}

// Most levels one column task covers (the screened kernels' ranges have 4 to 6).
constexpr int MAX_LEVELS = 6;

// One 3D octave column's terms for levels [y0, y0+n): octave3_column's
// arithmetic with the sums left out, in a rolled loop over the levels.
template <typename S>
__device__ __forceinline__ void octave_terms(const S& s, const GenTable& t, int state, double sc0, int o, double X,
                                             double Z, int y0, int n, double* out) {
    const double amp = exp2_neg(o);
    const double sc = sc0 * amp;
    YEntry ya[17];
    y_entries(s, state, ya);
    const Gen g = t(state);
    const Lattice3 L = lattice3(g, X * sc, Z * sc);
    const double weight = static_cast<double>(1 << o);  // 1 / amp, exact
    int activeCell = -1;
    double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        const YEntry e = ya[y0 + k];
        if (e.cell != activeCell) {
            activeCell = e.cell;
            cell_corners(g, L, e, c00, c01, c10, c11);
        }
        out[k] = 0.0 + cell_sample(L, e, c00, c01, c10, c11, weight);  // the first-octave form, same sum
    }
}

// Exact density signs of the column at coarse (cx, cz) for levels [y0, y0+n),
// n <= MAX_LEVELS, climate sampled at block (4cx+2, 4cz+2). All 32 lanes must
// call it with the same arguments; every lane returns the same bits. The levels
// are runtime values and every loop has one call site: the path is rare, and
// unrolled or instantiated per level range its FP64 code (hundreds of KB)
// streamed through the instruction cache on each call.
// The fallback path's shape and density steps out of line (code size: the path
// runs rarely, each time from a cold instruction cache).
static __device__ __noinline__ void shape_of(double temperature, double rain, double n4, double n5, double& d5, double& d7) {
    column_shape(temperature, rain, n4, n5, d5, d7);
}
static __device__ __noinline__ double density_of(int y, double d5, double d7, double n1, double n2, double n3) {
    return density_at(y, d5, d7, n1, n2, n3);
}

template <typename S>
__device__ unsigned exact_column_warp(const S& s, int cx, int cz, int y0, int n) {
    const int lane = threadIdx.x & 31;
    GenTable t;
    t.perm = s.perm;
    t.off = &s.off[0][0];
    const double X = static_cast<double>(cx), Z = static_cast<double>(cz);
    const double BX = static_cast<double>(cx * 4 + 2), BZ = static_cast<double>(cz * 4 + 2);
    // shape: 36 terms over two rounds of lanes
    double s0 = 0.0, s1 = 0.0;
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
        const int i = r * 32 + lane;
        const double v = i < 36 ? shape_term(t, i, X, Z, BX, BZ) : 0.0;
        if (r == 0) s0 = v;
        else s1 = v;
    }
    double raw[3];
    raw[0] = ordered_sum(s0, 0, 4);
    raw[1] = ordered_sum(s0, 4, 4);
    raw[2] = ordered_sum(s0, 8, 2);
    const double n4 = ordered_sum(s0, 10, 10);
    double n5 = 0.0 + lane_value(s0, 20);
    for (int q = 21; q < 32; ++q) n5 = n5 + lane_value(s0, q);
    for (int q = 0; q < 4; ++q) n5 = n5 + lane_value(s1, q);
    double temperature, rain;
    climate_combine(raw, temperature, rain);
    double d5, d7;
    shape_of(temperature, rain, n4, n5, d5, d7);
    // 3D octaves: lanes 0-15 noise2, 16-31 noise3, then lanes 0-7 noise1
    double tA[MAX_LEVELS], tB[MAX_LEVELS];
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
        double* out = r == 0 ? tA : tB;
        const int st = r == 0 ? (lane < 16 ? ST_N2 + lane : ST_N3 + lane - 16) : ST_N1 + lane;
        if (r == 0 || lane < 8) {
            octave_terms(s, t, st, r == 0 ? NOISE_XZ : NOISE_XZ / 80.0, r == 0 ? (lane & 15) : lane, X, Z, y0, n, out);
        } else {
            for (int k = 0; k < n; ++k) out[k] = 0.0;
        }
    }
    unsigned bits = 0;
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        const double n2 = ordered_sum(tA[k], 0, 16);
        const double n3 = ordered_sum(tA[k], 16, 16);
        const double n1 = ordered_sum(tB[k], 0, 8);
        if (density_of(y0 + k, d5, d7, n1, n2, n3) > 0.0) bits |= 1u << (y0 + k);
    }
    return bits;
}

}  // namespace exactwarp
}  // namespace bsf
