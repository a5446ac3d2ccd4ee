// Device-side exact arithmetic for the Beta 1.7.3 terrain path on sm_103a.
//
// Every FP64 expression keeps the operand order of the reference generator
// (src/beta173/noise/*.java, src/beta173/BetaTerrain173.java) and the library
// is compiled with --fmad=false, so no multiply-add is ever contracted and all
// results are bit-identical to Java's strict IEEE doubles.
#pragma once

#include <cstdint>

namespace bsf {

constexpr std::uint64_t LCG_MUL = 0x5DEECE66DULL;
constexpr std::uint64_t LCG_ADD = 0xBULL;
constexpr std::uint64_t LCG_MASK = (1ULL << 48) - 1ULL;

// Perlin/simplex generator index layout of one world's state cache.
// Terrain stream (Random(seed)): noise2 x16, noise3 x16, noise1 x8, [8 skipped],
// noise4 x10, noise5 x16 (BetaTerrain173.java:84-91); climate streams
// temperature x4 (seed*9871), rain x4 (seed*39811), blend x2 (seed*543321)
// (WorldChunkManager173.java:24-31).
constexpr int ST_N2 = 0;
constexpr int ST_N3 = 16;
constexpr int ST_N1 = 32;
constexpr int ST_N4 = 40;
constexpr int ST_N5 = 50;
constexpr int ST_TEMP = 66;
constexpr int ST_RAIN = 70;
constexpr int ST_BLEND = 74;
constexpr int ST_COUNT = 76;
constexpr int PERM_BYTES = 256;
constexpr int WORLD_PERM_BYTES = ST_COUNT * PERM_BYTES;  // 19,456
constexpr int WORLD_OFFSETS = ST_COUNT * 4;              // a, b, c, pad (doubles)

// Java Random draws per Perlin constructor with no nextInt rejection:
// 3 nextDouble (2 draws each) + 256 nextInt.
constexpr int DRAWS_PER_CONSTRUCTOR = 262;

// 3D octave groups of the density field and their scales (BetaTerrain173.java:667-742).
constexpr double NOISE_XZ = 684.412;
constexpr double NOISE_Y = 684.412;
constexpr int OCT3 = 40;  // 16 noise2 + 16 noise3 + 8 noise1

__device__ __forceinline__ std::uint64_t lcg_step(std::uint64_t s) {
    return (s * LCG_MUL + LCG_ADD) & LCG_MASK;
}

// Java `(int) v; if (v < (double) i) --i;` for |v| < 2^31.
__device__ __forceinline__ int jfloor(double v) {
    int i = __double2int_rz(v);
    return v < static_cast<double>(i) ? i - 1 : i;
}

// 2^-k for 0 <= k <= 1022, built from its bits. x * exp2_neg(k) equals the
// IEEE quotient x / 2^k exactly (both are the exact scaling while the result
// stays normal) without an FP64 division, which GB300's narrow FP64 pipe runs
// as a long iteration.
__device__ __forceinline__ double exp2_neg(int k) {
    return __longlong_as_double(static_cast<long long>(1023 - k) << 52);
}

__device__ __forceinline__ double fade(double v) {
    return v * v * v * (v * (v * 6.0 - 15.0) + 10.0);
}

__device__ __forceinline__ double lerp(double t, double a, double b) { return a + t * (b - a); }

// NoiseGeneratorPerlin173.a(int,double,double,double) (:132-151) as selects:
// u = x for h<8 else y; v = y for h<4, x for h in {12,14}, else z; signs from h&1, h&2.
__device__ __forceinline__ double grad3(int hash, double x, double y, double z) {
    const int h = hash & 15;
    const double u = h < 8 ? x : y;
    const double v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}

// NoiseGeneratorPerlin173.a(int,double,double) legacy 2D gradient (:112-130),
// including its signed-zero terms.
__device__ __forceinline__ double grad2_legacy(int hash, double x, double z) {
    const double zeroX = 0.0 * x;
    switch (hash & 15) {
        case 0: return x + 0.0;
        case 1: return -x + 0.0;
        case 2: return x + -0.0;
        case 3: return -x + -0.0;
        case 4: return x + z;
        case 5: return -x + z;
        case 6: return x + -z;
        case 7: return -x + -z;
        case 8: return zeroX + z;
        case 9: return -zeroX + z;
        case 10: return zeroX + -z;
        case 11: return -zeroX + -z;
        case 12: return zeroX + x;
        case 13: return -zeroX + z;
        case 14: return zeroX + -x;
        default: return -zeroX + -z;
    }
}

struct Gen {
    const std::uint8_t* p;  // 256-entry permutation (index & 255 == Java's 512-entry table)
    double a, b, c;
};

__device__ __forceinline__ int P(const std::uint8_t* p, int i) { return p[i & 255]; }

// One Y sample of a 3D octave: lattice index, fraction of the cell's first
// sample (the legacy corner cache uses it for the whole cell,
// NoiseGeneratorPerlin173.java:262-271), and this sample's own fade.
struct YEntry {
    double cellFrac;  // fraction at the first Y of this entry's cell
    double fade;      // fade(own fraction)
    int yi;           // floor & 255
    int cell;         // cell ordinal within the 17-sample column
};

// Y axis of one octave for y = 0..16: v = y*sy + b (fromY = 0).
__device__ __forceinline__ void build_yaxis(double sy, double b, YEntry* out) {
    int prev = -1;
    int cell = -1;
    double cellFrac = 0.0;
#pragma unroll 1
    for (int y = 0; y < 17; ++y) {
        double v = (0.0 + static_cast<double>(y)) * sy + b;
        const int f = jfloor(v);
        const int yi = f & 255;
        v -= static_cast<double>(f);
        if (y == 0 || yi != prev) {
            prev = yi;
            ++cell;
            cellFrac = v;
        }
        out[y].cellFrac = cellFrac;
        out[y].fade = fade(v);
        out[y].yi = yi;
        out[y].cell = cell;
    }
}

// X/Z lattice of one 3D octave column (x = xs + a, z = zs + c already scaled).
struct Lattice3 {
    double x, x1, xf, z, z1, zf;
    int zi, xp0, xp1;
};
__device__ __forceinline__ Lattice3 lattice3(const Gen& g, double xs, double zs) {
    Lattice3 L;
    double x = xs + g.a;
    const int fx = jfloor(x);
    const int xi = fx & 255;
    x -= static_cast<double>(fx);
    L.x = x;
    L.xf = fade(x);
    double z = zs + g.c;
    const int fz = jfloor(z);
    L.zi = fz & 255;
    z -= static_cast<double>(fz);
    L.z = z;
    L.zf = fade(z);
    L.x1 = x - 1.0;
    L.z1 = z - 1.0;
    L.xp0 = P(g.p, xi);
    L.xp1 = P(g.p, xi + 1);
    return L;
}

// Corner gradients of the Y cell of sample e, lerped along X.
__device__ __forceinline__ void cell_corners(const Gen& g, const Lattice3& L, const YEntry& e, double& c00,
                                             double& c01, double& c10, double& c11) {
    const double y = e.cellFrac;
    const double y1 = y - 1.0;
    const int p0 = L.xp0 + e.yi;
    const int p00 = P(g.p, p0) + L.zi;
    const int p01 = P(g.p, p0 + 1) + L.zi;
    const int p1 = L.xp1 + e.yi;
    const int p10 = P(g.p, p1) + L.zi;
    const int p11 = P(g.p, p1 + 1) + L.zi;
    c00 = lerp(L.xf, grad3(P(g.p, p00), L.x, y, L.z), grad3(P(g.p, p10), L.x1, y, L.z));
    c01 = lerp(L.xf, grad3(P(g.p, p01), L.x, y1, L.z), grad3(P(g.p, p11), L.x1, y1, L.z));
    c10 = lerp(L.xf, grad3(P(g.p, p00 + 1), L.x, y, L.z1), grad3(P(g.p, p10 + 1), L.x1, y, L.z1));
    c11 = lerp(L.xf, grad3(P(g.p, p01 + 1), L.x, y1, L.z1), grad3(P(g.p, p11 + 1), L.x1, y1, L.z1));
}

// weight * noise at sample e from its cell's corners.
__device__ __forceinline__ double cell_sample(const Lattice3& L, const YEntry& e, double c00, double c01, double c10,
                                              double c11, double weight) {
    const double r0 = lerp(e.fade, c00, c01);
    const double r1 = lerp(e.fade, c10, c11);
    return lerp(L.zf, r0, r1) * weight;
}

// Adds weight * noise for samples y in [Y0, Y0+N) of one 3D octave column
// (x = xs + a, z = zs + c already scaled), reusing corner gradients per Y cell.
template <int Y0, int N>
__device__ __forceinline__ void octave3_column(const Gen& g, double xs, double zs, const YEntry* ya,
                                               double weight, double* acc, bool first) {
    const Lattice3 L = lattice3(g, xs, zs);
    int activeCell = -1;
    double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const YEntry e = ya[Y0 + k];
        if (e.cell != activeCell) {
            activeCell = e.cell;
            cell_corners(g, L, e, c00, c01, c10, c11);
        }
        const double v = cell_sample(L, e, c00, c01, c10, c11, weight);
        acc[k] = first ? 0.0 + v : acc[k] + v;
    }
}

// Legacy 2D octave sample (NoiseGeneratorPerlin173.java:188-223): corner 0 uses
// the 2D gradient, the others the 3D one with y = 0.
__device__ __forceinline__ double octave2(const Gen& g, double xs, double zs) {
    double x = xs + g.a;
    const int fx = jfloor(x);
    const int xi = fx & 255;
    x -= static_cast<double>(fx);
    const double xf = fade(x);
    double z = zs + g.c;
    const int fz = jfloor(z);
    const int zi = fz & 255;
    z -= static_cast<double>(fz);
    const double zf = fade(z);
    const int a0 = P(g.p, xi) + 0;
    const int a1 = P(g.p, a0) + zi;
    const int b0 = P(g.p, xi + 1) + 0;
    const int b1 = P(g.p, b0) + zi;
    const double q0 = lerp(xf, grad2_legacy(P(g.p, a1), x, z), grad3(P(g.p, b1), x - 1.0, 0.0, z));
    const double q1 = lerp(xf, grad3(P(g.p, a1 + 1), x, 0.0, z - 1.0), grad3(P(g.p, b1 + 1), x - 1.0, 0.0, z - 1.0));
    return lerp(zf, q0, q1);
}

// NoiseGenerator2173 simplex gradient (:61-75).
__device__ __forceinline__ double simplex_grad(int g, double x, double z) {
    switch (g) {
        case 0: return 1.0 * x + 1.0 * z;
        case 1: return -1.0 * x + 1.0 * z;
        case 2: return 1.0 * x + -1.0 * z;
        case 3: return -1.0 * x + -1.0 * z;
        case 4:
        case 6: return 1.0 * x + 0.0 * z;
        case 5:
        case 7: return -1.0 * x + 0.0 * z;
        case 8:
        case 10: return 0.0 * x + 1.0 * z;
        default: return 0.0 * x + -1.0 * z;
    }
}

__device__ __forceinline__ int simplex_floor(double v) {
    return v > 0.0 ? __double2int_rz(v) : __double2int_rz(v) - 1;
}

// One simplex sample (NoiseGenerator2173.aStrided body, :111-174) without the
// octave weight: returns 70 * (n0 + n1 + n2).
__device__ __forceinline__ double simplex2(const Gen& s, double xs, double zs) {
    constexpr double F = 0.3660254037844386;   // 0.5 * (sqrt(3) - 1)
    constexpr double G = 0.21132486540518713;  // (3 - sqrt(3)) / 6
    const double d5 = xs + s.a;
    const double d6 = zs + s.b;
    const double d7 = (d5 + d6) * F;
    const int j1 = simplex_floor(d5 + d7);
    const int k1 = simplex_floor(d6 + d7);
    const double d8 = static_cast<double>(j1 + k1) * G;
    const double d9 = static_cast<double>(j1) - d8;
    const double d10 = static_cast<double>(k1) - d8;
    const double d11 = d5 - d9;
    const double d12 = d6 - d10;
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
    double t0 = 0.5 - d11 * d11 - d12 * d12;
    double n0;
    if (t0 < 0.0) n0 = 0.0;
    else { t0 *= t0; n0 = t0 * t0 * simplex_grad(g0, d11, d12); }
    double t1 = 0.5 - d13 * d13 - d14 * d14;
    double n1;
    if (t1 < 0.0) n1 = 0.0;
    else { t1 *= t1; n1 = t1 * t1 * simplex_grad(g1, d13, d14); }
    double t2 = 0.5 - d15 * d15 - d16 * d16;
    double n2;
    if (t2 < 0.0) n2 = 0.0;
    else { t2 *= t2; n2 = t2 * t2 * simplex_grad(g2, d15, d16); }
    return 70.0 * (n0 + n1 + n2);
}

// Generators staged in shared memory: permutations [idx][256] and offsets
// [idx][3] (a, b, c); Gen views are built on demand to keep registers free.
struct GenTable {
    const std::uint8_t* perm;
    const double* off;
    __device__ __forceinline__ Gen operator()(int idx) const {
        Gen g;
        g.p = perm + idx * 256;
        g.a = off[idx * 3 + 0];
        g.b = off[idx * 3 + 1];
        g.c = off[idx * 3 + 2];
        return g;
    }
};

__device__ __forceinline__ void climate_combine(const double* raw, double& temperature, double& rain);

// Climate at integer block (bx, bz) after normalisation
// (NoiseGeneratorOctaves2173.java:66-104 octave loop;
// WorldChunkManager173.java:95-126 formula). The climate generators sit at
// table indices 66..75 (temperature 4, rain 4, blend 2).
__device__ __forceinline__ void climate_at(const GenTable& t, int bx, int bz, double& temperature,
                                           double& rain) {
    const double X = static_cast<double>(bx);
    const double Z = static_cast<double>(bz);
    double raw[3];
    const int base[3] = {0, 4, 8};
    const int count[3] = {4, 4, 2};
    const double scale[3] = {0.02500000037252903, 0.05000000074505806, 0.25};
    const double octScale[3] = {0.25, 0.3333333333333333, 0.5882352941176471};
#pragma unroll
    for (int grp = 0; grp < 3; ++grp) {
        const double d2 = scale[grp] / 1.5;
        double d6 = 1.0;
        double d7 = 1.0;
        double acc = 0.0;
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            if (o < count[grp]) {
                const double sx = d2 * d7;
                const double w = 0.55 / d6;
                acc += simplex2(t(ST_TEMP + base[grp] + o), X * sx, Z * sx) * w;
                d7 *= octScale[grp];
                d6 *= 0.5;
            }
        }
        raw[grp] = acc;
    }
    climate_combine(raw, temperature, rain);
}

// Temperature and rain from the three raw octave sums (WorldChunkManager173.java:95-126).
__device__ __forceinline__ void climate_combine(const double* raw, double& temperature, double& rain) {
    const double d0 = raw[2] * 1.1 + 0.5;
    double d1 = 0.01;
    double d2 = 1.0 - d1;
    double d3 = (raw[0] * 0.15 + 0.7) * d2 + d0 * d1;
    d1 = 0.0020;
    d2 = 1.0 - d1;
    double d4 = (raw[1] * 0.15 + 0.5) * d2 + d0 * d1;
    d3 = 1.0 - (1.0 - d3) * (1.0 - d3);
    if (d3 < 0.0) d3 = 0.0;
    if (d4 < 0.0) d4 = 0.0;
    if (d3 > 1.0) d3 = 1.0;
    if (d4 > 1.0) d4 = 1.0;
    temperature = d3;
    rain = d4;
}

// Column shape terms d5 (height scale) and d7 (height centre) of
// generateTerrainNoise (BetaTerrain173.java:753-804) for yLen = 17.
__device__ __forceinline__ void column_shape(double temperature, double rain, double n4, double n5,
                                             double& outD5, double& outD7) {
    const double d2 = temperature;
    const double d3 = rain * d2;
    double d4 = 1.0 - d3;
    d4 *= d4;
    d4 *= d4;
    d4 = 1.0 - d4;
    double d5 = (n4 + 256.0) / 512.0;
    d5 *= d4;
    if (d5 > 1.0) d5 = 1.0;
    double d6 = n5 / 8000.0;
    if (d6 < 0.0) d6 = -d6 * 0.3;
    d6 = d6 * 3.0 - 2.0;
    if (d6 < 0.0) {
        d6 /= 2.0;
        if (d6 < -1.0) d6 = -1.0;
        d6 /= 1.4;
        d6 /= 2.0;
        d5 = 0.0;
    } else {
        if (d6 > 1.0) d6 = 1.0;
        d6 /= 8.0;
    }
    if (d5 < 0.0) d5 = 0.0;
    d5 += 0.5;
    d6 = d6 * 17.0 / 16.0;
    outD5 = d5;
    outD7 = 17.0 / 2.0 + d6 * 4.0;
}

// noise4 (10 octaves) and noise5 (16 octaves) of lattice column (X, Z), the
// reference's 2D octave sums (BetaTerrain173.java:731-737) in its order.
__device__ __forceinline__ void noise45(const GenTable& t, double X, double Z, double& n4, double& n5) {
    double amp = 1.0;
    double acc = 0.0;
    for (int o = 0; o < 10; ++o) {
        const double sc = 1.121 * amp;
        const double v = octave2(t(ST_N4 + o), X * sc, Z * sc) * (1.0 / amp);
        acc = o == 0 ? 0.0 + v : acc + v;
        amp /= 2.0;
    }
    n4 = acc;
    amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double sc = 200.0 * amp;
        const double v = octave2(t(ST_N5 + o), X * sc, Z * sc) * (1.0 / amp);
        acc = o == 0 ? 0.0 + v : acc + v;
        amp /= 2.0;
    }
    n5 = acc;
}

// Density at lattice level y (BetaTerrain173.java:808-830), yLen = 17.
__device__ __forceinline__ double density_at(int y, double d5, double d7, double n1, double n2, double n3) {
    double d9 = (static_cast<double>(y) - d7) * 12.0 / d5;
    if (d9 < 0.0) d9 *= 4.0;
    const double d10 = n2 / 512.0;
    const double d11 = n3 / 512.0;
    const double d12 = (n1 / 10.0 + 1.0) / 2.0;
    double d8;
    if (d12 < 0.0) d8 = d10;
    else if (d12 > 1.0) d8 = d11;
    else d8 = d10 + (d11 - d10) * d12;
    d8 -= d9;
    if (y > 13) {
        const double d13 = static_cast<double>(static_cast<float>(y - 13) / 3.0F);
        d8 = d8 * (1.0 - d13) + -10.0 * d13;
    }
    return d8;
}

}  // namespace bsf
