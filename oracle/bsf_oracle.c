/*
 * CPU oracle (test infrastructure only; see bsf_oracle.h).
 *
 * A restatement of the reference's Java Beta 1.7.3 generator
 * (the Java sources under src/beta173) and of the native worker stage semantics
 * (native/src headers, gpu_p20_benchmark.cpp). Expression order follows the
 * Java sources so that every FP64 result is bit-identical under strict
 * IEEE evaluation (compile with -ffp-contract=off).
 */
#include "bsf_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../betaseedfinder_gb300/csrc/p19_table.inc"

/* ========================================================================== */
/* java.util.Random: JDK Random.setSeed/next/nextDouble/nextInt (restated from
 * the JDK specification; the reference's C++ copy is p20_exact_math.hpp:19-52). */
#define OR_MULT 0x5DEECE66DULL
#define OR_ADD 0xBULL
#define OR_MASK ((1ULL << 48) - 1ULL)

void or_rand_set_seed(or_rand* r, int64_t seed) { r->s = ((uint64_t)seed ^ OR_MULT) & OR_MASK; }

int32_t or_rand_next(or_rand* r, int bits) {
    r->s = (r->s * OR_MULT + OR_ADD) & OR_MASK;
    return (int32_t)(uint32_t)(r->s >> (48 - bits));
}

double or_rand_next_double(or_rand* r) {
    int64_t hi = (int64_t)or_rand_next(r, 26);
    int64_t lo = (int64_t)or_rand_next(r, 27);
    return (double)((hi << 27) + lo) * 0x1.0p-53;
}

int32_t or_rand_next_int(or_rand* r, int32_t bound) {
    int32_t rr = or_rand_next(r, 31);
    int32_t m = bound - 1;
    if ((bound & m) == 0) return (int32_t)(((int64_t)bound * (int64_t)rr) >> 31);
    for (int32_t u = rr; (int32_t)((uint32_t)u - (uint32_t)(rr = u % bound) + (uint32_t)m) < 0;
         u = or_rand_next(r, 31)) {
    }
    return rr;
}

/* NoiseGeneratorPerlin173.reseed (noise/NoiseGeneratorPerlin173.java:63-77);
 * NoiseGenerator2173.reseed is the same sequence (noise/NoiseGenerator2173.java:27-48). */
void or_perlin_init(or_perlin* g, or_rand* r) {
    g->a = or_rand_next_double(r) * 256.0;
    g->b = or_rand_next_double(r) * 256.0;
    g->c = or_rand_next_double(r) * 256.0;
    for (int i = 0; i < 256; ++i) g->p[i] = i;
    for (int i = 0; i < 256; ++i) {
        int j = or_rand_next_int(r, 256 - i) + i;
        int t = g->p[i];
        g->p[i] = g->p[j];
        g->p[j] = t;
        g->p[i + 256] = g->p[i];
    }
}

/* NoiseGeneratorPerlin173.consumeConstructorRandom (:80-87). */
void or_perlin_consume(or_rand* r) {
    or_rand_next_double(r);
    or_rand_next_double(r);
    or_rand_next_double(r);
    for (int i = 0; i < 256; ++i) or_rand_next_int(r, 256 - i);
}

/* BetaTerrain173 constructor order (BetaTerrain173.java:77-93) and
 * WorldChunkManager173 climate generators (WorldChunkManager173.java:24-31). */
void or_world_init(or_world* w, int64_t seed) {
    or_rand r;
    or_rand_set_seed(&r, (int64_t)((uint64_t)seed * 9871ULL));
    for (int i = 0; i < 4; ++i) or_perlin_init(&w->temp[i], &r);
    or_rand_set_seed(&r, (int64_t)((uint64_t)seed * 39811ULL));
    for (int i = 0; i < 4; ++i) or_perlin_init(&w->rain[i], &r);
    or_rand_set_seed(&r, (int64_t)((uint64_t)seed * 543321ULL));
    for (int i = 0; i < 2; ++i) or_perlin_init(&w->blend[i], &r);

    or_rand_set_seed(&r, seed);
    for (int i = 0; i < 16; ++i) or_perlin_init(&w->n2[i], &r);
    for (int i = 0; i < 16; ++i) or_perlin_init(&w->n3[i], &r);
    for (int i = 0; i < 8; ++i) or_perlin_init(&w->n1[i], &r);
    for (int i = 0; i < 8; ++i) or_perlin_consume(&r);
    for (int i = 0; i < 10; ++i) or_perlin_init(&w->n4[i], &r);
    for (int i = 0; i < 16; ++i) or_perlin_init(&w->n5[i], &r);
}

static const or_perlin* world_state(const or_world* w, int index) {
    if (index < 16) return &w->n2[index];
    if (index < 32) return &w->n3[index - 16];
    if (index < 40) return &w->n1[index - 32];
    if (index < 50) return &w->n4[index - 40];
    if (index < 66) return &w->n5[index - 50];
    if (index < 70) return &w->temp[index - 66];
    if (index < 74) return &w->rain[index - 70];
    if (index < 76) return &w->blend[index - 74];
    return 0;
}

int or_world_state(int64_t seed, int index, uint8_t* perm256, double* abc3) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    if (!w) return -1;
    or_world_init(w, seed);
    const or_perlin* g = world_state(w, index);
    if (!g) { free(w); return -1; }
    for (int i = 0; i < 256; ++i) perm256[i] = (uint8_t)g->p[i];
    abc3[0] = g->a; abc3[1] = g->b; abc3[2] = g->c;
    free(w);
    return 0;
}

/* ========================================================================== */
/* Perlin gradients: NoiseGeneratorPerlin173.a(int,double,double,double) (:132-151)
 * and the 2D legacy a(int,double,double) (:112-130). */
static double grad3(int h, double x, double y, double z) {
    switch (h & 15) {
        case 0: return x + y;
        case 1: return -x + y;
        case 2: return x + -y;
        case 3: return -x + -y;
        case 4: return x + z;
        case 5: return -x + z;
        case 6: return x + -z;
        case 7: return -x + -z;
        case 8: return y + z;
        case 9: return -y + z;
        case 10: return y + -z;
        case 11: return -y + -z;
        case 12: return y + x;
        case 13: return -y + z;
        case 14: return y + -x;
        default: return -y + -z;
    }
}

static double grad2_legacy(int h, double x, double z) {
    double zeroX = 0.0 * x;
    switch (h & 15) {
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

static inline double lerp(double t, double a, double b) { return a + t * (b - a); }
static inline double fade(double v) { return v * v * v * (v * (v * 6.0 - 15.0) + 10.0); }
/* Java `(int) v; if (v < (double) i) --i;` for |v| < 2^31. */
static inline int jfloor(double v) {
    int i = (int)v;
    if (v < (double)i) --i;
    return i;
}

/* NoiseGeneratorPerlin173.a(double[],...) legacy exact method (:172-285),
 * extended with an integer sample stride on X/Z the way
 * addNoiseCachedAxesStrided (:386-480) extends it (step 1 = legacy call). */
void or_perlin_add(const or_perlin* g, double* out, double fromX, double fromY, double fromZ,
                   int xLen, int yLen, int zLen, double stepX, double stepZ,
                   double sx, double sy, double sz, double amplitude) {
    const int* d = g->p;
    if (yLen == 1) {
        double w = 1.0 / amplitude;
        int k = 0;
        for (int ix = 0; ix < xLen; ++ix) {
            double x = (fromX + (double)ix * stepX) * sx + g->a;
            int fx = jfloor(x);
            int xi = fx & 255;
            x -= (double)fx;
            double xf = x * x * x * (x * (x * 6.0 - 15.0) + 10.0);
            for (int iz = 0; iz < zLen; ++iz) {
                double z = (fromZ + (double)iz * stepZ) * sz + g->c;
                int fz = jfloor(z);
                int zi = fz & 255;
                z -= (double)fz;
                double zf = z * z * z * (z * (z * 6.0 - 15.0) + 10.0);
                int a0 = d[xi] + 0;
                int a1 = d[a0] + zi;
                int b0 = d[xi + 1] + 0;
                int b1 = d[b0] + zi;
                double q0 = lerp(xf, grad2_legacy(d[a1], x, z), grad3(d[b1], x - 1.0, 0.0, z));
                double q1 = lerp(xf, grad3(d[a1 + 1], x, 0.0, z - 1.0), grad3(d[b1 + 1], x - 1.0, 0.0, z - 1.0));
                double v = lerp(zf, q0, q1);
                out[k++] += v * w;
            }
        }
        return;
    }
    double w = 1.0 / amplitude;
    int k = 0;
    int prev = -1;
    double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
    for (int ix = 0; ix < xLen; ++ix) {
        double x = (fromX + (double)ix * stepX) * sx + g->a;
        int fx = jfloor(x);
        int xi = fx & 255;
        x -= (double)fx;
        double xf = x * x * x * (x * (x * 6.0 - 15.0) + 10.0);
        for (int iz = 0; iz < zLen; ++iz) {
            double z = (fromZ + (double)iz * stepZ) * sz + g->c;
            int fz = jfloor(z);
            int zi = fz & 255;
            z -= (double)fz;
            double zf = z * z * z * (z * (z * 6.0 - 15.0) + 10.0);
            for (int iy = 0; iy < yLen; ++iy) {
                double y = (fromY + (double)iy) * sy + g->b;
                int fy = jfloor(y);
                int yi = fy & 255;
                y -= (double)fy;
                double yf = y * y * y * (y * (y * 6.0 - 15.0) + 10.0);
                if (iy == 0 || yi != prev) {
                    prev = yi;
                    int p0 = d[xi] + yi;
                    int p00 = d[p0] + zi;
                    int p01 = d[p0 + 1] + zi;
                    int p1 = d[xi + 1] + yi;
                    int p10 = d[p1] + zi;
                    int p11 = d[p1 + 1] + zi;
                    c00 = lerp(xf, grad3(d[p00], x, y, z), grad3(d[p10], x - 1.0, y, z));
                    c01 = lerp(xf, grad3(d[p01], x, y - 1.0, z), grad3(d[p11], x - 1.0, y - 1.0, z));
                    c10 = lerp(xf, grad3(d[p00 + 1], x, y, z - 1.0), grad3(d[p10 + 1], x - 1.0, y, z - 1.0));
                    c11 = lerp(xf, grad3(d[p01 + 1], x, y - 1.0, z - 1.0), grad3(d[p11 + 1], x - 1.0, y - 1.0, z - 1.0));
                }
                double r0 = lerp(yf, c00, c01);
                double r1 = lerp(yf, c10, c11);
                double v = lerp(zf, r0, r1);
                out[k++] += v * w;
            }
        }
    }
}

/* One 17-level column of one octave with the legacy Y-cell corner cache,
 * emitting only y >= yLo: when the first emitted y sits inside a cell that
 * started lower, the corners are taken from that cell's first y, exactly as
 * the full legacy loop would (NoiseGeneratorPerlin173.java:262-271; masked
 * variant semantics at :486-491). out[y] += value * (1/amplitude). */
static void perlin_column17(const or_perlin* g, double xs, double sy, double zs, int yLo,
                            double amplitude, double* out) {
    const int* d = g->p;
    double w = 1.0 / amplitude;
    double x = xs + g->a;
    int fx = jfloor(x);
    int xi = fx & 255;
    x -= (double)fx;
    double xf = fade(x);
    double z = zs + g->c;
    int fz = jfloor(z);
    int zi = fz & 255;
    z -= (double)fz;
    double zf = fade(z);
    int prev = -1;
    int cellIndex = -1;
    double cellY = 0.0;
    double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
    int computedCell = -2;
    for (int iy = 0; iy < 17; ++iy) {
        double y = (0.0 + (double)iy) * sy + g->b;
        int fy = jfloor(y);
        int yi = fy & 255;
        y -= (double)fy;
        if (iy == 0 || yi != prev) {
            prev = yi;
            ++cellIndex;
            cellY = y;
        }
        if (iy < yLo) continue;
        if (computedCell != cellIndex) {
            computedCell = cellIndex;
            double yc = cellY;
            int p0 = d[xi] + yi;
            int p00 = d[p0] + zi;
            int p01 = d[p0 + 1] + zi;
            int p1 = d[xi + 1] + yi;
            int p10 = d[p1] + zi;
            int p11 = d[p1 + 1] + zi;
            c00 = lerp(xf, grad3(d[p00], x, yc, z), grad3(d[p10], x - 1.0, yc, z));
            c01 = lerp(xf, grad3(d[p01], x, yc - 1.0, z), grad3(d[p11], x - 1.0, yc - 1.0, z));
            c10 = lerp(xf, grad3(d[p00 + 1], x, yc, z - 1.0), grad3(d[p10 + 1], x - 1.0, yc, z - 1.0));
            c11 = lerp(xf, grad3(d[p01 + 1], x, yc - 1.0, z - 1.0), grad3(d[p11 + 1], x - 1.0, yc - 1.0, z - 1.0));
        }
        double yfd = fade(y);
        double r0 = lerp(yfd, c00, c01);
        double r1 = lerp(yfd, c10, c11);
        double v = lerp(zf, r0, r1);
        out[iy] += v * w;
    }
}

void or_perlin_column17_test(const uint8_t* perm256, const double* abc, double xs, double sy, double zs,
                             int yLo, double* out17) {
    or_perlin g;
    for (int i = 0; i < 256; ++i) { g.p[i] = perm256[i]; g.p[i + 256] = perm256[i]; }
    g.a = abc[0]; g.b = abc[1]; g.c = abc[2];
    for (int y = 0; y < 17; ++y) out17[y] = 0.0;
    perlin_column17(&g, xs, sy, zs, yLo, 1.0, out17);
}

double or_perlin3_point(const or_perlin* g, double xs, double ys, double zs) {
    /* NoiseGeneratorPerlin173.a(double,double,double) (:89-110): a fresh cell. */
    const int* d = g->p;
    double x = xs + g->a, y = ys + g->b, z = zs + g->c;
    int fx = jfloor(x), fy = jfloor(y), fz = jfloor(z);
    int xi = fx & 255, yi = fy & 255, zi = fz & 255;
    x -= (double)fx; y -= (double)fy; z -= (double)fz;
    double xf = fade(x), yf = fade(y), zf = fade(z);
    int p0 = d[xi] + yi, p00 = d[p0] + zi, p01 = d[p0 + 1] + zi;
    int p1 = d[xi + 1] + yi, p10 = d[p1] + zi, p11 = d[p1 + 1] + zi;
    double c00 = lerp(xf, grad3(d[p00], x, y, z), grad3(d[p10], x - 1.0, y, z));
    double c01 = lerp(xf, grad3(d[p01], x, y - 1.0, z), grad3(d[p11], x - 1.0, y - 1.0, z));
    double c10 = lerp(xf, grad3(d[p00 + 1], x, y, z - 1.0), grad3(d[p10 + 1], x - 1.0, y, z - 1.0));
    double c11 = lerp(xf, grad3(d[p01 + 1], x, y - 1.0, z - 1.0), grad3(d[p11 + 1], x - 1.0, y - 1.0, z - 1.0));
    return lerp(zf, lerp(yf, c00, c01), lerp(yf, c10, c11));
}

double or_perlin2_point(const or_perlin* g, double xs, double zs) {
    double out = 0.0;
    or_perlin_add(g, &out, xs, 10.0, zs, 1, 1, 1, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0);
    return out;
}

/* NoiseGenerator2173.aStrided (noise/NoiseGenerator2173.java:86-176). */
static const double SIMPLEX_F = 0.3660254037844386;  /* 0.5 * (sqrt(3) - 1) */
static const double SIMPLEX_G = 0.21132486540518713; /* (3 - sqrt(3)) / 6 */

static inline int simplex_floor(double v) { return v > 0.0 ? (int)v : (int)v - 1; }

static double simplex_grad(int g, double x, double z) {
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

void or_simplex_add(const or_perlin* g, double* out, double x0, double z0, int xLen, int zLen,
                    int strideX, int strideZ, double sx, double sz, double weight) {
    const int* e = g->p;
    int k = 0;
    for (int l = 0; l < xLen; ++l) {
        double d5 = (x0 + (double)(l * strideX)) * sx + g->a;
        for (int i1 = 0; i1 < zLen; ++i1) {
            double d6 = (z0 + (double)(i1 * strideZ)) * sz + g->b;
            double d7 = (d5 + d6) * SIMPLEX_F;
            int j1 = simplex_floor(d5 + d7);
            int k1 = simplex_floor(d6 + d7);
            double d8 = (double)(j1 + k1) * SIMPLEX_G;
            double d9 = (double)j1 - d8;
            double d10 = (double)k1 - d8;
            double d11 = d5 - d9;
            double d12 = d6 - d10;
            int b0, b1;
            if (d11 > d12) { b0 = 1; b1 = 0; } else { b0 = 0; b1 = 1; }
            double d13 = d11 - (double)b0 + SIMPLEX_G;
            double d14 = d12 - (double)b1 + SIMPLEX_G;
            double d15 = d11 - 1.0 + 2.0 * SIMPLEX_G;
            double d16 = d12 - 1.0 + 2.0 * SIMPLEX_G;
            int l1 = j1 & 255;
            int i2 = k1 & 255;
            int j2 = e[l1 + e[i2]] % 12;
            int k2 = e[l1 + b0 + e[i2 + b1]] % 12;
            int l2 = e[l1 + 1 + e[i2 + 1]] % 12;
            double d17 = 0.5 - d11 * d11 - d12 * d12;
            double d18;
            if (d17 < 0.0) d18 = 0.0;
            else { d17 *= d17; d18 = d17 * d17 * simplex_grad(j2, d11, d12); }
            double d19 = 0.5 - d13 * d13 - d14 * d14;
            double d20;
            if (d19 < 0.0) d20 = 0.0;
            else { d19 *= d19; d20 = d19 * d19 * simplex_grad(k2, d13, d14); }
            double d21 = 0.5 - d15 * d15 - d16 * d16;
            double d22;
            if (d21 < 0.0) d22 = 0.0;
            else { d21 *= d21; d22 = d21 * d21 * simplex_grad(l2, d15, d16); }
            out[k++] += 70.0 * (d18 + d20 + d22) * weight;
        }
    }
}

double or_simplex_point(const or_perlin* g, double xs, double zs) {
    double out = 0.0;
    or_simplex_add(g, &out, xs, zs, 1, 1, 1, 1, 1.0, 1.0, 1.0);
    return out;
}

/* NoiseGeneratorOctaves2173.aStrided (noise/NoiseGeneratorOctaves2173.java:66-104). */
static void simplex_octaves(const or_perlin* gens, int n, double* out, double x0, double z0,
                            int xLen, int zLen, int strideX, int strideZ,
                            double d2, double d3, double d4, double d5) {
    d2 /= 1.5;
    d3 /= 1.5;
    for (int k = 0; k < xLen * zLen; ++k) out[k] = 0.0;
    double d6 = 1.0, d7 = 1.0;
    for (int l = 0; l < n; ++l) {
        or_simplex_add(&gens[l], out, x0, z0, xLen, zLen, strideX, strideZ, d2 * d7, d3 * d7, 0.55 / d6);
        d7 *= d4;
        d6 *= d5;
    }
}

/* WorldChunkManager173.getBiomeNoise / getClimateNoiseStrided climate formula
 * (WorldChunkManager173.java:85-130, 140-219) over a strided block grid. */
static void climate_grid(const or_world* w, int startX, int startZ, int sizeX, int sizeZ,
                         int strideX, int strideZ, double* temp, double* rain, double* blend) {
    simplex_octaves(w->temp, 4, temp, (double)startX, (double)startZ, sizeX, sizeZ, strideX, strideZ,
                    0.02500000037252903, 0.02500000037252903, 0.25, 0.5);
    simplex_octaves(w->rain, 4, rain, (double)startX, (double)startZ, sizeX, sizeZ, strideX, strideZ,
                    0.05000000074505806, 0.05000000074505806, 0.3333333333333333, 0.5);
    simplex_octaves(w->blend, 2, blend, (double)startX, (double)startZ, sizeX, sizeZ, strideX, strideZ,
                    0.25, 0.25, 0.5882352941176471, 0.5);
    for (int i = 0; i < sizeX * sizeZ; ++i) {
        double d0 = blend[i] * 1.1 + 0.5;
        double d1 = 0.01;
        double d2 = 1.0 - d1;
        double d3 = (temp[i] * 0.15 + 0.7) * d2 + d0 * d1;
        d1 = 0.0020;
        d2 = 1.0 - d1;
        double d4 = (rain[i] * 0.15 + 0.5) * d2 + d0 * d1;
        d3 = 1.0 - (1.0 - d3) * (1.0 - d3);
        if (d3 < 0.0) d3 = 0.0;
        if (d4 < 0.0) d4 = 0.0;
        if (d3 > 1.0) d3 = 1.0;
        if (d4 > 1.0) d4 = 1.0;
        temp[i] = d3;
        rain[i] = d4;
    }
}

void or_climate(const or_world* w, int blockX, int blockZ, double* temperature, double* rain) {
    double t, r, b;
    climate_grid(w, blockX, blockZ, 1, 1, 1, 1, &t, &r, &b);
    *temperature = t;
    *rain = r;
}

/* Per-column shape terms of generateTerrainNoise (BetaTerrain173.java:753-804):
 * d5 (height scale) and d7 (height centre) from climate and noise4/noise5. */
static void column_shape(double temperature, double rain, double n4, double n5, int yLen,
                         double* outD5, double* outD7) {
    double d2 = temperature;
    double d3 = rain * d2;
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
    d6 = d6 * (double)yLen / 16.0;
    *outD5 = d5;
    *outD7 = (double)yLen / 2.0 + d6 * 4.0;
}

/* Per-y density of generateTerrainNoise (BetaTerrain173.java:808-830). */
static double density_at(int j3, int yLen, double d5, double d7, double n1, double n2, double n3) {
    double d8;
    double d9 = ((double)j3 - d7) * 12.0 / d5;
    if (d9 < 0.0) d9 *= 4.0;
    double d10 = n2 / 512.0;
    double d11 = n3 / 512.0;
    double d12 = (n1 / 10.0 + 1.0) / 2.0;
    if (d12 < 0.0) d8 = d10;
    else if (d12 > 1.0) d8 = d11;
    else d8 = d10 + (d11 - d10) * d12;
    d8 -= d9;
    if (j3 > yLen - 4) {
        double d13 = (double)((float)(j3 - (yLen - 4)) / 3.0F);
        d8 = d8 * (1.0 - d13) + -10.0 * d13;
    }
    return d8;
}

/* BetaTerrain173.generateTerrainNoise (:667-834) over a lattice whose column
 * (i,j) sits at coarse (fromX + i*step, fromZ + j*step); temp/rain hold the
 * climate already sampled for each column (index i*zLen+j). yLen = 17. */
/* The five octave sums of generateTerrainNoise (:684-738) over the lattice:
 * n1/n2/n3 [cols][17], n4/n5 [cols], zero-initialised by the caller. */
static void terrain_noise_arrays(const or_world* w, int fromX, int fromZ, int xLen, int zLen, int step,
                                 double* n1, double* n2, double* n3, double* n4, double* n5) {
    const int yLen = 17;
    double amp;
    double fx = (double)fromX, fz = (double)fromZ, st = (double)step;
    /* NoiseGeneratorOctaves173.generateNoise (noise/NoiseGeneratorOctaves173.java:46-90). */
    amp = 1.0;
    for (int o = 0; o < 10; ++o) { or_perlin_add(&w->n4[o], n4, fx, 10.0, fz, xLen, 1, zLen, st, st, 1.121 * amp, 1.0 * amp, 1.121 * amp, amp); amp /= 2.0; }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) { or_perlin_add(&w->n5[o], n5, fx, 10.0, fz, xLen, 1, zLen, st, st, 200.0 * amp, 1.0 * amp, 200.0 * amp, amp); amp /= 2.0; }
    double d0 = 684.412, d1 = 684.412;
    amp = 1.0;
    for (int o = 0; o < 8; ++o) { or_perlin_add(&w->n1[o], n1, fx, 0.0, fz, xLen, yLen, zLen, st, st, d0 / 80.0 * amp, d1 / 160.0 * amp, d0 / 80.0 * amp, amp); amp /= 2.0; }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) { or_perlin_add(&w->n2[o], n2, fx, 0.0, fz, xLen, yLen, zLen, st, st, d0 * amp, d1 * amp, d0 * amp, amp); amp /= 2.0; }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) { or_perlin_add(&w->n3[o], n3, fx, 0.0, fz, xLen, yLen, zLen, st, st, d0 * amp, d1 * amp, d0 * amp, amp); amp /= 2.0; }
}

static void terrain_noise(const or_world* w, double* noise, int fromX, int fromZ, int xLen, int zLen,
                          int step, const double* temp, const double* rain) {
    const int yLen = 17;
    int cols = xLen * zLen;
    double* n4 = (double*)calloc((size_t)cols, sizeof(double));
    double* n5 = (double*)calloc((size_t)cols, sizeof(double));
    double* n1 = (double*)calloc((size_t)cols * yLen, sizeof(double));
    double* n2 = (double*)calloc((size_t)cols * yLen, sizeof(double));
    double* n3 = (double*)calloc((size_t)cols * yLen, sizeof(double));
    terrain_noise_arrays(w, fromX, fromZ, xLen, zLen, step, n1, n2, n3, n4, n5);
    int k1 = 0;
    for (int c = 0; c < cols; ++c) {
        double d5, d7;
        column_shape(temp[c], rain[c], n4[c], n5[c], yLen, &d5, &d7);
        for (int j3 = 0; j3 < yLen; ++j3, ++k1) {
            noise[k1] = density_at(j3, yLen, d5, d7, n1[k1], n2[k1], n3[k1]);
        }
    }
    free(n4); free(n5); free(n1); free(n2); free(n3);
}

/* Sparse-lattice density column as the worker kernels evaluate it
 * (gpu_p20_benchmark.cpp:517-578, p33_shared_y.hpp:262-326,
 * p30_compact_lower.hpp:193-223, coarse_exact_core.hpp:311-348): the same
 * generateTerrainNoise arithmetic for one lattice column, climate at the given
 * block. Outputs y in [yLo, 17). */
void or_density_column(const or_world* w, int cx, int cz, int climX, int climZ, int yLo, double* out17) {
    double temp, rain;
    or_climate(w, climX, climZ, &temp, &rain);
    double n1[17] = {0}, n2[17] = {0}, n3[17] = {0}, n4 = 0.0, n5 = 0.0;
    double X = (double)cx, Z = (double)cz;
    double amp = 1.0;
    for (int o = 0; o < 16; ++o) { perlin_column17(&w->n2[o], X * (684.412 * amp), 684.412 * amp, Z * (684.412 * amp), yLo, amp, n2); amp /= 2.0; }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) { perlin_column17(&w->n3[o], X * (684.412 * amp), 684.412 * amp, Z * (684.412 * amp), yLo, amp, n3); amp /= 2.0; }
    amp = 1.0;
    for (int o = 0; o < 8; ++o) { perlin_column17(&w->n1[o], X * (684.412 / 80.0 * amp), 684.412 / 160.0 * amp, Z * (684.412 / 80.0 * amp), yLo, amp, n1); amp /= 2.0; }
    amp = 1.0;
    for (int o = 0; o < 10; ++o) { or_perlin_add(&w->n4[o], &n4, X, 10.0, Z, 1, 1, 1, 1.0, 1.0, 1.121 * amp, 1.0 * amp, 1.121 * amp, amp); amp /= 2.0; }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) { or_perlin_add(&w->n5[o], &n5, X, 10.0, Z, 1, 1, 1, 1.0, 1.0, 200.0 * amp, 1.0 * amp, 200.0 * amp, amp); amp /= 2.0; }
    double d5, d7;
    column_shape(temp, rain, n4, n5, 17, &d5, &d7);
    for (int y = 0; y < 17; ++y) out17[y] = y < yLo ? 0.0 : density_at(y, 17, d5, d7, n1[y], n2[y], n3[y]);
}

/* generateChunkBaseTerrain (BetaTerrain173.java:120-138) = getBiomeNoise for the
 * chunk's 16x16 blocks + generateBareTerrain (:582-665). */
void or_chunk_base_terrain(const or_world* w, int chunkX, int chunkZ, uint8_t* blocks) {
    double temp[256], rain[256], blend[256];
    climate_grid(w, chunkX * 16, chunkZ * 16, 16, 16, 1, 1, temp, rain, blend);
    /* generateTerrainNoise samples temperature[k2*16+i3], k2 = j2*3+1 (:741-749). */
    double ct[25], cr[25];
    for (int j2 = 0; j2 < 5; ++j2)
        for (int l2 = 0; l2 < 5; ++l2) {
            int k2 = j2 * 3 + 3 / 2, i3 = l2 * 3 + 3 / 2;
            ct[j2 * 5 + l2] = temp[k2 * 16 + i3];
            cr[j2 * 5 + l2] = rain[k2 * 16 + i3];
        }
    double noise[5 * 17 * 5];
    terrain_noise(w, noise, chunkX * 4, chunkZ * 4, 5, 5, 1, ct, cr);
    const int l = 5, b2 = 17;
    for (int i1 = 0; i1 < 4; ++i1) {
        for (int j1 = 0; j1 < 4; ++j1) {
            for (int k1 = 0; k1 < 16; ++k1) {
                double d0 = 0.125;
                double d1 = noise[((i1 + 0) * l + j1 + 0) * b2 + k1 + 0];
                double d2 = noise[((i1 + 0) * l + j1 + 1) * b2 + k1 + 0];
                double d3 = noise[((i1 + 1) * l + j1 + 0) * b2 + k1 + 0];
                double d4 = noise[((i1 + 1) * l + j1 + 1) * b2 + k1 + 0];
                double d5 = (noise[((i1 + 0) * l + j1 + 0) * b2 + k1 + 1] - d1) * d0;
                double d6 = (noise[((i1 + 0) * l + j1 + 1) * b2 + k1 + 1] - d2) * d0;
                double d7 = (noise[((i1 + 1) * l + j1 + 0) * b2 + k1 + 1] - d3) * d0;
                double d8 = (noise[((i1 + 1) * l + j1 + 1) * b2 + k1 + 1] - d4) * d0;
                for (int l1 = 0; l1 < 8; ++l1) {
                    double d9 = 0.25;
                    double d10 = d1;
                    double d11 = d2;
                    double d12 = (d3 - d1) * d9;
                    double d13 = (d4 - d2) * d9;
                    for (int i2 = 0; i2 < 4; ++i2) {
                        int x = i2 + i1 * 4;
                        int y = k1 * 8 + l1;
                        double d14 = 0.25;
                        double d15 = d10;
                        double d16 = (d11 - d10) * d14;
                        for (int k2 = 0; k2 < 4; ++k2) {
                            int z = j1 * 4 + k2;
                            double t = temp[(i1 * 4 + i2) * 16 + j1 * 4 + k2];
                            int block = 0;
                            if (y < 64) block = (t < 0.5 && y >= 63) ? 3 : 2;
                            if (d15 > 0.0) block = 1;
                            blocks[(x * 16 + z) * 128 + y] = (uint8_t)block;
                            d15 += d16;
                        }
                        d10 += d12;
                        d11 += d13;
                    }
                    d1 += d5;
                    d2 += d6;
                    d3 += d7;
                    d4 += d8;
                }
            }
        }
    }
}

static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* Bitmap hash (defined by this project): sum over the 512 little-endian
 * 64-bit words w_i of mix64(w_i + (i+1) * 0x9E3779B97F4A7C15), mod 2^64. */
uint64_t or_bitmap_hash(const uint8_t* bm) {
    uint64_t h = 0;
    for (int i = 0; i < 512; ++i) {
        uint64_t v = 0;
        for (int b = 0; b < 8; ++b) v |= (uint64_t)bm[i * 8 + b] << (8 * b);
        h += mix64(v + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ULL);
    }
    return h;
}

static uint64_t chunk_bitmap_world(const or_world* w, int chunkX, int chunkZ, uint8_t* bm) {
    uint8_t blocks[32768];
    or_chunk_base_terrain(w, chunkX, chunkZ, blocks);
    memset(bm, 0, 4096);
    for (int i = 0; i < 32768; ++i)
        if (blocks[i] == 1) bm[i >> 3] |= (uint8_t)(1u << (i & 7));
    return or_bitmap_hash(bm);
}

/* Test hook: the chunk path's five noise sums at the 5x5 lattice columns of chunk
 * (chunkX, chunkZ), i.e. coarse (4*chunkX + i, 4*chunkZ + j), column index i*5+j:
 * n1/n2/n3 [25][17], n4/n5 [25]. */
void or_chunk_noise_test(int64_t seed, int chunkX, int chunkZ, double* n1, double* n2, double* n3, double* n4,
                         double* n5) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, seed);
    memset(n1, 0, sizeof(double) * 25 * 17);
    memset(n2, 0, sizeof(double) * 25 * 17);
    memset(n3, 0, sizeof(double) * 25 * 17);
    memset(n4, 0, sizeof(double) * 25);
    memset(n5, 0, sizeof(double) * 25);
    terrain_noise_arrays(w, chunkX * 4, chunkZ * 4, 5, 5, 1, n1, n2, n3, n4, n5);
    free(w);
}

uint64_t or_chunk_stone_bitmap(int64_t seed, int chunkX, int chunkZ, uint8_t* bm) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, seed);
    uint64_t h = chunk_bitmap_world(w, chunkX, chunkZ, bm);
    free(w);
    return h;
}

/* ---- simple thread pool helper -------------------------------------------- */
typedef void (*or_task_fn)(void* ctx, int index);
typedef struct {
    or_task_fn fn;
    void* ctx;
    int n;
    volatile int next;
    pthread_mutex_t lock;
} or_pool;

static void* pool_worker(void* arg) {
    or_pool* p = (or_pool*)arg;
    for (;;) {
        pthread_mutex_lock(&p->lock);
        int i = p->next++;
        pthread_mutex_unlock(&p->lock);
        if (i >= p->n) break;
        p->fn(p->ctx, i);
    }
    return 0;
}

static void run_parallel(or_task_fn fn, void* ctx, int n, int threads) {
    if (threads <= 1 || n <= 1) {
        for (int i = 0; i < n; ++i) fn(ctx, i);
        return;
    }
    or_pool p;
    p.fn = fn; p.ctx = ctx; p.n = n; p.next = 0;
    pthread_mutex_init(&p.lock, 0);
    if (threads > 256) threads = 256;
    pthread_t tids[256];
    for (int t = 0; t < threads; ++t) pthread_create(&tids[t], 0, pool_worker, &p);
    for (int t = 0; t < threads; ++t) pthread_join(tids[t], 0);
    pthread_mutex_destroy(&p.lock);
}

typedef struct { const int64_t* seeds; int cx, cz; uint8_t* bitmaps; uint64_t* hashes; } bitmap_ctx;
static void bitmap_task(void* c, int i) {
    bitmap_ctx* b = (bitmap_ctx*)c;
    b->hashes[i] = or_chunk_stone_bitmap(b->seeds[i], b->cx, b->cz, b->bitmaps + (size_t)i * 4096);
}

void or_chunk_bitmaps(const int64_t* seeds, int n, int chunkX, int chunkZ,
                      uint8_t* bitmaps, uint64_t* hashes, int threads) {
    bitmap_ctx c = {seeds, chunkX, chunkZ, bitmaps, hashes};
    run_parallel(bitmap_task, &c, n, threads);
}

/* ========================================================================== */
/* Worker hunt profiles (gpu_p20_benchmark.cpp:7262-7290). */
void or_profile_get(int id, or_profile* p) {
    switch (id) {
        case 1: p->p20MinCount = 1; p->upperMinCount = 8; p->highMinCount = 6; p->p19MinScore = BSF_P19_THRESHOLD; p->coarseMinCells = 85; p->megaTopologyFilter = 1; break;
        case 2: p->p20MinCount = 3; p->upperMinCount = 19; p->highMinCount = 12; p->p19MinScore = 6.70; p->coarseMinCells = 95; p->megaTopologyFilter = 0; break;
        case 3: p->p20MinCount = 3; p->upperMinCount = 19; p->highMinCount = 20; p->p19MinScore = 6.70; p->coarseMinCells = 700; p->megaTopologyFilter = 0; break;
        default: p->p20MinCount = 1; p->upperMinCount = 5; p->highMinCount = 5; p->p19MinScore = BSF_P19_THRESHOLD; p->coarseMinCells = 85; p->megaTopologyFilter = 0; break;
    }
}

/* P20 axis (gpu_p20_benchmark.cpp:41-52; BetaTerrain173.java:1801-1809). */
static const int P20_AXIS[8] = {0, 2, 5, 7, 8, 10, 13, 15};
static int is_p20_axis(int i) { for (int k = 0; k < 8; ++k) if (P20_AXIS[k] == i) return 1; return 0; }

/* stage0gpu::highestReentryYIndex (stage0_exact_gpu.hpp:552-566). */
static int highest_reentry(uint32_t mask) {
    int sawPos = 0, sawGap = 0, highest = -1;
    for (int y = 0; y < 17; ++y) {
        int pos = (mask >> y) & 1u;
        if (pos) {
            if (sawPos && sawGap) highest = y;
            sawPos = 1;
        } else if (sawPos) {
            sawGap = 1;
        }
    }
    return highest;
}

/* fillMonsterShapeStats (gpu_p20_benchmark.cpp:1022-1088). */
static void shape_stats(const uint8_t* grid, int* largestOut, int* widthOut, int* depthOut, int* touchesOut) {
    const int size = 16;
    uint8_t visited[256] = {0};
    int queue[256];
    int largest = 0, minX = size, maxX = -1, minZ = size, maxZ = -1, touches = 0;
    for (int x = 0; x < size; ++x) {
        for (int z = 0; z < size; ++z) {
            int index = x * size + z;
            if (grid[index] == 0) continue;
            if (x < minX) minX = x;
            if (x > maxX) maxX = x;
            if (z < minZ) minZ = z;
            if (z > maxZ) maxZ = z;
            if (x == 0 || z == 0 || x == size - 1 || z == size - 1) touches = 1;
            if (visited[index]) continue;
            int head = 0, tail = 0, cluster = 0;
            visited[index] = 1;
            queue[tail++] = index;
            while (head < tail) {
                int cur = queue[head++];
                ++cluster;
                int cx = cur / size, cz = cur % size;
                int nx[4] = {cx - 1, cx + 1, cx, cx};
                int nz[4] = {cz, cz, cz - 1, cz + 1};
                for (int k = 0; k < 4; ++k) {
                    if (nx[k] < 0 || nz[k] < 0 || nx[k] >= size || nz[k] >= size) continue;
                    int nb = nx[k] * size + nz[k];
                    if (grid[nb] == 0 || visited[nb]) continue;
                    visited[nb] = 1;
                    queue[tail++] = nb;
                }
            }
            if (cluster > largest) largest = cluster;
        }
    }
    *largestOut = largest;
    *widthOut = largest == 0 ? 0 : maxX - minX + 1;
    *depthOut = largest == 0 ? 0 : maxZ - minZ + 1;
    *touchesOut = touches;
}

/* buildMonsterFeatures (gpu_p20_benchmark.cpp:1090-1114). */
void or_monster_features(const uint8_t* highest256, or_features* f) {
    uint8_t y88[256] = {0}, y96[256] = {0};
    memset(f, 0, sizeof(*f));
    for (int c = 0; c < 256; ++c) {
        uint8_t e = highest256[c];
        if (e == 0xFF) continue;
        int h = e;
        if (h >= 11) { ++f->fullY88; y88[c] = 1; }
        if (h >= 12) { ++f->fullY96; y96[c] = 1; }
        if (h >= 13) ++f->fullY104;
        if (h >= 14) ++f->fullY112;
    }
    shape_stats(y88, &f->y88Largest, &f->y88Width, &f->y88Depth, &f->y88Touches);
    shape_stats(y96, &f->y96Largest, &f->y96Width, &f->y96Depth, &f->y96Touches);
}

/* Tree feature values (expressions of p19_monster_gate.hpp trees, ids as in p19_table.inc). */
static double p19_feature(int id, int scout, const or_features* p) {
    const double EPS = BSF_P19_EPSILON;
    switch (id) {
        case 0: return (double)scout;
        case 1: return (double)p->fullY88;
        case 2: return (double)p->fullY96;
        case 3: return (double)p->fullY104;
        case 4: return (double)p->fullY112;
        case 5: return (double)p->y88Largest;
        case 6: return (double)p->y88Width;
        case 7: return (double)p->y88Depth;
        case 8: return (double)p->y96Largest;
        case 9: return (double)p->y96Width;
        case 10: return (double)p->y96Depth;
        case 11: return (double)p->fullY88 / ((double)scout + EPS);
        case 12: return (double)(p->y88Width + p->y88Depth + p->y96Width + p->y96Depth);
        case 13: return (double)(p->y96Width * p->y96Depth);
        case 14: return (double)(p->y88Width * p->y88Depth);
        case 15: return (double)p->y88Largest / ((double)p->fullY88 + EPS);
        case 16: return (double)(p->fullY96 + p->fullY104 + p->fullY112);
        case 17: return (double)p->y96Largest / ((double)p->fullY96 + EPS);
        case 18: return (double)p->fullY104 / ((double)p->fullY96 + EPS);
        case 19: return (double)p->fullY96 / ((double)p->fullY88 + EPS);
        default: return (double)(p->y88Largest + p->y96Largest);
    }
}

/* p19native::score (p19_monster_gate.hpp:48-67): mean of 16 trees summed in order. */
double or_p19_score(int scout, const or_features* f) {
    double sum = 0.0;
    for (int t = 0; t < BSF_P19_TREE_COUNT; ++t) {
        int n = bsf_p19_root[t];
        while (bsf_p19_feature[n] >= 0) {
            double v = p19_feature(bsf_p19_feature[n], scout, f);
            n = v <= bsf_p19_value[n] ? bsf_p19_left[n] : bsf_p19_right[n];
        }
        sum = t == 0 ? bsf_p19_value[n] : sum + bsf_p19_value[n];
    }
    return sum / (double)BSF_P19_TREE_COUNT;
}

/* p19native::hasExtremeTopologySignal (p19_monster_gate.hpp:77-79). */
int or_p19_extreme(const or_features* f) { return f->y88Largest >= 14 || f->y96Largest >= 14; }

/* megaTopologyReject (gpu_p20_benchmark.cpp:1116-1128 = src/MegaFilter.java:27-48). */
int or_mega_topology_reject(double score, int extreme, const or_features* f) {
    if (extreme) return 0;
    if (!(score < 5.0)) return 0;
    return f->fullY112 == 0 || f->y96Largest < 4;
}

/* Coarse 61x61x17 sign lattice (coarse_exact_core.hpp:218-350 with the
 * centre offset of p35_direct_coarse.hpp): coarse coords -28..32 + centre*4,
 * climate at block 4c+2. signs[(x*61+z)*17+y]. */
void or_coarse_signs(const or_world* w, int centerChunkX, int centerChunkZ, uint8_t* signs) {
    const int S = 61;
    int fromX = -28 + centerChunkX * 4, fromZ = -28 + centerChunkZ * 4;
    double* temp = (double*)malloc(sizeof(double) * S * S);
    double* rain = (double*)malloc(sizeof(double) * S * S);
    double* blend = (double*)malloc(sizeof(double) * S * S);
    double* noise = (double*)malloc(sizeof(double) * S * S * 17);
    climate_grid(w, fromX * 4 + 2, fromZ * 4 + 2, S, S, 4, 4, temp, rain, blend);
    terrain_noise(w, noise, fromX, fromZ, S, S, 1, temp, rain);
    for (int i = 0; i < S * S * 17; ++i) signs[i] = noise[i] > 0.0 ? 1 : 0;
    free(temp); free(rain); free(blend); free(noise);
}

/* coarsecore::scoreSigns (coarse_exact_core.hpp:83-169). */
int or_coarse_score(const uint8_t* signs) {
    const int S = 61, Y = 17, COLS = S * S, CELLS = COLS * Y;
    int* labels = (int*)calloc(CELLS, sizeof(int));
    int* queue = (int*)malloc(sizeof(int) * CELLS);
    int* colSeen = (int*)calloc(COLS, sizeof(int));
    int* colMinY = (int*)malloc(sizeof(int) * COLS);
    int* compCols = (int*)malloc(sizeof(int) * COLS);
    int best = 0, nextId = 1;
#define IDX3(x, y, z) (((x) * S + (z)) * Y + (y))
    for (int x = 0; x < S; ++x)
        for (int z = 0; z < S; ++z)
            for (int y = 0; y < Y; ++y) {
                int start = IDX3(x, y, z);
                if (labels[start] != 0 || signs[start] == 0) continue;
                int id = nextId++;
                int head = 0, tail = 0;
                queue[tail++] = start;
                labels[start] = id;
                int cells = 0, maxY = 0, colCount = 0, touchBottom = 0, touchSide = 0;
                while (head < tail) {
                    int idx = queue[head++];
                    int cy = idx % Y, tmp = idx / Y, cz = tmp % S, cx = tmp / S;
                    ++cells;
                    if (cy > maxY) maxY = cy;
                    if (cy == 0) touchBottom = 1;
                    if (cx == 0 || cz == 0 || cx == S - 1 || cz == S - 1) touchSide = 1;
                    int col = cx * S + cz;
                    if (colSeen[col] != id) { colSeen[col] = id; compCols[colCount++] = col; colMinY[col] = cy; }
                    else if (cy < colMinY[col]) colMinY[col] = cy;
                    int nb[6]; int nn = 0;
                    if (cx + 1 < S) nb[nn++] = IDX3(cx + 1, cy, cz);
                    if (cx > 0) nb[nn++] = IDX3(cx - 1, cy, cz);
                    if (cy + 1 < Y) nb[nn++] = IDX3(cx, cy + 1, cz);
                    if (cy > 0) nb[nn++] = IDX3(cx, cy - 1, cz);
                    if (cz + 1 < S) nb[nn++] = IDX3(cx, cy, cz + 1);
                    if (cz > 0) nb[nn++] = IDX3(cx, cy, cz - 1);
                    for (int k = 0; k < nn; ++k)
                        if (labels[nb[k]] == 0 && signs[nb[k]] != 0) { labels[nb[k]] = id; queue[tail++] = nb[k]; }
                }
                if (cells <= best || maxY < 8 || touchBottom || touchSide) continue;
                int reentry = 0;
                for (int i = 0; i < colCount && !reentry; ++i) {
                    int col = compCols[i];
                    int ccx = col / S, ccz = col - ccx * S;
                    int minY = colMinY[col];
                    if (minY <= 0 || minY >= Y) continue;
                    for (int ly = minY - 1; ly >= 0; --ly) {
                        int idx = IDX3(ccx, ly, ccz);
                        if (signs[idx] != 0 && labels[idx] != id) {
                            if (minY - ly - 1 >= 1) reentry = 1;
                            break;
                        }
                    }
                }
                if (reentry) best = cells;
            }
#undef IDX3
    free(labels); free(queue); free(colSeen); free(colMinY); free(compCols);
    return best;
}

void or_coarse_signs_seed(int64_t seed, int centerChunkX, int centerChunkZ, uint8_t* signs) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, seed);
    or_coarse_signs(w, centerChunkX, centerChunkZ, signs);
    free(w);
}

int or_coarse_score_seed(int64_t seed, int centerChunkX, int centerChunkZ) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    uint8_t* signs = (uint8_t*)malloc(61 * 61 * 17);
    or_world_init(w, seed);
    or_coarse_signs(w, centerChunkX, centerChunkZ, signs);
    int s = or_coarse_score(signs);
    free(signs); free(w);
    return s;
}

/* loadRelevantCoarseGridAroundZero + findBestCoarseFloatingCellsLazy +
 * hasCoarseReentryColumnForComponent + completeLazyCoarseGridAndScoreFull
 * (IslandSearchEngine.java:3331-3564, 3726-3759; limits :78-84): component
 * search from upper-slice starts, lower levels generated per requested column
 * in rounds, components touching level 0 or the side abandoned at once. The
 * grid is the coarse lattice of or_coarse_signs (columns through
 * or_density_column, climate at block 4c+2). */
int or_coarse_score_lazy_seed(int64_t seed, int centerChunkX, int centerChunkZ, or_lazy_stats* stats) {
    enum { S = 61, Y = 17, COLS = S * S, CELLS = COLS * Y, MIN_Y = 8 };
    enum { MAX_LOWER = 512, MAX_ROUNDS = 32, MAX_QUEUE = 12000 };
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, seed);
    const int fromX = -28 + centerChunkX * 4, fromZ = -28 + centerChunkZ * 4;
    double* values = (double*)malloc(sizeof(double) * CELLS);
    uint8_t* lowerDone = (uint8_t*)calloc(COLS, 1);
    uint8_t* request = (uint8_t*)calloc(COLS, 1);
    int* labels = (int*)calloc(CELLS, sizeof(int));
    int* queue = (int*)malloc(sizeof(int) * CELLS);
    int* colSeen = (int*)calloc(COLS, sizeof(int));
    int* colMinY = (int*)malloc(sizeof(int) * COLS);
    int* compCols = (int*)malloc(sizeof(int) * COLS);
    double col17[17];
    int lowerColumns = 0, rounds = 0, fallback = 0, best = 0, nextId = 1;
#define LIDX(x, y, z) (((x) * S + (z)) * Y + (y))
    for (int i = 0; i < CELLS; ++i) values[i] = -INFINITY;  /* not generated: not positive */
    for (int x = 0; x < S; ++x)
        for (int z = 0; z < S; ++z) {
            const int cx = fromX + x, cz = fromZ + z;
            or_density_column(w, cx, cz, cx * 4 + 2, cz * 4 + 2, MIN_Y, col17);
            for (int y = MIN_Y; y < Y; ++y) values[LIDX(x, y, z)] = col17[y];
        }
    /* completeCoarseDensityLowerColumnsAroundZeroInto: levels 0..MIN_Y-1 of the requested columns */
#define COMPLETE_REQUESTED()                                                              \
    for (int col = 0; col < COLS; ++col) {                                              \
        if (!request[col] || lowerDone[col]) continue;                                  \
        const int x = col / S, z = col % S, cx = fromX + x, cz = fromZ + z;               \
        or_density_column(w, cx, cz, cx * 4 + 2, cz * 4 + 2, 0, col17);                   \
        for (int y = 0; y < MIN_Y; ++y) values[LIDX(x, y, z)] = col17[y];                  \
        lowerDone[col] = 1;                                                             \
        ++lowerColumns;                                                                 \
    }                                                                                   \
    memset(request, 0, COLS)
    for (int x = 0; x < S && !fallback; ++x)
        for (int z = 0; z < S && !fallback; ++z)
            for (int y = MIN_Y; y < Y && !fallback; ++y) {
                const int start = LIDX(x, y, z);
                if (labels[start] != 0 || !(values[start] > 0.0)) continue;
                const int id = nextId++;
                int head = 0, tail = 0, invalid = 0, compRounds = 0;
                queue[tail++] = start;
                labels[start] = id;
                memset(request, 0, COLS);
                for (;;) {
                    while (head < tail && !invalid) {
                        const int idx = queue[head++];
                        const int cy = idx % Y, tmp = idx / Y, cz = tmp % S, cx = tmp / S;
                        if (cy == 0 || cx == 0 || cz == 0 || cx == S - 1 || cz == S - 1) {
                            invalid = 1;
                            break;
                        }
                        static const int dirs[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
                        for (int d = 0; d < 6; ++d) {
                            const int nx = cx + dirs[d][0], ny = cy + dirs[d][1], nz = cz + dirs[d][2];
                            if (nx < 0 || nx >= S || ny < 0 || ny >= Y || nz < 0 || nz >= S) continue;
                            const int ni = LIDX(nx, ny, nz);
                            if (ny < MIN_Y && !lowerDone[nx * S + nz]) {
                                request[nx * S + nz] = 1;
                                continue;
                            }
                            if (values[ni] > 0.0) {
                                if (labels[ni] < 0) {
                                    invalid = 1;
                                    break;
                                }
                                if (labels[ni] == 0) {
                                    labels[ni] = id;
                                    queue[tail++] = ni;
                                }
                            }
                        }
                    }
                    if (invalid) break;
                    int requested = 0;
                    for (int col = 0; col < COLS; ++col) {
                        if (request[col] && !lowerDone[col]) ++requested;
                        else request[col] = 0;
                    }
                    if (requested == 0) break;
                    COMPLETE_REQUESTED();
                    ++compRounds;
                    if (lowerColumns > MAX_LOWER || rounds + compRounds > MAX_ROUNDS || tail > MAX_QUEUE) {
                        fallback = 1;
                        break;
                    }
                    head = 0;  /* new lower cells can neighbour any reached cell: rescan */
                }
                if (fallback) break;
                rounds += compRounds;
                if (invalid) {
                    for (int i = 0; i < tail; ++i) labels[queue[i]] = -1;
                    continue;
                }
                int colCount = 0;
                for (int i = 0; i < tail; ++i) {
                    const int idx = queue[i];
                    const int py = idx % Y, col = idx / Y;
                    if (colSeen[col] != id) {
                        colSeen[col] = id;
                        compCols[colCount++] = col;
                        colMinY[col] = py;
                    } else if (py < colMinY[col]) {
                        colMinY[col] = py;
                    }
                }
                if (tail <= best) continue;
                /* the re-entry test reads the lower slice of every component column */
                for (int i = 0; i < colCount; ++i)
                    if (!lowerDone[compCols[i]]) request[compCols[i]] = 1;
                COMPLETE_REQUESTED();
                int reentry = 0;
                for (int i = 0; i < colCount && !reentry; ++i) {
                    const int col = compCols[i], ccx = col / S, ccz = col % S, minY = colMinY[col];
                    if (minY <= 0 || minY >= Y) continue;
                    for (int ly = minY - 1; ly >= 0; --ly) {
                        const int idx = LIDX(ccx, ly, ccz);
                        if (values[idx] > 0.0 && labels[idx] != id) {
                            if (minY - ly - 1 >= 1) reentry = 1;  /* MIN_FLOATING_GAP_STEPS */
                            break;
                        }
                    }
                }
                if (reentry) best = tail;
            }
    if (fallback) {
        /* completeLazyCoarseGridAndScoreFull: every lower slice, then the full scorer */
        for (int col = 0; col < COLS; ++col) request[col] = 1;
        COMPLETE_REQUESTED();
        uint8_t* signs = (uint8_t*)malloc(CELLS);
        for (int i = 0; i < CELLS; ++i) signs[i] = values[i] > 0.0 ? 1 : 0;
        best = or_coarse_score(signs);
        free(signs);
    }
#undef COMPLETE_REQUESTED
#undef LIDX
    if (stats) {
        stats->lowerColumns = lowerColumns;
        stats->rounds = rounds;
        stats->fallbackToFull = fallback;
    }
    free(values); free(lowerDone); free(request); free(labels); free(queue);
    free(colSeen); free(colMinY); free(compCols); free(w);
    return best;
}

/* One region through the worker's stage0stream stages
 * (gpu_p20_benchmark.cpp:7421-7502): P20 on the 64 axis columns, Upper on the
 * rest when the gated P20 count is positive, Lower for upper-positive columns
 * when Upper >= upperMin, then P19 + extreme bypass + Mega topology, then the
 * coarse score for P19 survivors. */
void or_stage0_region(const or_world* w, int ccx, int ccz, const or_profile* prof, int runCoarse,
                      or_region* out) {
    memset(out, 0, sizeof(*out));
    memset(out->highest, 0xFF, sizeof(out->highest));
    out->p19Score = NAN;
    int offX = ccx * 4, offZ = ccz * 4;
    double col[17];
    int p20 = 0;
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) {
            int ix = P20_AXIS[i], iz = P20_AXIS[j];
            int cx = -28 + ix * 4 + offX, cz = -28 + iz * 4 + offZ;
            or_density_column(w, cx, cz, cx * 4 + 2, cz * 4 + 2, 11, col);
            uint8_t m = 0;
            for (int y = 11; y < 17; ++y) if (col[y] > 0.0) m |= (uint8_t)(1u << (y - 11));
            out->upperMask[ix * 16 + iz] = m;
            if (m) ++p20;
        }
    out->p20 = p20;
    int p20Gate = prof->p20MinCount > 1 ? (p20 >= prof->p20MinCount ? p20 : 0) : p20;
    if (p20Gate <= 0) { out->upper = 0; return; }
    int upper = p20Gate;
    for (int ix = 0; ix < 16; ++ix)
        for (int iz = 0; iz < 16; ++iz) {
            if (is_p20_axis(ix) && is_p20_axis(iz)) continue;
            int cx = -28 + ix * 4 + offX, cz = -28 + iz * 4 + offZ;
            or_density_column(w, cx, cz, cx * 4 + 2, cz * 4 + 2, 11, col);
            uint8_t m = 0;
            for (int y = 11; y < 17; ++y) if (col[y] > 0.0) m |= (uint8_t)(1u << (y - 11));
            out->upperMask[ix * 16 + iz] = m;
            if (m) ++upper;
        }
    out->upper = upper;
    if (upper < prof->upperMinCount) return;
    int high = 0;
    for (int c = 0; c < 256; ++c) {
        if (!out->upperMask[c]) continue;
        int ix = c >> 4, iz = c & 15;
        int cx = -28 + ix * 4 + offX, cz = -28 + iz * 4 + offZ;
        or_density_column(w, cx, cz, cx * 4 + 2, cz * 4 + 2, 0, col);
        uint32_t mask = (uint32_t)out->upperMask[c] << 11;
        for (int y = 0; y < 11; ++y) if (col[y] > 0.0) mask |= 1u << y;
        int h = highest_reentry(mask);
        out->highest[c] = h < 0 ? 0xFF : (uint8_t)h;
        if (h >= 11) ++high;
    }
    out->high = high;
    if (!(p20 >= prof->p20MinCount && upper >= prof->upperMinCount && high >= prof->highMinCount)) return;
    out->p19Evaluated = 1;
    or_monster_features(out->highest, &out->f);
    out->p19Score = or_p19_score(upper, &out->f);
    out->p19Extreme = or_p19_extreme(&out->f);
    out->p19Pass = out->p19Extreme || out->p19Score >= prof->p19MinScore;
    out->megaReject = out->p19Pass && prof->megaTopologyFilter &&
                      or_mega_topology_reject(out->p19Score, out->p19Extreme, &out->f);
    if (out->p19Pass && !out->megaReject && runCoarse) {
        uint8_t* signs = (uint8_t*)malloc(61 * 61 * 17);
        or_coarse_signs(w, ccx, ccz, signs);
        out->coarseEvaluated = 1;
        out->coarse = or_coarse_score(signs);
        free(signs);
    }
}

/* Response record packing (gpu_p20_benchmark.cpp:7504-7554). */
void or_pack_record(const or_region* r, int research, uint8_t* o) {
    int a = r->p20, b = r->upper, c = r->high, d = r->coarse;
    o[0] = (uint8_t)(a < 0 ? 0 : (a > 255 ? 255 : a));
    o[1] = (uint8_t)(b < 0 ? 0 : (b > 255 ? 255 : b));
    o[2] = (uint8_t)(c < 0 ? 0 : (c > 255 ? 255 : c));
    o[3] = (uint8_t)(r->p19Pass ? 1 : 0);
    o[4] = (uint8_t)(d & 0xFF);
    o[5] = (uint8_t)((d >> 8) & 0xFF);
    o[6] = (uint8_t)(r->p19Extreme ? 1 : 0);
    o[7] = (uint8_t)(r->megaReject ? 1 : 0);
    uint64_t bits;
    memcpy(&bits, &r->p19Score, 8);
    for (int k = 0; k < 8; ++k) o[8 + k] = (uint8_t)(bits >> (8 * k));
    if (!research) return;
#define PUT16(off, v) do { int vv = (v); unsigned int u = (unsigned)(vv < 0 ? 0 : (vv > 65535 ? 65535 : vv)); o[off] = (uint8_t)(u & 0xFF); o[(off) + 1] = (uint8_t)((u >> 8) & 0xFF); } while (0)
    PUT16(16, r->f.fullY88);
    PUT16(18, r->f.fullY96);
    PUT16(20, r->f.fullY104);
    PUT16(22, r->f.fullY112);
    PUT16(24, r->f.y88Largest);
    o[26] = (uint8_t)r->f.y88Width;
    o[27] = (uint8_t)r->f.y88Depth;
    o[28] = (uint8_t)(r->f.y88Touches ? 1 : 0);
    PUT16(29, r->f.y96Largest);
    o[31] = (uint8_t)r->f.y96Width;
    o[32] = (uint8_t)r->f.y96Depth;
    o[33] = (uint8_t)(r->f.y96Touches ? 1 : 0);
#undef PUT16
}

/* Stream centres (gpu_p20_benchmark.cpp:7316-7317 = GpuStage0Scout.java:19-21). */
static const int CENTER_X[8] = {0, 15, 0, 15, -15, -15, 0, 15};
static const int CENTER_Z[8] = {0, 0, 15, 15, 0, 15, -15, -15};

typedef struct { const int64_t* seeds; int centers, research; or_profile prof; uint8_t* out; } batch_ctx;
static void batch_task(void* c, int i) {
    batch_ctx* b = (batch_ctx*)c;
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, b->seeds[i]);
    size_t rec = b->research ? 34 : 16;
    for (int k = 0; k < b->centers; ++k) {
        or_region r;
        or_stage0_region(w, CENTER_X[k], CENTER_Z[k], &b->prof, 1, &r);
        or_pack_record(&r, b->research, b->out + ((size_t)i * b->centers + k) * rec);
    }
    free(w);
}

void or_stage0_batch(const int64_t* seeds, int n, int centers, int profileId, int research,
                     uint8_t* out, int threads) {
    batch_ctx c;
    c.seeds = seeds; c.centers = centers; c.research = research; c.out = out;
    or_profile_get(profileId, &c.prof);
    run_parallel(batch_task, &c, n, threads);
}

/* ========================================================================== */
/* MEGA exact scan: IslandSearchEngine.findFloatingIslandInSeed exact part
 * (IslandSearchEngine.java:2861-2977), floodFillFlat (:4096-4202),
 * isMatch (:3972-4003), compareComponents (:4079-4094). */
#define ISLAND_FLOOR_Y 68

void or_match_defaults(or_match_settings* s) {
    s->minBlocks = 1000; s->minColumns = 100; s->minYForMatch = 60;
    s->minWidth = 10; s->minDepth = 10; s->minAvgThickness = 2.0;
}

typedef struct {
    int blocks, columns;
    int minX, maxX, minZ, maxZ, minY, maxY;
    int64_t sumX, sumZ;
    int centerX, centerZ;
    int touchesBottom, touchesSide;
} comp;

static int java_round_div(int64_t sum, int n) {
    double v = (double)sum / (double)n;
    double f = floor(v);
    return (int)(v - f >= 0.5 ? f + 1.0 : f);
}

static void flood(const uint8_t* stone, uint8_t* visited, int* queue, int* colSeen, int mark,
                  int sx, int sy, int sz, int sizeX, int sizeY, int sizeZ,
                  int minWorldX, int minWorldZ, int floodMinY, comp* c, int* queueLen) {
    int yz = sizeY * sizeZ;
    int head = 0, tail = 0;
    int start = (sx * sizeY + sy) * sizeZ + sz;
    queue[tail++] = start;
    visited[start] = 1;
    c->blocks = 0; c->columns = 0;
    c->minX = INT_MAX; c->maxX = INT_MIN; c->minZ = INT_MAX; c->maxZ = INT_MIN;
    c->minY = INT_MAX; c->maxY = INT_MIN;
    c->sumX = 0; c->sumZ = 0; c->centerX = 0; c->centerZ = 0;
    c->touchesBottom = 0; c->touchesSide = 0;
#define TRY(ni) do { int _n = (ni); if (!visited[_n] && stone[_n]) { visited[_n] = 1; queue[tail++] = _n; } } while (0)
    while (head < tail) {
        int index = queue[head++];
        int x = index / yz;
        int rem = index - x * yz;
        int y = rem / sizeZ;
        int z = rem - y * sizeZ;
        int wx = minWorldX + x, wz = minWorldZ + z;
        c->blocks++;
        int ci = x * sizeZ + z;
        if (colSeen[ci] != mark) { colSeen[ci] = mark; c->columns++; c->sumX += wx; c->sumZ += wz; }
        if (wx < c->minX) c->minX = wx;
        if (wx > c->maxX) c->maxX = wx;
        if (wz < c->minZ) c->minZ = wz;
        if (wz > c->maxZ) c->maxZ = wz;
        if (y < c->minY) c->minY = y;
        if (y > c->maxY) c->maxY = y;
        if (y == 0) c->touchesBottom = 1;
        if (x == 0 || x == sizeX - 1 || z == 0 || z == sizeZ - 1) c->touchesSide = 1;
        if (x > 0) TRY(index - yz);
        if (x < sizeX - 1) TRY(index + yz);
        if (y > floodMinY) TRY(index - sizeZ);
        else if (y > 0 && stone[index - sizeZ]) c->touchesBottom = 1;
        if (y < sizeY - 1) TRY(index + sizeZ);
        if (z > 0) TRY(index - 1);
        if (z < sizeZ - 1) TRY(index + 1);
    }
#undef TRY
    if (c->columns > 0) {
        c->centerX = java_round_div(c->sumX, c->columns);
        c->centerZ = java_round_div(c->sumZ, c->columns);
    }
    if (queueLen) *queueLen = tail;
}

static int is_match(const comp* c, const or_match_settings* s) {
    if (c->blocks < s->minBlocks) return 0;
    if (c->columns < s->minColumns) return 0;
    if (c->maxY < s->minYForMatch) return 0;
    if (c->touchesBottom) return 0;
    int width = c->maxX - c->minX + 1, depth = c->maxZ - c->minZ + 1;
    if (width < s->minWidth) return 0;
    if (depth < s->minDepth) return 0;
    double avg = (double)c->blocks / (double)(c->columns > 1 ? c->columns : 1);
    return avg >= s->minAvgThickness;
}

static int compare_comp(const comp* a, const comp* b) {
    if (a->blocks != b->blocks) return a->blocks < b->blocks ? -1 : 1;
    if (a->columns != b->columns) return a->columns < b->columns ? -1 : 1;
    int areaA = (a->maxX - a->minX + 1) * (a->maxZ - a->minZ + 1);
    int areaB = (b->maxX - b->minX + 1) * (b->maxZ - b->minZ + 1);
    if (areaA != areaB) return areaA < areaB ? -1 : 1;
    return 0;
}

/* Exact scan at one radius; optionally returns the preview column model. */
static int exact_scan_impl(const or_world* w, int ccx, int ccz, int radius, const or_match_settings* s,
                           or_island* out, int32_t* pMinY, int32_t* pMaxY, int pCap) {
    int sizeX = (radius * 2 + 1) * 16, sizeZ = sizeX, sizeY = 128;
    int minWorldX = (ccx - radius) * 16, minWorldZ = (ccz - radius) * 16;
    size_t volume = (size_t)sizeX * sizeY * sizeZ;
    uint8_t* stone = (uint8_t*)calloc(volume, 1);
    uint8_t* visited = (uint8_t*)calloc(volume, 1);
    int* queue = (int*)malloc(sizeof(int) * volume);
    int* colSeen = (int*)calloc((size_t)sizeX * sizeZ, sizeof(int));
    int candCap = (radius * 2 + 1) * (radius * 2 + 1) * 4 * 128;
    int* cands = (int*)malloc(sizeof(int) * candCap);
    int candCount = 0;
    uint8_t* blocks = (uint8_t*)malloc(32768);
    int copyStartY = ISLAND_FLOOR_Y - 1;
    for (int cx = ccx - radius; cx <= ccx + radius; ++cx)
        for (int cz = ccz - radius; cz <= ccz + radius; ++cz) {
            or_chunk_base_terrain(w, cx, cz, blocks);
            int baseX = (cx - (ccx - radius)) * 16, baseZ = (cz - (ccz - radius)) * 16;
            for (int x = 0; x < 16; ++x)
                for (int z = 0; z < 16; ++z) {
                    int cand = (x == 4 || x == 12) && (z == 4 || z == 12);
                    for (int y = copyStartY; y < sizeY; ++y) {
                        if (blocks[(x * 16 + z) * 128 + y] != 1) continue;
                        int flat = ((baseX + x) * sizeY + y) * sizeZ + (baseZ + z);
                        stone[flat] = 1;
                        if (cand && y >= ISLAND_FLOOR_Y && blocks[(x * 16 + z) * 128 + y - 1] != 1)
                            cands[candCount++] = flat;
                    }
                }
        }
    free(blocks);
    comp best;
    int haveBest = 0, mark = 1;
    int yz = sizeY * sizeZ;
    for (int i = 0; i < candCount; ++i) {
        int index = cands[i];
        if (!stone[index] || visited[index]) continue;
        int x = index / yz, rem = index - x * yz, y = rem / sizeZ, z = rem - y * sizeZ;
        comp c;
        int qlen = 0;
        flood(stone, visited, queue, colSeen, mark++, x, y, z, sizeX, sizeY, sizeZ,
              minWorldX, minWorldZ, ISLAND_FLOOR_Y, &c, &qlen);
        if (!is_match(&c, s)) continue;
        if (!haveBest || compare_comp(&c, &best) > 0) {
            best = c;
            haveBest = 1;
            if (pMinY) {
                int width = c.maxX - c.minX + 1, depth = c.maxZ - c.minZ + 1;
                if (width * depth <= pCap) {
                    for (int k = 0; k < width * depth; ++k) { pMinY[k] = INT_MAX; pMaxY[k] = INT_MIN; }
                    for (int q = 0; q < qlen; ++q) {
                        int id = queue[q];
                        int qx = id / yz, qr = id - qx * yz, qy = qr / sizeZ, qz = qr - qy * sizeZ;
                        int t = (minWorldX + qx - c.minX) * depth + (minWorldZ + qz - c.minZ);
                        if (qy < pMinY[t]) pMinY[t] = qy;
                        if (qy > pMaxY[t]) pMaxY[t] = qy;
                    }
                }
            }
        }
    }
    free(stone); free(visited); free(queue); free(colSeen); free(cands);
    memset(out, 0, sizeof(*out));
    out->radiusUsed = radius;
    if (!haveBest) return 0;
    out->found = 1;
    out->blocks = best.blocks; out->columns = best.columns;
    out->minX = best.minX; out->maxX = best.maxX; out->minZ = best.minZ; out->maxZ = best.maxZ;
    out->minY = best.minY; out->maxY = best.maxY;
    out->centerX = best.centerX; out->centerZ = best.centerZ;
    out->touchesSide = best.touchesSide; out->touchesBottom = best.touchesBottom;
    out->sumX = best.sumX; out->sumZ = best.sumZ;
    return 1;
}

int or_exact_scan(int64_t seed, int ccx, int ccz, int radius, const or_match_settings* s, or_island* out) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, seed);
    int r = exact_scan_impl(w, ccx, ccz, radius, s, out, 0, 0, 0);
    free(w);
    return r;
}

int or_preview(int64_t seed, int ccx, int ccz, int radius, const or_match_settings* s, or_island* out,
               int32_t* minY, int32_t* maxY, int capacity) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, seed);
    int r = exact_scan_impl(w, ccx, ccz, radius, s, out, minY, maxY, capacity);
    free(w);
    return r;
}

static const int BORDER_RADII[5] = {10, 13, 16, 20, 24};
static int island_cmp(const or_island* a, const or_island* b) {
    comp ca, cb;
    ca.blocks = a->blocks; ca.columns = a->columns; ca.minX = a->minX; ca.maxX = a->maxX; ca.minZ = a->minZ; ca.maxZ = a->maxZ;
    cb.blocks = b->blocks; cb.columns = b->columns; cb.minX = b->minX; cb.maxX = b->maxX; cb.minZ = b->minZ; cb.maxZ = b->maxZ;
    return compare_comp(&ca, &cb);
}

/* verifySideBorderMatch (IslandSearchEngine.java:3188-3260). */
static int border_verify(const or_world* w, int ccx, int ccz, const or_match_settings* s, or_island* best) {
    for (int k = 0; k < 5; ++k) {
        int radius = BORDER_RADII[k];
        if (radius <= best->radiusUsed) continue;
        or_island e;
        if (!exact_scan_impl(w, ccx, ccz, radius, s, &e, 0, 0, 0)) return 0;
        *best = e;
        if (!best->touchesSide) return 1;
    }
    return 1;
}

/* processGpuRegionAttempt (IslandSearchEngine.java:1878-1971): exact scan at
 * the search radius with border verification, then the radius-16 hot scan
 * (with its own border verification) when coarse >= 120, keeping the larger. */
static int resolve_region_world(const or_world* w, int ccx, int ccz, int radius, int coarse,
                                const or_match_settings* s, or_island* out) {
    or_island normal;
    int haveNormal = exact_scan_impl(w, ccx, ccz, radius, s, &normal, 0, 0, 0);
    if (haveNormal && normal.touchesSide && radius < 24) haveNormal = border_verify(w, ccx, ccz, s, &normal);
    int have = haveNormal;
    or_island match = normal;
    if (radius < 16 && coarse >= 120) {
        or_island hot;
        int haveHot = exact_scan_impl(w, ccx, ccz, 16, s, &hot, 0, 0, 0);
        if (haveHot && hot.touchesSide && hot.radiusUsed < 24) haveHot = border_verify(w, ccx, ccz, s, &hot);
        if (haveHot && (!have || island_cmp(&hot, &match) > 0)) { match = hot; have = 1; }
    }
    memset(out, 0, sizeof(*out));
    if (have) *out = match;
    else out->radiusUsed = radius;
    return have;
}

int or_resolve_region(int64_t seed, int ccx, int ccz, int radius, int coarse,
                      const or_match_settings* s, or_island* out) {
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, seed);
    int r = resolve_region_world(w, ccx, ccz, radius, coarse, s, out);
    free(w);
    return r;
}

/* ---- full MEGA pipeline (CPU baseline) ----------------------------------- */
typedef struct {
    const int64_t* seeds;
    int radius;
    or_profile prof;
    const or_match_settings* s;
    or_region* regions;
    or_island* islands;
    uint8_t* hasIsland;
} mega_ctx;

static void mega_task(void* c, int i) {
    mega_ctx* m = (mega_ctx*)c;
    or_world* w = (or_world*)malloc(sizeof(or_world));
    or_world_init(w, m->seeds[i]);
    for (int k = 0; k < 8; ++k) {
        or_region* r = &m->regions[(size_t)i * 8 + k];
        or_stage0_region(w, CENTER_X[k], CENTER_Z[k], &m->prof, 1, r);
        m->hasIsland[(size_t)i * 8 + k] = 0;
        if (r->coarseEvaluated && r->coarse >= m->prof.coarseMinCells) {
            resolve_region_world(w, CENTER_X[k], CENTER_Z[k], m->radius, r->coarse, m->s,
                                 &m->islands[(size_t)i * 8 + k]);
            m->hasIsland[(size_t)i * 8 + k] = 1;
        }
    }
    free(w);
}

int or_mega_pipeline(const int64_t* seeds, int n, int profileId, int radius,
                     const or_match_settings* s, int threads,
                     or_pipeline_counts* counts, or_island* islands, int64_t* islandRegion, int islandCap) {
    mega_ctx m;
    m.seeds = seeds; m.radius = radius; m.s = s;
    or_profile_get(profileId, &m.prof);
    m.regions = (or_region*)malloc(sizeof(or_region) * (size_t)n * 8);
    m.islands = (or_island*)calloc((size_t)n * 8, sizeof(or_island));
    m.hasIsland = (uint8_t*)calloc((size_t)n * 8, 1);
    run_parallel(mega_task, &m, n, threads);
    or_pipeline_counts cnt;
    memset(&cnt, 0, sizeof(cnt));
    int written = 0;
    for (size_t r = 0; r < (size_t)n * 8; ++r) {
        const or_region* g = &m.regions[r];
        const or_profile* p = &m.prof;
        cnt.regions++;
        if (g->p20 >= p->p20MinCount) cnt.p20Passed++;
        if (g->p20 >= p->p20MinCount && g->upper >= p->upperMinCount) cnt.upperPassed++;
        if (g->p19Evaluated) cnt.highPassed++;
        if (g->p19Pass) cnt.p19Passed++;
        if (g->megaReject) cnt.megaRejected++;
        if (g->coarseEvaluated) cnt.coarseEvaluated++;
        if (m.hasIsland[r]) {
            cnt.coarsePassed++;
            if (m.islands[r].found) cnt.islands++;
            if (written < islandCap) {
                if (islands) islands[written] = m.islands[r];
                if (islandRegion) islandRegion[written] = (int64_t)r;
                ++written;
            }
        }
    }
    cnt.worlds = (uint64_t)n;
    if (counts) *counts = cnt;
    free(m.regions); free(m.islands); free(m.hasIsland);
    return written;
}

/* SplitMix64 deterministic seed (IslandSearchEngine.java:2551-2556). */
uint64_t or_splitmix_seed(uint64_t sequenceSeed, uint64_t attempt) {
    uint64_t z = sequenceSeed + attempt * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
