// Screened coarse 61x61x17 lattice signs for sm_103a.
//
// Persistent grid, one 512-thread CTA per SM looping over the queued regions.
// Per region the CTA stages the world's generators, the 40 3D Y axes (FP64 and
// FP32) and an axis table of the region's 61 X and 61 Z coarse coordinates for
// the 66 lattice octaves (exact FP64 index / fraction / fade, stored in FP32).
// Columns are processed in tiles of 512: the column shape (climate + noise4/5)
// and then the three Y ranges of the 40 3D octaves, all in FP32 with error
// bounds (bsf_screen.cuh). Undecided columns are recomputed in exact FP64, so
// the 17-bit sign masks equal those of the exact coarse kernel bit for bit.
#include "bsf_device.cuh"
#include "bsf_internal.h"
#include "bsf_screen.cuh"

#include <cstdio>
#include <stdexcept>

namespace bsf {
namespace {

using namespace screen;

constexpr int CT = 512;
constexpr int SIDE = 61;
constexpr int COLS = SIDE * SIDE;
constexpr int NOCT = 66;
constexpr int TILE = 512;
constexpr int FB_CAP = 1024;

struct AxisS {
    float f, fd;
    int i;
};

struct CoarseSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    YEntry y64[OCT3][17];
    YF yf[OCT3][17];
    AxisS axis[NOCT][2][SIDE];
    float shape[TILE][4];
    std::uint32_t mask[TILE];
    std::uint32_t fb[FB_CAP];
    int fbCount;
};

__device__ __forceinline__ GenTable gtab(const CoarseSmem& s) {
    GenTable t;
    t.perm = s.perm;
    t.off = &s.off[0][0];
    return t;
}

__device__ __forceinline__ double octave_scale(int o) {
    if (o < 16) return NOISE_XZ / static_cast<double>(1 << o);
    if (o < 32) return NOISE_XZ / static_cast<double>(1 << (o - 16));
    if (o < 40) return (NOISE_XZ / 80.0) / static_cast<double>(1 << (o - 32));
    if (o < 50) return 1.121 / static_cast<double>(1 << (o - 40));
    return 200.0 / static_cast<double>(1 << (o - 50));
}

__device__ __forceinline__ AxisF axf(const AxisS& a) { return AxisF{a.f, a.f - 1.0f, a.fd, a.i}; }

template <int Y0, int N>
__device__ unsigned exact_bits(const CoarseSmem& s, double X, double Z, double d5, double d7) {
    const GenTable t = gtab(s);
    double a1[N], a2[N], a3[N];
    double amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double sc = NOISE_XZ * amp;
        octave3_column<Y0, N>(t(ST_N2 + o), X * sc, Z * sc, s.y64[o], 1.0 / amp, a2, o == 0);
        amp /= 2.0;
    }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double sc = NOISE_XZ * amp;
        octave3_column<Y0, N>(t(ST_N3 + o), X * sc, Z * sc, s.y64[16 + o], 1.0 / amp, a3, o == 0);
        amp /= 2.0;
    }
    amp = 1.0;
    for (int o = 0; o < 8; ++o) {
        const double sc = (NOISE_XZ / 80.0) * amp;
        octave3_column<Y0, N>(t(ST_N1 + o), X * sc, Z * sc, s.y64[32 + o], 1.0 / amp, a1, o == 0);
        amp /= 2.0;
    }
    unsigned bits = 0;
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (density_at(Y0 + k, d5, d7, a1[k], a2[k], a3[k]) > 0.0) bits |= 1u << (Y0 + k);
    return bits;
}

// Exact column in FP64 for Y range r (0: [0,6), 1: [6,12), 2: [12,17)).
__device__ __noinline__ unsigned exact_column(const CoarseSmem& s, int cx, int cz, int r) {
    const GenTable t = gtab(s);
    double temp, rain, d5, d7;
    climate_at(t, cx * 4 + 2, cz * 4 + 2, temp, rain);
    const double X = static_cast<double>(cx), Z = static_cast<double>(cz);
    double amp = 1.0, acc = 0.0, n4, n5;
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
    column_shape(temp, rain, n4, n5, d5, d7);
    if (r == 0) return exact_bits<0, 6>(s, X, Z, d5, d7);
    if (r == 1) return exact_bits<6, 6>(s, X, Z, d5, d7);
    return exact_bits<12, 5>(s, X, Z, d5, d7);
}

// Column shape (climate at block 4c+2 + noise4/5) in FP32 with bounds.
__device__ __noinline__ void coarse_shape(CoarseSmem& s, int originX, int originZ, int kx, int kz, float* sh) {
    const int cx = originX + kx, cz = originZ + kz;
    Fe temp, rain;
    climate_f(gtab(s), cx * 4 + 2, cz * 4 + 2, temp, rain);
    float n4 = 0.0f, n5 = 0.0f;
#pragma unroll
    for (int o = 0; o < 10; ++o) {
        const float v = octave2f(s.perm + (ST_N4 + o) * PERM_BYTES, axf(s.axis[ST_N4 + o][0][kx]),
                                 axf(s.axis[ST_N4 + o][1][kz])) * static_cast<float>(1 << o);
        n4 = o == 0 ? v : n4 + v;
    }
#pragma unroll
    for (int o = 0; o < 16; ++o) {
        const float v = octave2f(s.perm + (ST_N5 + o) * PERM_BYTES, axf(s.axis[ST_N5 + o][0][kx]),
                                 axf(s.axis[ST_N5 + o][1][kz])) * static_cast<float>(1 << o);
        n5 = o == 0 ? v : n5 + v;
    }
    Fe d5, d7;
    if (column_shape_f(temp, rain, Fe{n4, E_N4}, Fe{n5, E_N5}, d5, d7)) {
        sh[0] = d5.v; sh[1] = d5.e; sh[2] = d7.v; sh[3] = d7.e;
    } else {
        sh[0] = 0.0f; sh[1] = -1.0f; sh[2] = 0.0f; sh[3] = 0.0f;
    }
}

template <int Y0, int N>
__device__ __noinline__ bool screened_range(const CoarseSmem& s, int kx, int kz, const float* shape, unsigned& bits) {
    if (shape[1] < 0.0f) return false;
    float a1[N], a2[N], a3[N];
#pragma unroll 1
    for (int o = 0; o < 16; ++o)
        octave3f<Y0, N>(s.perm + (ST_N2 + o) * PERM_BYTES, axf(s.axis[ST_N2 + o][0][kx]), axf(s.axis[ST_N2 + o][1][kz]),
                        s.yf[o], static_cast<float>(1 << o), a2, o == 0);
#pragma unroll 1
    for (int o = 0; o < 16; ++o)
        octave3f<Y0, N>(s.perm + (ST_N3 + o) * PERM_BYTES, axf(s.axis[ST_N3 + o][0][kx]), axf(s.axis[ST_N3 + o][1][kz]),
                        s.yf[16 + o], static_cast<float>(1 << o), a3, o == 0);
#pragma unroll 1
    for (int o = 0; o < 8; ++o)
        octave3f<Y0, N>(s.perm + (ST_N1 + o) * PERM_BYTES, axf(s.axis[ST_N1 + o][0][kx]), axf(s.axis[ST_N1 + o][1][kz]),
                        s.yf[32 + o], static_cast<float>(1 << o), a1, o == 0);
    const Fe d5{shape[0], shape[1]}, d7{shape[2], shape[3]};
    unsigned b = 0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const int sg = density_sign_f(Y0 + k, d5, d7, a1[k], a2[k], a3[k]);
        if (sg == 0) return false;
        if (sg > 0) b |= 1u << (Y0 + k);
    }
    bits = b;
    return true;
}

__global__ void __launch_bounds__(CT, 1) k_coarse_signs_fast(StateCache cache, const RegionRef* __restrict__ queue,
                                                             const int* count, int maxCount,
                                                             std::uint32_t* __restrict__ signs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CoarseSmem& s = *reinterpret_cast<CoarseSmem*>(smem_raw);
    const int tid = threadIdx.x;
    const int jobs = min(*count, maxCount);
    for (int job = blockIdx.x; job < jobs; job += gridDim.x) {
        const RegionRef ref = queue[job];
        const int originX = -28 + center_chunk_x(ref.center) * 4;
        const int originZ = -28 + center_chunk_z(ref.center) * 4;
        __syncthreads();
        {
            const uint4* src =
                reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(ref.world) * WORLD_PERM_BYTES);
            uint4* dst = reinterpret_cast<uint4*>(s.perm);
            for (int k = tid; k < WORLD_PERM_BYTES / 16; k += CT) dst[k] = src[k];
            const double* o = cache.offsets + static_cast<std::size_t>(ref.world) * WORLD_OFFSETS;
            for (int k = tid; k < ST_COUNT * 3; k += CT) s.off[k / 3][k % 3] = o[(k / 3) * 4 + (k % 3)];
        }
        if (tid == 0) s.fbCount = 0;
        __syncthreads();
        if (tid < OCT3) {
            const int o = tid;
            const int k = o < 16 ? o : (o < 32 ? o - 16 : o - 32);
            const double amp = 1.0 / static_cast<double>(1 << k);
            const double sy = o < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
            build_yaxis(sy, s.off[o][1], s.y64[o]);
            build_yf(s.y64[o], s.yf[o]);
        }
        for (int e = tid; e < NOCT * 2 * SIDE; e += CT) {
            const int o = e / (2 * SIDE), a = (e / SIDE) & 1, k = e % SIDE;
            const double coord = static_cast<double>((a == 0 ? originX : originZ) + k);
            const AxisF ax = make_axis(coord * octave_scale(o), s.off[o][a == 0 ? 0 : 2]);
            s.axis[o][a][k] = AxisS{ax.f, ax.fd, ax.i};
        }
        __syncthreads();
        for (int base = 0; base < COLS; base += TILE) {
            // column shapes (climate + noise4/5) of the tile
            const int g = base + tid;
            s.mask[tid] = 0;
            if (g < COLS) coarse_shape(s, originX, originZ, g / SIDE, g % SIDE, s.shape[tid]);
            __syncthreads();
            // three Y ranges per column
            for (int t = tid; t < TILE * 3; t += CT) {
                const int c = t % TILE, r = t / TILE;
                const int gg = base + c;
                if (gg >= COLS) continue;
                const int kx = gg / SIDE, kz = gg % SIDE;
                unsigned bits = 0;
                bool ok;
                if (r == 0) ok = screened_range<0, 6>(s, kx, kz, s.shape[c], bits);
                else if (r == 1) ok = screened_range<6, 6>(s, kx, kz, s.shape[c], bits);
                else ok = screened_range<12, 5>(s, kx, kz, s.shape[c], bits);
                if (ok) {
                    if (bits) atomicOr(&s.mask[c], bits);
                } else {
                    const int slot = atomicAdd(&s.fbCount, 1);
                    if (slot < FB_CAP) s.fb[slot] = static_cast<std::uint32_t>((r << 16) | c);
                    else atomicOr(&s.mask[c], exact_column(s, originX + kx, originZ + kz, r));
                }
            }
            __syncthreads();
            const int nfb = min(s.fbCount, FB_CAP);
            for (int k = tid; k < nfb; k += CT) {
                const std::uint32_t e = s.fb[k];
                const int c = e & 0xFFFF, r = e >> 16;
                const int gg = base + c;
                atomicOr(&s.mask[c], exact_column(s, originX + gg / SIDE, originZ + gg % SIDE, r));
            }
            __syncthreads();
            if (g < COLS) signs[static_cast<std::size_t>(job) * COLS + g] = s.mask[tid];
            if (tid == 0) s.fbCount = 0;
            __syncthreads();
        }
    }
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

int g_sms = 0;

}  // namespace

void init_coarse_fast() {
    check(cudaFuncSetAttribute(k_coarse_signs_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(CoarseSmem)),
          "coarse fast smem");
    int dev = 0;
    check(cudaGetDevice(&dev), "device");
    check(cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
}

void launch_coarse_signs_fast(const StateCache& cache, const RegionRef* dQueue, const int* dCount, int maxCount,
                              std::uint32_t* dSigns, cudaStream_t stream) {
    if (maxCount <= 0) return;
    const int grid = maxCount < g_sms ? maxCount : g_sms;
    k_coarse_signs_fast<<<grid, CT, sizeof(CoarseSmem), stream>>>(cache, dQueue, dCount, maxCount, dSigns);
    check(cudaGetLastError(), "k_coarse_signs_fast");
}

}  // namespace bsf
