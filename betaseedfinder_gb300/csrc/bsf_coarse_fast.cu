// Screened coarse 61x61x17 lattice signs for sm_103a.
//
// Persistent grid of CTAs (launch shape chosen by the autotuner, 512 threads
// and one CTA per SM on GB300) looping over half-regions (X rows 0..30 and
// 31..60 of each queued region). Per half-region the CTA stages the world's
// generators, the 40 FP32 Y axes and an axis table of its 31 X and 61 Z coarse
// coordinates for the 66 lattice octaves (exact FP64 index / fraction / fade,
// stored as FP32). It then computes every column's shape (climate at block
// 4c+2 + noise4/5) into shared memory and hands out the three Y ranges of the
// columns, 32 tasks at a time, to whichever warp asks next; each task sums the
// 3D octaves in FP32 with error bounds (bsf_screen.cuh) from the largest down
// until its signs are certain. Undecided ranges are recomputed in exact FP64 by
// the warp that met them, so the 17-bit sign masks equal those of the FP64
// coarse kernel bit for bit.
#include "bsf_device.cuh"
#include "bsf_exact_warp.cuh"
#include "bsf_internal.h"
#include "bsf_screen.cuh"

#include <cmath>
#include <cstdio>
#include <stdexcept>

namespace bsf {
namespace {

using namespace screen;

constexpr int SIDE = 61;
constexpr int COLS = SIDE * SIDE;
constexpr int HALF_ROWS = 31;  // X rows of the first half; the second has 30
constexpr int NOCT = 66;
constexpr int HALF_COLS = HALF_ROWS * SIDE;  // columns of the larger half-region

__constant__ float2 cc_octave_scale[NOCT];  // octave_scale(o) split into a float pair

struct CoarseSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    YF yf[OCT3][17];
    float xf[NOCT][HALF_ROWS], xd[NOCT][HALF_ROWS];
    float zf[NOCT][SIDE], zd[NOCT][SIDE];
    std::uint8_t xi[NOCT][HALF_ROWS], zi[NOCT][SIDE];
    float shape[HALF_COLS][4];  // screened column shapes (d5, its bound, d7, its bound; bound < 0: undecided)
    std::uint32_t mask[HALF_COLS];
    std::uint16_t climate[HALF_COLS];  // columns whose d5 needs the climate and noise4
    float4 clim[10];                   // climate generators' offsets as float pairs (climate_split)
    float2 offSplit[NOCT][2];          // the lattice octaves' X (a) and Z (c) offsets as float pairs
    int cursor, screened, fallbacks, climateCount;
};

__device__ __forceinline__ GenTable gtab(const CoarseSmem& s) {
    GenTable t;
    t.perm = s.perm;
    t.off = &s.off[0][0];
    return t;
}

__device__ __forceinline__ double octave_scale(int o) {
    // base / 2^k, the scaling exact either way
    if (o < 16) return NOISE_XZ * exp2_neg(o);
    if (o < 32) return NOISE_XZ * exp2_neg(o - 16);
    if (o < 40) return (NOISE_XZ / 80.0) * exp2_neg(o - 32);
    if (o < 50) return 1.121 * exp2_neg(o - 40);
    return 200.0 * exp2_neg(o - 50);
}

__device__ __forceinline__ AxisF ax_x(const CoarseSmem& s, int o, int k) {
    const float f = s.xf[o][k];
    return AxisF{f, f - 1.0f, s.xd[o][k], s.xi[o][k]};
}
__device__ __forceinline__ AxisF ax_z(const CoarseSmem& s, int o, int k) {
    const float f = s.zf[o][k];
    return AxisF{f, f - 1.0f, s.zd[o][k], s.zi[o][k]};
}

// Exact FP64 column for Y range r by one whole warp (fallback pass).
__device__ __noinline__ unsigned exact_column_w(const CoarseSmem& s, int cx, int cz, int r) {
    // level 16 is air
    const int y0 = r == 0 ? 0 : (r == 1 ? 6 : 12), n = r == 2 ? TOP_SOLID_LEVEL - 11 : 6;
    return exactwarp::exact_column_warp(s, cx, cz, y0, n);
}


// Column shape (BetaTerrain173.java:739-804) in FP32 with bounds, in two
// passes; kx is the half-local row. The first takes noise5 and the d6/d7 half
// (shape_d7_f) of every column and reports whether d5 needs the climate: in the
// reference's d6 < 0 branch d5 is 0.5 whatever the climate and noise4 are. The
// second pass computes them for the compacted list of the other columns only,
// so the climate's simplex octaves run on full warps.
__device__ __noinline__ bool coarse_shape_first(const CoarseSmem& s, int kx, int kz, float* sh) {
    float n5 = 0.0f;
#pragma unroll 1  // rolled: the unrolled octaves overflow the instruction cache
    for (int o = 0; o < 16; ++o) {
        const float v = octave2f(s.perm + (ST_N5 + o) * PERM_BYTES, ax_x(s, ST_N5 + o, kx), ax_z(s, ST_N5 + o, kz)) *
                        static_cast<float>(1 << o);
        n5 = o == 0 ? v : n5 + v;
    }
    Fe d7{0.0f, 0.0f};
    bool zeroD5 = false;
    if (!shape_d7_f(Fe{n5, E_N5}, d7, zeroD5)) {
        sh[0] = 0.0f; sh[1] = -1.0f; sh[2] = 0.0f; sh[3] = 0.0f;
        return false;
    }
    sh[0] = 0.5f; sh[1] = 0.0f; sh[2] = d7.v; sh[3] = d7.e;
    return !zeroD5;
}

__device__ __noinline__ void coarse_shape_climate(const CoarseSmem& s, int cx, int cz, int kx, int kz, float* sh) {
    Fe temp, rain;
    climate_f(gtab(s), s.clim, cx * 4 + 2, cz * 4 + 2, temp, rain);
    float n4 = 0.0f;
#pragma unroll 1
    for (int o = 0; o < 10; ++o) {
        const float v = octave2f(s.perm + (ST_N4 + o) * PERM_BYTES, ax_x(s, ST_N4 + o, kx),
                                 ax_z(s, ST_N4 + o, kz)) * static_cast<float>(1 << o);
        n4 = o == 0 ? v : n4 + v;
    }
    const Fe d5 = shape_d5_f(temp, rain, Fe{n4, E_N4});
    sh[0] = d5.v;
    sh[1] = d5.e;
}

// Screened signs of levels [y0, y0 + n), n <= 6, from the column's shape; one
// instantiation for all three level ranges (three had thrashed the instruction
// cache whenever warps worked on different ranges).
__device__ __noinline__ bool screened_range(const CoarseSmem& s, int kx, int kz, const float* shape, int y0, int n,
                                            unsigned& bits) {
    if (shape[1] < 0.0f) return false;
    auto oct = [&](int st, int o, float* v) {  // state st's octave o (st is also its Y-table index)
        octave3f_y<6>(s.perm + st * PERM_BYTES, ax_x(s, st, kx), ax_z(s, st, kz), s.yf[st], y0,
                      static_cast<float>(1 << o), v);
    };
    return progressive_signs<6>(y0, n, Fe{shape[0], shape[1]}, Fe{shape[2], shape[3]}, oct, bits);
}

// CT threads per CTA, MINB CTAs per SM: chosen by the autotuner.
template <int CT, int MINB>
__global__ void __launch_bounds__(CT, MINB) k_coarse_signs_fast(StateCache cache, const RegionRef* __restrict__ queue,
                                                             const int* count, int maxCount,
                                                             std::uint32_t* __restrict__ signs,
                                                             unsigned long long* stats, int forceExact) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CoarseSmem& s = *reinterpret_cast<CoarseSmem*>(smem_raw);
    const int tid = threadIdx.x;
    const int jobs = min(*count, maxCount);
    if (tid == 0) { s.screened = 0; s.fallbacks = 0; s.climateCount = 0; }
    for (int item = blockIdx.x; item < jobs * 2; item += gridDim.x) {
        const int job = item >> 1, half = item & 1;
        const RegionRef ref = queue[job];
        const int row0 = half == 0 ? 0 : HALF_ROWS;
        const int rows = half == 0 ? HALF_ROWS : SIDE - HALF_ROWS;
        const int originX = -28 + center_chunk_x(ref.center) * 4;
        const int originZ = -28 + center_chunk_z(ref.center) * 4;
        __syncthreads();
        {
            const uint4* src =
                reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(ref.world) * WORLD_PERM_BYTES);
            uint4* dst = reinterpret_cast<uint4*>(s.perm);
            for (int k = tid; k < WORLD_PERM_BYTES / 16; k += CT) dst[k] = src[k];
            const double* o = cache.offsets + static_cast<std::size_t>(ref.world) * WORLD_OFFSETS;
            for (int k = tid; k < ST_COUNT * 3; k += CT) {
                const double v = o[(k / 3) * 4 + (k % 3)];
                s.off[k / 3][k % 3] = v;
                if (k / 3 < NOCT && k % 3 != 1) {
                    const DF d = df_of(v);
                    s.offSplit[k / 3][(k % 3) / 2] = make_float2(d.h, d.l);
                }
            }
        }
        __syncthreads();
        if (tid < OCT3) {
            const int o = tid;
            const int k = o < 16 ? o : (o < 32 ? o - 16 : o - 32);
            const double amp = exp2_neg(k);
            const double sy = o < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
            YEntry ya[17];
            build_yaxis(sy, s.off[o][1], ya);
            build_yf(ya, s.yf[o]);
        } else if (tid < OCT3 + 10) {
            s.clim[tid - OCT3] = climate_split(s.off[ST_TEMP + tid - OCT3]);
        }
        for (int e = tid; e < NOCT * (rows + SIDE); e += CT) {
            const int o = e / (rows + SIDE), k = e % (rows + SIDE);
            // double-float entries (bsf_screen.cuh make_axis_df), FP64 where a floor is too close to call
            const float2 sc = cc_octave_scale[o];
            if (k < rows) {
                const int coord = originX + row0 + k;
                const float2 of = s.offSplit[o][0];
                AxisF ax;
                if (!make_axis_df(coord, DF{sc.x, sc.y}, DF{of.x, of.y}, ax))
                    ax = make_axis(static_cast<double>(coord) * octave_scale(o), s.off[o][0]);
                s.xf[o][k] = ax.f;
                s.xd[o][k] = ax.fd;
                s.xi[o][k] = static_cast<std::uint8_t>(ax.i);
            } else {
                const int kz = k - rows;
                const int coord = originZ + kz;
                const float2 of = s.offSplit[o][1];
                AxisF az;
                if (!make_axis_df(coord, DF{sc.x, sc.y}, DF{of.x, of.y}, az))
                    az = make_axis(static_cast<double>(coord) * octave_scale(o), s.off[o][2]);
                s.zf[o][kz] = az.f;
                s.zd[o][kz] = az.fd;
                s.zi[o][kz] = static_cast<std::uint8_t>(az.i);
            }
        }
        __syncthreads();
        // Shapes of the half-region's columns first (kept in smem), then its
        // 3 x cols column-range tasks handed out 32 at a time: a screened task
        // stops once its signs are certain, so costs vary, and a fixed split
        // would leave the CTA waiting for its slowest warp at every barrier.
        const int cols = rows * SIDE;
        const int lane0 = tid & 31;
        for (int base = 0; base < cols; base += CT) {
            const int g = base + tid;
            bool need = false;
            if (g < cols) {
                need = coarse_shape_first(s, g / SIDE, g % SIDE, s.shape[g]);
                s.mask[g] = 0;
            }
            const unsigned vote = __ballot_sync(0xffffffffu, need);
            int slot = 0;
            if (lane0 == 0 && vote) slot = atomicAdd(&s.climateCount, __popc(vote));
            slot = __shfl_sync(0xffffffffu, slot, 0);
            if (need) s.climate[slot + __popc(vote & ((1u << lane0) - 1u))] = static_cast<std::uint16_t>(g);
        }
        if (tid == 0) s.cursor = 0;
        __syncthreads();
        {
            const int m = s.climateCount;
            for (int j = tid; j < m; j += CT) {
                const int g = s.climate[j];
                const int kx = g / SIDE, kz = g % SIDE;
                coarse_shape_climate(s, originX + row0 + kx, originZ + kz, kx, kz, s.shape[g]);
            }
        }
        __syncthreads();
        if (tid == 0) s.climateCount = 0;
        // chunk b: range b / chunks of columns (b % chunks) * 32 + lane. Range-major, so
        // the warps run one range's code at a time (three at once overflow the
        // instruction cache).
        const int chunks = (cols + 31) >> 5;
        const int total = chunks * 3 * 32;
        // returns the task's column range left undecided (r << 11 | column), or -1
        auto task = [&](int t) -> int {
            const int b = t >> 5, r = b / chunks;
            const int c = (b % chunks) * 32 + (t & 31);
            if (c >= cols) return -1;
            const int kx = c / SIDE, kz = c % SIDE;
            atomicAdd(&s.screened, 1);
            unsigned bits = 0;
            bool ok;
            if (forceExact) ok = false;
            else ok = screened_range(s, kx, kz, s.shape[c], r * 6, r == 2 ? TOP_SOLID_LEVEL - 11 : 6, bits);  // 16 is air
            if (ok) {
                if (bits) atomicOr(&s.mask[c], bits);
                return -1;
            }
            atomicAdd(&s.fallbacks, 1);
            return (r << 11) | c;
        };
        // Undecided column ranges are resolved right away by the warp that met
        // them, all 32 lanes on one column, while the other warps go on claiming.
        const int lane = tid & 31;
        for (;;) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&s.cursor, 32);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= total) break;
            const int e = base + lane < total ? task(base + lane) : -1;
            unsigned todo = __ballot_sync(0xffffffffu, e >= 0);
            while (todo) {
                const int src = __ffs(todo) - 1;
                todo &= todo - 1;
                const int f = __shfl_sync(0xffffffffu, e, src);
                const int c = f & 0x7FF, r = f >> 11;
                const unsigned bits = exact_column_w(s, originX + row0 + c / SIDE, originZ + c % SIDE, r);
                if (lane == 0) atomicOr(&s.mask[c], bits);
            }
        }
        __syncthreads();
        for (int g = tid; g < cols; g += CT)
            signs[static_cast<std::size_t>(job) * COLS + static_cast<std::size_t>(row0) * SIDE + g] = s.mask[g];
    }
    __syncthreads();
    if (tid == 0 && stats) {
        atomicAdd(&stats[2], static_cast<unsigned long long>(s.screened));
        atomicAdd(&stats[3], static_cast<unsigned long long>(s.fallbacks));
    }
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

struct Variant {
    const char* name;
    int threads;
    void (*kernel)(StateCache, const RegionRef*, const int*, int, std::uint32_t*, unsigned long long*, int);
    int grid;
};
Variant g_variants[] = {
    // 640 threads at 96 registers (some spills) hide latency better than 512 at
    // 128 (Stage0: 37.65 vs 38.72 ms per 16,384 worlds); it is the default
    {"640x1", 640, k_coarse_signs_fast<640, 1>, 0},
    {"512x1", 512, k_coarse_signs_fast<512, 1>, 0},
    {"256x2", 256, k_coarse_signs_fast<256, 2>, 0},
    {"384x1", 384, k_coarse_signs_fast<384, 1>, 0},
};
constexpr int kVariants = sizeof(g_variants) / sizeof(g_variants[0]);
int g_variant = 0;

}  // namespace

int coarse_fast_variants() { return kVariants; }
const char* coarse_fast_variant_name(int v) { return g_variants[v].name; }
void set_coarse_fast_variant(int v) { g_variant = (v >= 0 && v < kVariants) ? v : 0; }
int get_coarse_fast_variant() { return g_variant; }

void init_coarse_fast() {
    float2 scales[NOCT];
    for (int o = 0; o < NOCT; ++o) {  // octave_scale(o) in the same IEEE operations as the device
        const double base = o < 32 ? NOISE_XZ : (o < 40 ? NOISE_XZ / 80.0 : (o < 50 ? 1.121 : 200.0));
        const int k = o < 16 ? o : (o < 32 ? o - 16 : (o < 40 ? o - 32 : (o < 50 ? o - 40 : o - 50)));
        const double v = base * std::ldexp(1.0, -k);
        const float h = static_cast<float>(v);
        scales[o] = make_float2(h, static_cast<float>(v - static_cast<double>(h)));
    }
    check(cudaMemcpyToSymbol(cc_octave_scale, scales, sizeof(scales)), "octave scales");
    int dev = 0, sms = 0;
    check(cudaGetDevice(&dev), "device");
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
    for (Variant& v : g_variants) {
        check(cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(CoarseSmem)),
              "coarse fast smem");
        int perSm = 0;
        check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, v.kernel, v.threads, sizeof(CoarseSmem)),
              "occupancy");
        v.grid = sms * (perSm > 0 ? perSm : 1);
    }
}

void launch_coarse_signs_fast(const StateCache& cache, const RegionRef* dQueue, const int* dCount, int maxCount,
                              std::uint32_t* dSigns, unsigned long long* stats, cudaStream_t stream,
                              bool persistent, bool forceExact) {
    if (maxCount <= 0) return;
    const Variant& v = g_variants[g_variant];
    // one CTA per half-region of the queue's capacity; CTAs past the device-side count exit at once
    const int grid = (!persistent || 2 * maxCount < v.grid) ? 2 * maxCount : v.grid;
    v.kernel<<<grid, v.threads, sizeof(CoarseSmem), stream>>>(cache, dQueue, dCount, maxCount, dSigns, stats,
                                                              forceExact ? 1 : 0);
    check(cudaGetLastError(), "k_coarse_signs_fast");
}

}  // namespace bsf
