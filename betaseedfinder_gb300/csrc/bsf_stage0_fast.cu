// Screened Stage0 (P20 -> Upper -> Lower) + P19 for sm_103a.
//
// Persistent grid, one 512-thread CTA per SM looping over worlds. Per world the
// CTA stages in shared memory: the 76 generators, the FP64 and FP32 Y axes of
// the 40 3D octaves, and an axis table holding, for each of the 66 lattice
// octaves (40 3D + 26 2D), the exact lattice index / fraction / fade of the 46
// distinct X and 46 distinct Z coarse coordinates that the 8 region centres
// use (X = -88..92 step 4). Every column task then runs its octaves in FP32
// (bsf_screen.cuh) and only columns whose density signs are not decided by the
// error bound are recomputed in exact FP64, so the masks, counts and P19
// outputs are bit-identical to the exact kernel (bsf_stage0.cu).
#include "bsf_device.cuh"
#include "bsf_internal.h"
#include "bsf_screen.cuh"

#include <cstdio>
#include <stdexcept>

namespace bsf {

#include "p19_table.inc"

namespace {

using namespace screen;

constexpr int FT = 512;          // threads per CTA
constexpr int NAX = 46;          // distinct coarse coordinates per axis over the 8 centres
constexpr int NOCT = 66;         // 40 3D + 26 2D lattice octaves (state index == octave index)
constexpr int FB_CAP = 1024;     // exact-fallback list entries

__constant__ unsigned char cf_axis[8] = {0, 2, 5, 7, 8, 10, 13, 15};
__constant__ unsigned char cf_nonaxis_cols[192];
__constant__ signed char cf_p19_feature[BSF_P19_NODE_COUNT];
__constant__ short cf_p19_left[BSF_P19_NODE_COUNT];
__constant__ short cf_p19_right[BSF_P19_NODE_COUNT];
__constant__ double cf_p19_value[BSF_P19_NODE_COUNT];
__constant__ short cf_p19_root[BSF_P19_TREE_COUNT];

struct AxisS {
    float f, fd;
    int i;
};

struct FastSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    YEntry y64[OCT3][17];
    YF yf[OCT3][17];
    AxisS axis[NOCT][2][NAX];
    float shape[8][256][4];  // d5.v, d5.e, d7.v, d7.e; d5.e < 0 marks an undecided column shape
    std::uint32_t mask17[8][256];
    std::uint16_t tasks[8 * 256];
    std::uint32_t fb[FB_CAP];
    int p20[8], upper[8], high[8], gate[8];
    int taskCount, fbCount;
    int feat[8][12];
    int evalMask;
};

__device__ __forceinline__ GenTable gtab(const FastSmem& s) {
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

__device__ void load_world_fast(FastSmem& s, const StateCache& cache, int world) {
    const uint4* src = reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(world) * WORLD_PERM_BYTES);
    uint4* dst = reinterpret_cast<uint4*>(s.perm);
    for (int k = threadIdx.x; k < WORLD_PERM_BYTES / 16; k += blockDim.x) dst[k] = src[k];
    const double* o = cache.offsets + static_cast<std::size_t>(world) * WORLD_OFFSETS;
    for (int k = threadIdx.x; k < ST_COUNT * 3; k += blockDim.x) s.off[k / 3][k % 3] = o[(k / 3) * 4 + (k % 3)];
}

// Exact FP64 column pieces for the fallback path.
__device__ void noise45_exact(const GenTable& t, double X, double Z, double& n4, double& n5) {
    double amp = 1.0, acc = 0.0;
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

template <int Y0, int N>
__device__ unsigned exact_bits(const FastSmem& s, double X, double Z, double d5, double d7) {
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

// Exact column (FP64) for Y range id r: 0 -> [11,17), 1 -> [0,6), 2 -> [6,11).
__device__ __noinline__ unsigned exact_task(const FastSmem& s, int c, int col, int r) {
    const int ix = col >> 4, iz = col & 15;
    const int cx = -28 + ix * 4 + center_chunk_x(c) * 4;
    const int cz = -28 + iz * 4 + center_chunk_z(c) * 4;
    const GenTable t = gtab(s);
    double temp, rain, n4, n5, d5, d7;
    climate_at(t, cx * 4 + 2, cz * 4 + 2, temp, rain);
    const double X = static_cast<double>(cx), Z = static_cast<double>(cz);
    noise45_exact(t, X, Z, n4, n5);
    column_shape(temp, rain, n4, n5, d5, d7);
    if (r == 0) return exact_bits<11, 6>(s, X, Z, d5, d7);
    if (r == 1) return exact_bits<0, 6>(s, X, Z, d5, d7);
    return exact_bits<6, 5>(s, X, Z, d5, d7);
}

// Screened column shape: climate + noise4/5 in FP32 with bounds.
__device__ __noinline__ void screened_shape(const FastSmem& s, int c, int col, float* out4) {
    const int ix = col >> 4, iz = col & 15;
    const int cx = -28 + ix * 4 + center_chunk_x(c) * 4;
    const int cz = -28 + iz * 4 + center_chunk_z(c) * 4;
    const int kx = ix + center_chunk_x(c) + 15, kz = iz + center_chunk_z(c) + 15;
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
        out4[0] = d5.v; out4[1] = d5.e; out4[2] = d7.v; out4[3] = d7.e;
    } else {
        out4[0] = 0.0f; out4[1] = -1.0f; out4[2] = 0.0f; out4[3] = 0.0f;
    }
}

// Screened density signs of one column for levels [Y0, Y0+N); returns false when undecided.
template <int Y0, int N>
__device__ __noinline__ bool screened_bits(const FastSmem& s, int c, int col, const float* shape, unsigned& bits) {
    if (shape[1] < 0.0f) return false;
    const int kx = (col >> 4) + center_chunk_x(c) + 15, kz = (col & 15) + center_chunk_z(c) + 15;
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

__device__ void push_fallback(FastSmem& s, int c, int col, int r) {
    const int slot = atomicAdd(&s.fbCount, 1);
    const std::uint32_t e = static_cast<std::uint32_t>((r << 12) | (c << 8) | col);
    if (slot < FB_CAP) {
        s.fb[slot] = e;
    } else {
        // list full: decide this column right here with the exact path
        atomicOr(&s.mask17[c][col], exact_task(s, c, col, r));
    }
}

__device__ void run_fallbacks(FastSmem& s) {
    __syncthreads();
    const int n = min(s.fbCount, FB_CAP);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const std::uint32_t e = s.fb[k];
        const int r = e >> 12, c = (e >> 8) & 15, col = e & 255;
        atomicOr(&s.mask17[c][col], exact_task(s, c, col, r));
    }
    __syncthreads();
    if (threadIdx.x == 0) s.fbCount = 0;
    __syncthreads();
}

// ---- P19 (same as the exact kernel) ---------------------------------------
__device__ __noinline__ void shape_stats(const std::uint8_t* grid, std::uint8_t* visited, std::uint16_t* queue, int& largestOut,
                            int& widthOut, int& depthOut, int& touchesOut) {
    for (int i = 0; i < 256; ++i) visited[i] = 0;
    int largest = 0, minX = 16, maxX = -1, minZ = 16, maxZ = -1, touches = 0;
    for (int x = 0; x < 16; ++x) {
        for (int z = 0; z < 16; ++z) {
            const int index = x * 16 + z;
            if (grid[index] == 0) continue;
            minX = min(minX, x);
            maxX = max(maxX, x);
            minZ = min(minZ, z);
            maxZ = max(maxZ, z);
            if (x == 0 || z == 0 || x == 15 || z == 15) touches = 1;
            if (visited[index]) continue;
            int head = 0, tail = 0, cluster = 0;
            visited[index] = 1;
            queue[tail++] = static_cast<std::uint16_t>(index);
            while (head < tail) {
                const int cur = queue[head++];
                ++cluster;
                const int cx = cur >> 4, cz = cur & 15;
                const int nx[4] = {cx - 1, cx + 1, cx, cx};
                const int nz[4] = {cz, cz, cz - 1, cz + 1};
                for (int k = 0; k < 4; ++k) {
                    if (nx[k] < 0 || nz[k] < 0 || nx[k] >= 16 || nz[k] >= 16) continue;
                    const int nb = nx[k] * 16 + nz[k];
                    if (grid[nb] == 0 || visited[nb]) continue;
                    visited[nb] = 1;
                    queue[tail++] = static_cast<std::uint16_t>(nb);
                }
            }
            largest = max(largest, cluster);
        }
    }
    largestOut = largest;
    widthOut = largest == 0 ? 0 : maxX - minX + 1;
    depthOut = largest == 0 ? 0 : maxZ - minZ + 1;
    touchesOut = touches;
}

__device__ double p19_feature(int id, int scout, const int* f) {
    const double EPS = BSF_P19_EPSILON;
    switch (id) {
        case 0: return static_cast<double>(scout);
        case 1: return static_cast<double>(f[0]);
        case 2: return static_cast<double>(f[1]);
        case 3: return static_cast<double>(f[2]);
        case 4: return static_cast<double>(f[3]);
        case 5: return static_cast<double>(f[4]);
        case 6: return static_cast<double>(f[5]);
        case 7: return static_cast<double>(f[6]);
        case 8: return static_cast<double>(f[7]);
        case 9: return static_cast<double>(f[8]);
        case 10: return static_cast<double>(f[9]);
        case 11: return static_cast<double>(f[0]) / (static_cast<double>(scout) + EPS);
        case 12: return static_cast<double>(f[5] + f[6] + f[8] + f[9]);
        case 13: return static_cast<double>(f[8] * f[9]);
        case 14: return static_cast<double>(f[5] * f[6]);
        case 15: return static_cast<double>(f[4]) / (static_cast<double>(f[0]) + EPS);
        case 16: return static_cast<double>(f[1] + f[2] + f[3]);
        case 17: return static_cast<double>(f[7]) / (static_cast<double>(f[1]) + EPS);
        case 18: return static_cast<double>(f[2]) / (static_cast<double>(f[1]) + EPS);
        case 19: return static_cast<double>(f[1]) / (static_cast<double>(f[0]) + EPS);
        default: return static_cast<double>(f[4] + f[7]);
    }
}

__device__ __noinline__ double p19_score(int scout, const int* f) {
    double sum = 0.0;
    for (int t = 0; t < BSF_P19_TREE_COUNT; ++t) {
        int nd = cf_p19_root[t];
        for (int depth = 0; depth < 64 && cf_p19_feature[nd] >= 0; ++depth) {
            const double v = p19_feature(cf_p19_feature[nd], scout, f);
            nd = v <= cf_p19_value[nd] ? cf_p19_left[nd] : cf_p19_right[nd];
        }
        sum = t == 0 ? cf_p19_value[nd] : sum + cf_p19_value[nd];
    }
    return sum / static_cast<double>(BSF_P19_TREE_COUNT);
}

__device__ __forceinline__ int highest_reentry(std::uint32_t mask) {
    bool sawPos = false, sawGap = false;
    int highest = -1;
    for (int y = 0; y < 17; ++y) {
        if ((mask >> y) & 1u) {
            if (sawPos && sawGap) highest = y;
            sawPos = true;
        } else if (sawPos) {
            sawGap = true;
        }
    }
    return highest;
}

__global__ void __launch_bounds__(FT, 1) k_stage0_fast(StateCache cache, int n, int centers, Profile prof,
                                                       RegionInfo* __restrict__ regions,
                                                       RegionRef* __restrict__ coarseQueue, int* coarseCount,
                                                       int coarseCapacity, int* fallbackStat) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FastSmem& s = *reinterpret_cast<FastSmem*>(smem_raw);
    const int tid = threadIdx.x;
    for (int world = blockIdx.x; world < n; world += gridDim.x) {
        __syncthreads();
        load_world_fast(s, cache, world);
        if (tid < 8) { s.p20[tid] = 0; s.upper[tid] = 0; s.high[tid] = 0; }
        if (tid == 0) { s.fbCount = 0; s.taskCount = 0; }
        for (int k = tid; k < 8 * 256; k += FT) (&s.mask17[0][0])[k] = 0;
        __syncthreads();
        if (tid < OCT3) {
            const int o = tid;
            const int k = o < 16 ? o : (o < 32 ? o - 16 : o - 32);
            const double amp = 1.0 / static_cast<double>(1 << k);
            const double sy = o < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
            build_yaxis(sy, s.off[o][1], s.y64[o]);
            build_yf(s.y64[o], s.yf[o]);
        }
        // Axis table: octave o, axis a (0 = x with offset a, 1 = z with offset c), coordinate -88 + 4k.
        for (int e = tid; e < NOCT * 2 * NAX; e += FT) {
            const int o = e / (2 * NAX), a = (e / NAX) & 1, k = e % NAX;
            const double coord = static_cast<double>(-88 + 4 * k);
            const AxisF ax = make_axis(coord * octave_scale(o), s.off[o][a == 0 ? 0 : 2]);
            s.axis[o][a][k] = AxisS{ax.f, ax.fd, ax.i};
        }
        __syncthreads();

        // P20: the 8x8 axis columns of every centre.
        for (int t = tid; t < centers * 64; t += FT) {
            const int c = t >> 6, k = t & 63;
            const int col = cf_axis[k >> 3] * 16 + cf_axis[k & 7];
            float* sh = s.shape[c][col];
            screened_shape(s, c, col, sh);
            unsigned bits;
            if (screened_bits<11, 6>(s, c, col, sh, bits)) s.mask17[c][col] = bits;
            else push_fallback(s, c, col, 0);
        }
        run_fallbacks(s);
        for (int t = tid; t < centers * 64; t += FT) {
            const int c = t >> 6, k = t & 63;
            if (s.mask17[c][cf_axis[k >> 3] * 16 + cf_axis[k & 7]]) atomicAdd(&s.p20[c], 1);
        }
        __syncthreads();
        if (tid == 0) {
            int nt = 0;
            for (int c = 0; c < centers; ++c) {
                const int g = prof.p20MinCount > 1 ? (s.p20[c] >= prof.p20MinCount ? s.p20[c] : 0) : s.p20[c];
                s.gate[c] = g;
                s.upper[c] = g;
                if (g > 0) s.tasks[nt++] = static_cast<std::uint16_t>(c);
            }
            s.taskCount = nt;
        }
        __syncthreads();
        const int upperCenters = s.taskCount;
        for (int t = tid; t < upperCenters * 192; t += FT) {
            const int c = s.tasks[t / 192];
            const int col = cf_nonaxis_cols[t % 192];
            float* sh = s.shape[c][col];
            screened_shape(s, c, col, sh);
            unsigned bits;
            if (screened_bits<11, 6>(s, c, col, sh, bits)) s.mask17[c][col] = bits;
            else push_fallback(s, c, col, 0);
        }
        run_fallbacks(s);
        for (int t = tid; t < upperCenters * 192; t += FT) {
            const int c = s.tasks[t / 192];
            if (s.mask17[c][cf_nonaxis_cols[t % 192]]) atomicAdd(&s.upper[c], 1);
        }
        __syncthreads();
        if (tid == 0) s.taskCount = 0;
        __syncthreads();
        for (int t = tid; t < centers * 256; t += FT) {
            const int c = t >> 8, col = t & 255;
            if (s.gate[c] > 0 && s.upper[c] >= prof.upperMinCount && s.mask17[c][col] != 0) {
                const int slot = atomicAdd(&s.taskCount, 1);
                s.tasks[slot] = static_cast<std::uint16_t>((c << 8) | col);
            }
        }
        __syncthreads();
        const int lowerTasks = s.taskCount * 2;
        for (int t = tid; t < lowerTasks; t += FT) {
            const int e = s.tasks[t >> 1];
            const int c = e >> 8, col = e & 255;
            const float* sh = s.shape[c][col];
            unsigned bits;
            bool ok;
            if (t & 1) ok = screened_bits<6, 5>(s, c, col, sh, bits);
            else ok = screened_bits<0, 6>(s, c, col, sh, bits);
            if (ok) {
                if (bits) atomicOr(&s.mask17[c][col], bits);
            } else {
                push_fallback(s, c, col, (t & 1) ? 2 : 1);
            }
        }
        run_fallbacks(s);
        // highest re-entry per lower column (reuse the fallback list as an 8x256 byte array)
        std::uint8_t* highest = reinterpret_cast<std::uint8_t*>(&s.shape[0][0][0]);
        __syncthreads();
        for (int k = tid; k < 8 * 256; k += FT) highest[k] = 0xFF;
        __syncthreads();
        for (int t = tid; t < s.taskCount; t += FT) {
            const int e = s.tasks[t];
            const int c = e >> 8, col = e & 255;
            const int h = highest_reentry(s.mask17[c][col]);
            highest[c * 256 + col] = h < 0 ? 0xFF : static_cast<std::uint8_t>(h);
            if (h >= 11) atomicAdd(&s.high[c], 1);
        }
        __syncthreads();
        std::uint8_t* scratch = reinterpret_cast<std::uint8_t*>(&s.axis[0][0][0]);  // 36 KB, axis table done
        if (tid == 0) {
            int m = 0;
            for (int c = 0; c < centers; ++c)
                if (s.p20[c] >= prof.p20MinCount && s.upper[c] >= prof.upperMinCount && s.high[c] >= prof.highMinCount)
                    m |= 1 << c;
            s.evalMask = m;
        }
        __syncthreads();
        if (tid < 16) {
            const int c = tid >> 1, which = tid & 1;
            if (c < centers && ((s.evalMask >> c) & 1)) {
                std::uint8_t* grid = scratch + tid * 1024;
                std::uint8_t* visited = grid + 256;
                std::uint16_t* queue = reinterpret_cast<std::uint16_t*>(grid + 512);
                int full[4] = {0, 0, 0, 0};
                for (int col = 0; col < 256; ++col) {
                    const int e = highest[c * 256 + col];
                    const int h = e == 0xFF ? -1 : e;
                    grid[col] = which == 0 ? (h >= 11) : (h >= 12);
                    if (h >= 11) ++full[0];
                    if (h >= 12) ++full[1];
                    if (h >= 13) ++full[2];
                    if (h >= 14) ++full[3];
                }
                int L, W, D, T;
                shape_stats(grid, visited, queue, L, W, D, T);
                if (which == 0) {
                    s.feat[c][0] = full[0]; s.feat[c][1] = full[1]; s.feat[c][2] = full[2]; s.feat[c][3] = full[3];
                    s.feat[c][4] = L; s.feat[c][5] = W; s.feat[c][6] = D; s.feat[c][10] = T;
                } else {
                    s.feat[c][7] = L; s.feat[c][8] = W; s.feat[c][9] = D; s.feat[c][11] = T;
                }
            }
        }
        __syncthreads();
        if (tid < centers) {
            const int c = tid;
            RegionInfo r;
            r.p19Score = __longlong_as_double(0x7ff8000000000000LL);
            r.coarse = 0;
            r.p20 = static_cast<std::int16_t>(s.p20[c]);
            r.upper = static_cast<std::int16_t>(s.upper[c]);
            r.high = static_cast<std::int16_t>(s.high[c]);
            r.p19Evaluated = 0; r.p19Pass = 0; r.p19Extreme = 0; r.megaReject = 0; r.coarseEvaluated = 0; r.pad0 = 0;
            r.fullY88 = r.fullY96 = r.fullY104 = r.fullY112 = r.y88Largest = r.y96Largest = 0;
            r.y88Width = r.y88Depth = r.y88Touches = r.y96Width = r.y96Depth = r.y96Touches = 0;
            r.pad1[0] = r.pad1[1] = 0;
            if ((s.evalMask >> c) & 1) {
                const int* f = s.feat[c];
                const double score = p19_score(s.upper[c], f);
                const bool extreme = f[4] >= 14 || f[7] >= 14;
                const bool pass = extreme || score >= prof.p19MinScore;
                const bool mega = pass && prof.megaTopologyFilter && !extreme && score < 5.0 && (f[3] == 0 || f[7] < 4);
                r.p19Evaluated = 1;
                r.p19Score = score;
                r.p19Pass = pass;
                r.p19Extreme = extreme;
                r.megaReject = mega;
                r.fullY88 = f[0]; r.fullY96 = f[1]; r.fullY104 = f[2]; r.fullY112 = f[3];
                r.y88Largest = f[4]; r.y88Width = f[5]; r.y88Depth = f[6]; r.y88Touches = f[10];
                r.y96Largest = f[7]; r.y96Width = f[8]; r.y96Depth = f[9]; r.y96Touches = f[11];
                if (pass && !mega && coarseQueue != nullptr) {
                    const int slot = atomicAdd(coarseCount, 1);
                    if (slot < coarseCapacity) coarseQueue[slot] = RegionRef{world, c};
                }
            }
            regions[static_cast<std::size_t>(world) * centers + c] = r;
        }
        if (tid == 0 && fallbackStat) atomicAdd(fallbackStat, 0);
    }
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

int g_grid = 0;

}  // namespace

void init_stage0_fast() {
    check(cudaMemcpyToSymbol(cf_p19_feature, bsf_p19_feature, sizeof(bsf_p19_feature)), "p19");
    check(cudaMemcpyToSymbol(cf_p19_left, bsf_p19_left, sizeof(bsf_p19_left)), "p19");
    check(cudaMemcpyToSymbol(cf_p19_right, bsf_p19_right, sizeof(bsf_p19_right)), "p19");
    check(cudaMemcpyToSymbol(cf_p19_value, bsf_p19_value, sizeof(bsf_p19_value)), "p19");
    check(cudaMemcpyToSymbol(cf_p19_root, bsf_p19_root, sizeof(bsf_p19_root)), "p19");
    unsigned char cols[192];
    int k = 0;
    auto isAxis = [](int i) { return i == 0 || i == 2 || i == 5 || i == 7 || i == 8 || i == 10 || i == 13 || i == 15; };
    for (int ix = 0; ix < 16; ++ix)
        for (int iz = 0; iz < 16; ++iz)
            if (!(isAxis(ix) && isAxis(iz))) cols[k++] = static_cast<unsigned char>(ix * 16 + iz);
    check(cudaMemcpyToSymbol(cf_nonaxis_cols, cols, sizeof(cols)), "columns");
    check(cudaFuncSetAttribute(k_stage0_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(FastSmem)),
          "stage0 fast smem");
    int dev = 0, sms = 0;
    check(cudaGetDevice(&dev), "device");
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
    g_grid = sms;
}

std::size_t stage0_fast_smem() { return sizeof(FastSmem); }

void launch_stage0_fast(const StateCache& cache, int n, int centers, const Profile& prof, RegionInfo* dRegions,
                        RegionRef* dCoarseQueue, int* dCoarseCount, int coarseCapacity, cudaStream_t stream) {
    if (n <= 0) return;
    const int grid = n < g_grid ? n : g_grid;
    k_stage0_fast<<<grid, FT, sizeof(FastSmem), stream>>>(cache, n, centers, prof, dRegions, dCoarseQueue,
                                                          dCoarseCount, coarseCapacity, nullptr);
    check(cudaGetLastError(), "k_stage0_fast");
}

}  // namespace bsf
