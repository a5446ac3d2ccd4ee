// World generator setup, Stage0 (P20 -> Upper -> Lower) + P19 gate, and the
// single-chunk terrain bitmap kernel, for sm_103a.
//
// Layout: one CTA per world. All 76 generator states of the world (19.5 KB of
// byte permutations + offsets) and the Y axes of its 40 3D octaves are staged
// in shared memory once; every (centre, column, Y range) task then reads them
// without further synchronisation.
#include "bsf_device.cuh"
#include "bsf_internal.h"

#include <cmath>
#include <cstdio>
#include <stdexcept>

namespace bsf {

#include "p19_table.inc"

namespace {

struct Jump {
    unsigned long long mul, add;
};
__constant__ Jump c_jump[74];

__constant__ signed char c_p19_feature[BSF_P19_NODE_COUNT];
__constant__ short c_p19_left[BSF_P19_NODE_COUNT];
__constant__ short c_p19_right[BSF_P19_NODE_COUNT];
__constant__ double c_p19_value[BSF_P19_NODE_COUNT];
__constant__ short c_p19_root[BSF_P19_TREE_COUNT];

// P20 axis (gpu_p20_benchmark.cpp:41-52) and its complement.
__constant__ unsigned char c_axis[8] = {0, 2, 5, 7, 8, 10, 13, 15};
__constant__ unsigned char c_nonaxis_cols[192];  // full-lattice columns outside the 8x8 P20 subset

constexpr int INIT_LANES = 96;
// Bytes per lane's permutation: 65 words, an odd count, so the 32 lanes' t[i]
// of one swap step fall in 32 different banks (a stride of 68 words put 4
// lanes in each bank).
constexpr int TAB_STRIDE = 260;

// nextInt's remainder r % b for the non-power-of-two bounds b = 256 - i of the
// shuffle, as r - b * umulhi64(r, M[b]) with M[b] = floor(2^64 / b) + 1: for
// r < 2^31 the product overshoots r / b by under 2^-33, while r / b sits at
// least 1/b <= 2^-1.6 below the next integer, so the quotient is exact.
__constant__ unsigned long long c_div_magic[257];

__device__ __forceinline__ void lane_stream(int lane, int& stream, int& pos) {
    if (lane < 74) { stream = 0; pos = lane; }
    else if (lane < 78) { stream = 1; pos = lane - 74; }
    else if (lane < 82) { stream = 2; pos = lane - 78; }
    else if (lane < 84) { stream = 3; pos = lane - 82; }
    else { stream = -1; pos = 0; }
}

__device__ __forceinline__ int stream_length(int stream) {
    return stream == 0 ? 74 : (stream == 3 ? 2 : 4);
}

// Cache index of constructor `pos` of `stream`, or -1 for the 8 skipped ones.
__device__ __forceinline__ int state_index(int stream, int pos) {
    if (stream == 0) return pos < 40 ? pos : (pos < 48 ? -1 : pos - 8);
    if (stream == 1) return ST_TEMP + pos;
    if (stream == 2) return ST_RAIN + pos;
    return ST_BLEND + pos;
}

__device__ __forceinline__ std::uint64_t stream_start(std::int64_t seed, int stream) {
    const std::uint64_t mult = stream == 0 ? 1ULL : (stream == 1 ? 9871ULL : (stream == 2 ? 39811ULL : 543321ULL));
    const std::uint64_t s = static_cast<std::uint64_t>(seed) * mult;
    return (s ^ LCG_MUL) & LCG_MASK;  // Random.setSeed scramble
}

__device__ __forceinline__ double next_double(std::uint64_t& s) {
    s = lcg_step(s);
    const std::uint64_t hi = s >> 22;
    s = lcg_step(s);
    const std::uint64_t lo = s >> 21;
    return static_cast<double>(static_cast<long long>((hi << 27) + lo)) * 0x1.0p-53;
}

__device__ __forceinline__ void store_state(std::uint8_t* perms, double* offs, int world, int index,
                                            const std::uint8_t* tab, double a, double b, double c) {
    uint4* dst = reinterpret_cast<uint4*>(perms + (static_cast<std::size_t>(world) * ST_COUNT + index) * PERM_BYTES);
    const std::uint32_t* src = reinterpret_cast<const std::uint32_t*>(tab);  // 4-byte aligned slot
#pragma unroll
    for (int k = 0; k < 16; ++k) dst[k] = make_uint4(src[4 * k], src[4 * k + 1], src[4 * k + 2], src[4 * k + 3]);
    double* o = offs + (static_cast<std::size_t>(world) * ST_COUNT + index) * 4;
    o[0] = a;
    o[1] = b;
    o[2] = c;
    o[3] = 0.0;
}

// Builds every generator of every world in the batch. Each lane speculates one
// constructor: the LCG is jumped to the constructor's first draw assuming no
// earlier nextInt rejection (NoiseGeneratorPerlin173.reseed, :63-77), and the
// 256 dependent Fisher-Yates swaps run serially inside the lane. A lane that
// meets a rejection (probability ~1e-7 per draw) invalidates itself and every
// later constructor of its stream; those are rebuilt serially, exactly as Java
// consumes Random, by one thread per affected stream.
__global__ void __launch_bounds__(INIT_LANES) k_world_init(const std::int64_t* __restrict__ seeds, int n,
                                                          std::uint8_t* __restrict__ perms,
                                                          double* __restrict__ offs, int* fallbackCount) {
    __shared__ __align__(16) std::uint8_t tab[INIT_LANES * TAB_STRIDE];
    __shared__ int firstReject[4];
    const int world = blockIdx.x;
    if (world >= n) return;
    const int lane = threadIdx.x;
    const std::int64_t seed = seeds[world];
    int stream, pos;
    lane_stream(lane, stream, pos);
    if (lane < 4) firstReject[lane] = 1 << 30;
    std::uint8_t* t = tab + lane * TAB_STRIDE;
    std::uint32_t* t32 = reinterpret_cast<std::uint32_t*>(t);
#pragma unroll
    for (int k = 0; k < 64; ++k) {
        const std::uint32_t b = static_cast<std::uint32_t>(k * 4);
        t32[k] = b | ((b + 1) << 8) | ((b + 2) << 16) | ((b + 3) << 24);
    }
    __syncthreads();
    double a = 0.0, b = 0.0, c = 0.0;
    const bool consumed = stream == 0 && pos >= 40 && pos < 48;
    if (stream >= 0) {
        std::uint64_t s = stream_start(seed, stream);
        s = (c_jump[pos].mul * s + c_jump[pos].add) & LCG_MASK;
        a = next_double(s) * 256.0;
        b = next_double(s) * 256.0;
        c = next_double(s) * 256.0;
        bool rejected = false;
        // a rolled loop: fully unrolled, the 256 steps were about 100 KB of code
#pragma unroll 4
        for (int i = 0; i < 256; ++i) {
            const int bound = 256 - i;  // warp-uniform
            s = lcg_step(s);
            const std::uint32_t r = static_cast<std::uint32_t>(s >> 17);
            int j;
            if ((bound & (bound - 1)) == 0) {
                j = static_cast<int>((static_cast<std::uint64_t>(bound) * r) >> 31);
            } else {
                const std::uint32_t q = static_cast<std::uint32_t>(__umul64hi(r, c_div_magic[bound]));
                const std::uint32_t v = r - q * static_cast<std::uint32_t>(bound);
                if (static_cast<std::int32_t>(r - v + static_cast<std::uint32_t>(bound - 1)) < 0) rejected = true;
                j = static_cast<int>(v);
            }
            j += i;
            if (!consumed) {
                const std::uint8_t ti = t[i];
                t[i] = t[j];
                t[j] = ti;
            }
        }
        if (rejected) atomicMin(&firstReject[stream], pos);
    }
    __syncthreads();
    if (stream >= 0 && !consumed && pos < firstReject[stream]) {
        store_state(perms, offs, world, state_index(stream, pos), t, a, b, c);
    }
    __syncthreads();
    if (lane < 4 && firstReject[lane] < (1 << 30)) {
        // Exact serial rebuild of the stream from the first invalid constructor.
        const int st = lane;
        std::uint64_t s = stream_start(seed, st);
        const int p0 = firstReject[st];
        s = (c_jump[p0].mul * s + c_jump[p0].add) & LCG_MASK;
        for (int p = p0; p < stream_length(st); ++p) {
            const double aa = next_double(s) * 256.0;
            const double bb = next_double(s) * 256.0;
            const double cc = next_double(s) * 256.0;
            for (int i = 0; i < 256; ++i) t[i] = static_cast<std::uint8_t>(i);
            for (int i = 0; i < 256; ++i) {
                const int bound = 256 - i;
                s = lcg_step(s);
                std::uint32_t r = static_cast<std::uint32_t>(s >> 17);
                int j;
                if ((bound & (bound - 1)) == 0) {
                    j = static_cast<int>((static_cast<std::uint64_t>(bound) * r) >> 31);
                } else {
                    std::uint32_t v = r % static_cast<std::uint32_t>(bound);
                    // Java nextInt redraws while bits - val + (bound-1) overflows. A
                    // draw is rejected with probability (2^31 mod bound) / 2^31 < 2^-23
                    // (bound <= 256), so the 64-redraw cap is reached with probability
                    // below 2^-1472 per draw: unreachable, and the rebuild stays exact.
                    for (int guard = 0; guard < 64 &&
                         static_cast<std::int32_t>(r - v + static_cast<std::uint32_t>(bound - 1)) < 0; ++guard) {
                        s = lcg_step(s);
                        r = static_cast<std::uint32_t>(s >> 17);
                        v = r % static_cast<std::uint32_t>(bound);
                    }
                    j = static_cast<int>(v);
                }
                j += i;
                const std::uint8_t ti = t[i];
                t[i] = t[j];
                t[j] = ti;
            }
            const int idx = state_index(st, p);
            if (idx >= 0) store_state(perms, offs, world, idx, t, aa, bb, cc);
        }
        atomicAdd(fallbackCount, 1);
    }
}

// ---------------------------------------------------------------------------
// Shared-memory staging of one world's generators.
struct WorldSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    YEntry ytab[OCT3][17];
};

__device__ __forceinline__ void load_world(WorldSmem& w, const StateCache& cache, int world) {
    const uint4* src = reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(world) * WORLD_PERM_BYTES);
    uint4* dst = reinterpret_cast<uint4*>(w.perm);
    for (int k = threadIdx.x; k < WORLD_PERM_BYTES / 16; k += blockDim.x) dst[k] = src[k];
    const double* o = cache.offsets + static_cast<std::size_t>(world) * WORLD_OFFSETS;
    for (int k = threadIdx.x; k < ST_COUNT * 3; k += blockDim.x) w.off[k / 3][k % 3] = o[(k / 3) * 4 + (k % 3)];
}

__device__ __forceinline__ double octave_sy(int o, double amp) {
    return o < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
}

// Y axes of the 40 3D octaves (noise2 0-15, noise3 16-31, noise1 32-39).
__device__ __forceinline__ void build_ytabs(WorldSmem& w) {
    const int o = threadIdx.x;
    if (o < OCT3) {
        const int k = o < 16 ? o : (o < 32 ? o - 16 : o - 32);
        const double amp = exp2_neg(k);  // exact power of two
        build_yaxis(octave_sy(o, amp), w.off[o][1], w.ytab[o]);
    }
}

__device__ __forceinline__ Gen gen_of(const WorldSmem& w, int idx) {
    Gen g;
    g.p = w.perm + idx * PERM_BYTES;
    g.a = w.off[idx][0];
    g.b = w.off[idx][1];
    g.c = w.off[idx][2];
    return g;
}

__device__ __forceinline__ GenTable gen_table(const WorldSmem& w) {
    GenTable t;
    t.perm = w.perm;
    t.off = &w.off[0][0];
    return t;
}

// noise4 / noise5 sums of one lattice column (BetaTerrain173.java:685-707).
__device__ __forceinline__ void noise45(const WorldSmem& w, double X, double Z, double& n4, double& n5) {
    double amp = 1.0;
    double acc = 0.0;
    for (int o = 0; o < 10; ++o) {
        const double s = 1.121 * amp;
        const double v = octave2(gen_of(w, ST_N4 + o), X * s, Z * s) * (1.0 / amp);
        acc = o == 0 ? 0.0 + v : acc + v;
        amp /= 2.0;
    }
    n4 = acc;
    amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double s = 200.0 * amp;
        const double v = octave2(gen_of(w, ST_N5 + o), X * s, Z * s) * (1.0 / amp);
        acc = o == 0 ? 0.0 + v : acc + v;
        amp /= 2.0;
    }
    n5 = acc;
}

// noise2 / noise3 / noise1 sums for lattice levels [Y0, Y0+N) of one column.
template <int Y0, int N>
__device__ __forceinline__ void noise123(const WorldSmem& w, double X, double Z, double* a1, double* a2, double* a3) {
    double amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double s = NOISE_XZ * amp;
        octave3_column<Y0, N>(gen_of(w, ST_N2 + o), X * s, Z * s, w.ytab[o], 1.0 / amp, a2, o == 0);
        amp /= 2.0;
    }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double s = NOISE_XZ * amp;
        octave3_column<Y0, N>(gen_of(w, ST_N3 + o), X * s, Z * s, w.ytab[16 + o], 1.0 / amp, a3, o == 0);
        amp /= 2.0;
    }
    amp = 1.0;
    for (int o = 0; o < 8; ++o) {
        const double s = (NOISE_XZ / 80.0) * amp;
        octave3_column<Y0, N>(gen_of(w, ST_N1 + o), X * s, Z * s, w.ytab[32 + o], 1.0 / amp, a1, o == 0);
        amp /= 2.0;
    }
}

template <int Y0, int N>
__device__ __forceinline__ unsigned column_sign_bits(const WorldSmem& w, double X, double Z, double d5, double d7) {
    double a1[N], a2[N], a3[N];
    noise123<Y0, N>(w, X, Z, a1, a2, a3);
    unsigned bits = 0;
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (density_at(Y0 + k, d5, d7, a1[k], a2[k], a3[k]) > 0.0) bits |= 1u << (Y0 + k);
    return bits;
}

// ---------------------------------------------------------------------------
// Stage0 per world.
constexpr int S0_THREADS = 256;

struct Stage0Smem {
    WorldSmem w;
    double shape[8][256][2];       // d5, d7 per (centre, column)
    std::uint32_t mask17[8][256];  // positive bits of the 17 lattice levels
    std::uint16_t tasks[8 * 256];
    int p20[8], upper[8], high[8], gate[8];
    int taskCount;
    int lowerCenters;
};

// serial 4-connected BFS on a 16x16 grid (fillMonsterShapeStats,
// gpu_p20_benchmark.cpp:1022-1088); scratch 256 B visited + 512 B queue.
__device__ void shape_stats(const std::uint8_t* grid, std::uint8_t* visited, std::uint16_t* queue, int& largestOut,
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
    // f: fullY88, fullY96, fullY104, fullY112, y88Largest, y88Width, y88Depth,
    //    y96Largest, y96Width, y96Depth
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

// Mean of the 16 regression trees summed in tree order (p19_monster_gate.hpp:48-67).
__device__ double p19_score(int scout, const int* f) {
    double sum = 0.0;
    for (int t = 0; t < BSF_P19_TREE_COUNT; ++t) {
        int nd = c_p19_root[t];
        for (int depth = 0; depth < 64 && c_p19_feature[nd] >= 0; ++depth) {
            const double v = p19_feature(c_p19_feature[nd], scout, f);
            nd = v <= c_p19_value[nd] ? c_p19_left[nd] : c_p19_right[nd];
        }
        sum = t == 0 ? c_p19_value[nd] : sum + c_p19_value[nd];
    }
    return sum / static_cast<double>(BSF_P19_TREE_COUNT);
}

__device__ __forceinline__ int highest_reentry(std::uint32_t mask) {
    // stage0gpu::highestReentryYIndex (stage0_exact_gpu.hpp:552-566)
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

__global__ void __launch_bounds__(S0_THREADS) k_stage0(StateCache cache, int n, int centers, Profile prof,
                                                       RegionInfo* __restrict__ regions,
                                                       RegionRef* __restrict__ coarseQueue, int* coarseCount,
                                                       int coarseCapacity) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Stage0Smem& s = *reinterpret_cast<Stage0Smem*>(smem_raw);
    const int world = blockIdx.x;
    if (world >= n) return;
    const int tid = threadIdx.x;
    load_world(s.w, cache, world);
    if (tid < 8) { s.p20[tid] = 0; s.upper[tid] = 0; s.high[tid] = 0; }
    for (int k = tid; k < 8 * 256; k += S0_THREADS) (&s.mask17[0][0])[k] = 0;
    __syncthreads();
    build_ytabs(s.w);
    __syncthreads();
    const GenTable cg = gen_table(s.w);

    // P20: the 8x8 axis columns of every centre (gpu_p20_benchmark.cpp:335-589).
    for (int t = tid; t < centers * 64; t += S0_THREADS) {
        const int c = t >> 6, k = t & 63;
        const int ix = c_axis[k >> 3], iz = c_axis[k & 7];
        const int cx = -28 + ix * 4 + center_chunk_x(c) * 4;
        const int cz = -28 + iz * 4 + center_chunk_z(c) * 4;
        double temp, rain, n4, n5, d5, d7;
        climate_at(cg, cx * 4 + 2, cz * 4 + 2, temp, rain);
        const double X = static_cast<double>(cx), Z = static_cast<double>(cz);
        noise45(s.w, X, Z, n4, n5);
        column_shape(temp, rain, n4, n5, d5, d7);
        const int col = ix * 16 + iz;
        s.shape[c][col][0] = d5;
        s.shape[c][col][1] = d7;
        const unsigned bits = column_sign_bits<11, 6>(s.w, X, Z, d5, d7);
        s.mask17[c][col] = bits;
        if (bits) atomicAdd(&s.p20[c], 1);
    }
    __syncthreads();
    if (tid == 0) {
        int nt = 0;
        for (int c = 0; c < centers; ++c) {
            const int g = prof.p20MinCount > 1 ? (s.p20[c] >= prof.p20MinCount ? s.p20[c] : 0) : s.p20[c];
            s.gate[c] = g;
            s.upper[c] = g;  // fullUpperCount starts from the gated P20 count (p33_shared_y.hpp:164)
            if (g > 0) s.tasks[nt++] = static_cast<std::uint16_t>(c);
        }
        s.taskCount = nt;
    }
    __syncthreads();

    // Upper: the 192 remaining columns of centres whose gated P20 count is positive.
    const int upperCenters = s.taskCount;
    for (int t = tid; t < upperCenters * 192; t += S0_THREADS) {
        const int c = s.tasks[t / 192];
        const int col = c_nonaxis_cols[t % 192];
        const int ix = col >> 4, iz = col & 15;
        const int cx = -28 + ix * 4 + center_chunk_x(c) * 4;
        const int cz = -28 + iz * 4 + center_chunk_z(c) * 4;
        double temp, rain, n4, n5, d5, d7;
        climate_at(cg, cx * 4 + 2, cz * 4 + 2, temp, rain);
        const double X = static_cast<double>(cx), Z = static_cast<double>(cz);
        noise45(s.w, X, Z, n4, n5);
        column_shape(temp, rain, n4, n5, d5, d7);
        s.shape[c][col][0] = d5;
        s.shape[c][col][1] = d7;
        const unsigned bits = column_sign_bits<11, 6>(s.w, X, Z, d5, d7);
        s.mask17[c][col] = bits;
        if (bits) atomicAdd(&s.upper[c], 1);
    }
    __syncthreads();
    if (tid == 0) s.taskCount = 0;
    __syncthreads();
    // Lower task list: upper-positive columns of centres with Upper >= upperMin.
    for (int t = tid; t < centers * 256; t += S0_THREADS) {
        const int c = t >> 8, col = t & 255;
        if (s.gate[c] > 0 && s.upper[c] >= prof.upperMinCount && s.mask17[c][col] != 0) {
            const int slot = atomicAdd(&s.taskCount, 1);
            s.tasks[slot] = static_cast<std::uint16_t>((c << 8) | col);
        }
    }
    __syncthreads();
    // Lower: levels 0..10 in two halves (p30_compact_lower.hpp:29-239).
    const int lowerTasks = s.taskCount * 2;
    for (int t = tid; t < lowerTasks; t += S0_THREADS) {
        const int e = s.tasks[t >> 1];
        const int c = e >> 8, col = e & 255;
        const int ix = col >> 4, iz = col & 15;
        const double X = static_cast<double>(-28 + ix * 4 + center_chunk_x(c) * 4);
        const double Z = static_cast<double>(-28 + iz * 4 + center_chunk_z(c) * 4);
        const double d5 = s.shape[c][col][0], d7 = s.shape[c][col][1];
        const unsigned bits = (t & 1) ? column_sign_bits<6, 5>(s.w, X, Z, d5, d7)
                                      : column_sign_bits<0, 6>(s.w, X, Z, d5, d7);
        if (bits) atomicOr(&s.mask17[c][col], bits);
    }
    __syncthreads();
    // highest re-entry per lower column; reuse the Y tables as P19 scratch afterwards.
    std::uint8_t* highest = reinterpret_cast<std::uint8_t*>(&s.shape[0][0][0]);  // [8][256], shape no longer needed
    __syncthreads();
    for (int k = tid; k < 8 * 256; k += S0_THREADS) highest[k] = 0xFF;
    __syncthreads();
    for (int t = tid; t < s.taskCount; t += S0_THREADS) {
        const int e = s.tasks[t];
        const int c = e >> 8, col = e & 255;
        const int h = highest_reentry(s.mask17[c][col]);
        highest[c * 256 + col] = h < 0 ? 0xFF : static_cast<std::uint8_t>(h);
        if (h >= 11) atomicAdd(&s.high[c], 1);
    }
    __syncthreads();

    // P19 features: grids y88 (highest >= 11) and y96 (highest >= 12) per centre.
    std::uint8_t* scratch = s.w.perm;  // 19.5 KB; the generators are no longer needed
    __shared__ int feat[8][12];
    __shared__ int evalMask;
    if (tid == 0) {
        int m = 0;
        for (int c = 0; c < centers; ++c)
            if (s.p20[c] >= prof.p20MinCount && s.upper[c] >= prof.upperMinCount && s.high[c] >= prof.highMinCount)
                m |= 1 << c;
        evalMask = m;
    }
    __syncthreads();
    if (tid < 16) {
        const int c = tid >> 1, which = tid & 1;
        if (c < centers && ((evalMask >> c) & 1)) {
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
                feat[c][0] = full[0]; feat[c][1] = full[1]; feat[c][2] = full[2]; feat[c][3] = full[3];
                feat[c][4] = L; feat[c][5] = W; feat[c][6] = D; feat[c][10] = T;
            } else {
                feat[c][7] = L; feat[c][8] = W; feat[c][9] = D; feat[c][11] = T;
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
        if ((evalMask >> c) & 1) {
            const int* f = feat[c];
            const double score = p19_score(s.upper[c], f);
            const bool extreme = f[4] >= 14 || f[7] >= 14;  // hasExtremeTopologySignal (p19_monster_gate.hpp:77-79)
            const bool pass = extreme || score >= prof.p19MinScore;
            // megaTopologyReject (gpu_p20_benchmark.cpp:1116-1128)
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
}

// ---------------------------------------------------------------------------
// One chunk's 16x128x16 stone bitmap per world (generateChunkBaseTerrain,
// BetaTerrain173.java:120-138 + generateBareTerrain :582-665).
struct ChunkSmem {
    WorldSmem w;
    double n1[25][17], n2[25][17], n3[25][17];
    double n4[25], n5[25], temp[25], rain[25];
    double dens[25][17];
    std::uint8_t bitmap[4096];
    unsigned long long hashPart[8];
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ void store_group(double (*dst)[17], int col, int y0, const double* src, int n) {
    for (int k = 0; k < n; ++k) dst[col][y0 + k] = src[k];
}

__global__ void __launch_bounds__(256) k_chunk_bitmap(StateCache cache, int n, int chunkX, int chunkZ,
                                                     std::uint8_t* __restrict__ bitmaps,
                                                     unsigned long long* __restrict__ hashes) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ChunkSmem& s = *reinterpret_cast<ChunkSmem*>(smem_raw);
    const int world = blockIdx.x;
    if (world >= n) return;
    const int tid = threadIdx.x;
    load_world(s.w, cache, world);
    __syncthreads();
    build_ytabs(s.w);
    __syncthreads();
    // Lattice column (i, j) sits at coarse (chunkX*4+i, chunkZ*4+j); its climate
    // is read at block (chunkX*16 + 3i+1, chunkZ*16 + 3j+1) (BetaTerrain173.java:741-749).
    if (tid < 75) {
        const int col = tid / 3, grp = tid % 3;
        const double X = static_cast<double>(chunkX * 4 + col / 5);
        const double Z = static_cast<double>(chunkZ * 4 + col % 5);
        if (grp == 0) {
            double a1[6], a2[6], a3[6];
            noise123<0, 6>(s.w, X, Z, a1, a2, a3);
            store_group(s.n1, col, 0, a1, 6); store_group(s.n2, col, 0, a2, 6); store_group(s.n3, col, 0, a3, 6);
        } else if (grp == 1) {
            double a1[6], a2[6], a3[6];
            noise123<6, 6>(s.w, X, Z, a1, a2, a3);
            store_group(s.n1, col, 6, a1, 6); store_group(s.n2, col, 6, a2, 6); store_group(s.n3, col, 6, a3, 6);
        } else {
            double a1[5], a2[5], a3[5];
            noise123<12, 5>(s.w, X, Z, a1, a2, a3);
            store_group(s.n1, col, 12, a1, 5); store_group(s.n2, col, 12, a2, 5); store_group(s.n3, col, 12, a3, 5);
        }
    } else if (tid < 100) {
        const int col = tid - 75;
        noise45(s.w, static_cast<double>(chunkX * 4 + col / 5), static_cast<double>(chunkZ * 4 + col % 5),
                s.n4[col], s.n5[col]);
    } else if (tid < 125) {
        const int col = tid - 100;
        const GenTable cg = gen_table(s.w);
        climate_at(cg, chunkX * 16 + (col / 5) * 3 + 1, chunkZ * 16 + (col % 5) * 3 + 1, s.temp[col], s.rain[col]);
    }
    __syncthreads();
    for (int k = tid; k < 25 * 17; k += 256) {
        const int col = k / 17, y = k % 17;
        double d5, d7;
        column_shape(s.temp[col], s.rain[col], s.n4[col], s.n5[col], d5, d7);
        s.dens[col][y] = density_at(y, d5, d7, s.n1[col][y], s.n2[col][y], s.n3[col][y]);
    }
    __syncthreads();
    {
        // Thread (i1, j1, k1): one 4x8x4 sub-cell, incremental fill in Java order.
        const int i1 = tid >> 6, j1 = (tid >> 4) & 3, k1 = tid & 15;
        const double d0 = 0.125;
        double d1 = s.dens[(i1 + 0) * 5 + j1 + 0][k1];
        double d2 = s.dens[(i1 + 0) * 5 + j1 + 1][k1];
        double d3 = s.dens[(i1 + 1) * 5 + j1 + 0][k1];
        double d4 = s.dens[(i1 + 1) * 5 + j1 + 1][k1];
        const double d5 = (s.dens[(i1 + 0) * 5 + j1 + 0][k1 + 1] - d1) * d0;
        const double d6 = (s.dens[(i1 + 0) * 5 + j1 + 1][k1 + 1] - d2) * d0;
        const double d7 = (s.dens[(i1 + 1) * 5 + j1 + 0][k1 + 1] - d3) * d0;
        const double d8 = (s.dens[(i1 + 1) * 5 + j1 + 1][k1 + 1] - d4) * d0;
        unsigned bytes[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) bytes[q] = 0;
#pragma unroll
        for (int l1 = 0; l1 < 8; ++l1) {
            double d10 = d1, d11 = d2;
            const double d12 = (d3 - d1) * 0.25;
            const double d13 = (d4 - d2) * 0.25;
#pragma unroll
            for (int i2 = 0; i2 < 4; ++i2) {
                double d15 = d10;
                const double d16 = (d11 - d10) * 0.25;
#pragma unroll
                for (int k2 = 0; k2 < 4; ++k2) {
                    if (d15 > 0.0) bytes[i2 * 4 + k2] |= 1u << l1;
                    d15 += d16;
                }
                d10 += d12;
                d11 += d13;
            }
            d1 += d5; d2 += d6; d3 += d7; d4 += d8;
        }
#pragma unroll
        for (int i2 = 0; i2 < 4; ++i2)
#pragma unroll
            for (int k2 = 0; k2 < 4; ++k2) {
                const int x = i1 * 4 + i2, z = j1 * 4 + k2;
                s.bitmap[(x * 16 + z) * 16 + k1] = static_cast<std::uint8_t>(bytes[i2 * 4 + k2]);
            }
    }
    __syncthreads();
    // Hash: sum of mix64(word_i + (i+1) * golden) over the 512 LE words.
    const unsigned long long* words = reinterpret_cast<const unsigned long long*>(s.bitmap);
    unsigned long long h = mix64(words[tid] + static_cast<unsigned long long>(tid + 1) * 0x9E3779B97F4A7C15ULL) +
                           mix64(words[tid + 256] + static_cast<unsigned long long>(tid + 257) * 0x9E3779B97F4A7C15ULL);
    for (int off = 16; off > 0; off >>= 1) h += __shfl_xor_sync(0xffffffffu, h, off);
    if ((tid & 31) == 0) s.hashPart[tid >> 5] = h;
    uint4* dst = reinterpret_cast<uint4*>(bitmaps + static_cast<std::size_t>(world) * 4096);
    dst[tid] = reinterpret_cast<const uint4*>(s.bitmap)[tid];
    __syncthreads();
    if (tid == 0) {
        unsigned long long t = 0;
        for (int k = 0; k < 8; ++k) t += s.hashPart[k];
        hashes[world] = t;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
Profile profile_by_id(int id) {
    // HuntProfileConfig table (gpu_p20_benchmark.cpp:7262-7290).
    switch (id) {
        case 1: return Profile{1, 8, 6, BSF_P19_THRESHOLD, 85, 1};
        case 2: return Profile{3, 19, 12, 6.70, 95, 0};
        case 3: return Profile{3, 19, 20, 6.70, 700, 0};
        default: return Profile{1, 5, 5, BSF_P19_THRESHOLD, 85, 0};
    }
}

static void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

void init_lcg_tables() {
    Jump j[74];
    unsigned long long mul = 1, add = 0;
    for (int k = 0; k < 74; ++k) {
        j[k].mul = mul & LCG_MASK;
        j[k].add = add & LCG_MASK;
        for (int step = 0; step < DRAWS_PER_CONSTRUCTOR; ++step) {
            add = (LCG_MUL * add + LCG_ADD) & LCG_MASK;
            mul = (LCG_MUL * mul) & LCG_MASK;
        }
    }
    check(cudaMemcpyToSymbol(c_jump, j, sizeof(j)), "jump table");
    unsigned long long magic[257] = {0};
    for (int b = 2; b <= 256; ++b)  // floor(2^64 / b) + 1; b is no power of two where it is read
        if (b & (b - 1)) magic[b] = ~0ULL / static_cast<unsigned long long>(b) + 1;
    check(cudaMemcpyToSymbol(c_div_magic, magic, sizeof(magic)), "division table");
    check(cudaMemcpyToSymbol(c_p19_feature, bsf_p19_feature, sizeof(bsf_p19_feature)), "p19 table");
    check(cudaMemcpyToSymbol(c_p19_left, bsf_p19_left, sizeof(bsf_p19_left)), "p19 table");
    check(cudaMemcpyToSymbol(c_p19_right, bsf_p19_right, sizeof(bsf_p19_right)), "p19 table");
    check(cudaMemcpyToSymbol(c_p19_value, bsf_p19_value, sizeof(bsf_p19_value)), "p19 table");
    check(cudaMemcpyToSymbol(c_p19_root, bsf_p19_root, sizeof(bsf_p19_root)), "p19 table");
    unsigned char cols[192];
    int k = 0;
    auto isAxis = [](int i) { return i == 0 || i == 2 || i == 5 || i == 7 || i == 8 || i == 10 || i == 13 || i == 15; };
    for (int ix = 0; ix < 16; ++ix)
        for (int iz = 0; iz < 16; ++iz)
            if (!(isAxis(ix) && isAxis(iz))) cols[k++] = static_cast<unsigned char>(ix * 16 + iz);
    check(cudaMemcpyToSymbol(c_nonaxis_cols, cols, sizeof(cols)), "column table");
    check(cudaFuncSetAttribute(k_stage0, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(Stage0Smem)), "smem");
    check(cudaFuncSetAttribute(k_chunk_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(ChunkSmem)), "smem");
}

void launch_world_init(const std::int64_t* dSeeds, int n, StateCache& cache, int* dFallbackCount,
                       cudaStream_t stream) {
    if (n <= 0) return;
    k_world_init<<<n, INIT_LANES, 0, stream>>>(dSeeds, n, cache.perms, cache.offsets, dFallbackCount);
    check(cudaGetLastError(), "k_world_init");
}

void launch_chunk_bitmaps(const StateCache& cache, int n, int chunkX, int chunkZ, std::uint8_t* dBitmaps,
                          std::uint64_t* dHashes, cudaStream_t stream) {
    if (n <= 0) return;
    k_chunk_bitmap<<<n, 256, sizeof(ChunkSmem), stream>>>(cache, n, chunkX, chunkZ, dBitmaps,
                                                         reinterpret_cast<unsigned long long*>(dHashes));
    check(cudaGetLastError(), "k_chunk_bitmap");
}

std::size_t stage0_shape_scratch_bytes(int) { return 0; }

void launch_stage0(const StateCache& cache, int n, int centers, const Profile& prof, double*,
                   RegionInfo* dRegions, RegionRef* dCoarseQueue, int* dCoarseCount, int coarseCapacity,
                   cudaStream_t stream) {
    if (n <= 0) return;
    k_stage0<<<n, S0_THREADS, sizeof(Stage0Smem), stream>>>(cache, n, centers, prof, dRegions, dCoarseQueue,
                                                            dCoarseCount, coarseCapacity);
    check(cudaGetLastError(), "k_stage0");
}

}  // namespace bsf
