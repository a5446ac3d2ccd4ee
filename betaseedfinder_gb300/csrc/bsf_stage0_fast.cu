// Screened Stage0 (P20 -> Upper -> Lower) and the P19 gate for sm_103a.
//
// k_stage0_fast: persistent grid of one CTA per SM slot, each taking two worlds
// at a time. Per world the CTA stages in shared memory (~93 KB): the 76
// generators, the FP32 Y axes of the 40 3D octaves, and an axis table holding,
// for each of the 66 lattice octaves (40 3D + 26 2D), the exact lattice index /
// fraction / fade of the 46 distinct X and 46 distinct Z coarse coordinates
// that the 8 region centres use (X = -88..92 step 4). Each phase's task list
// spans both worlds, so the rounds of the CTA's threads are fuller. Column tasks
// run their octaves in FP32 (bsf_screen.cuh); columns whose density signs the
// error bound cannot decide are recomputed in exact FP64, so every mask and
// count is bit-identical to the FP64 kernel (bsf_stage0.cu). Regions that pass
// the P20/Upper/High gates hand their highest-re-entry grid to k_p19 through a
// device queue.
//
// k_p19: one warp per queued region: the two 16x16 topology grids (Y88, Y96),
// the 16-tree score, the extreme bypass and the Mega topology rule
// (gpu_p20_benchmark.cpp:1022-1128, p19_monster_gate.hpp:48-79), then the
// coarse-queue append.
#include "bsf_device.cuh"
#include "bsf_exact_warp.cuh"
#include "bsf_internal.h"
#include "bsf_screen.cuh"

#include <cmath>
#include <cstdio>
#include <stdexcept>

namespace bsf {

#include "p19_table.inc"

namespace {

using namespace screen;

constexpr int NAX = 46;      // distinct coarse coordinates per axis over the 8 centres
constexpr int NOCT = 66;      // 40 3D + 26 2D lattice octaves (state index == octave index)
constexpr int PAIR = 2;        // worlds staged per CTA pass (measured: 9% faster than one)

__constant__ unsigned char cf_axis[8] = {0, 2, 5, 7, 8, 10, 13, 15};
__constant__ float2 cf_octave_scale[66];  // octave_scale(o) split into a float pair
__constant__ unsigned char cf_nonaxis_cols[192];
__constant__ signed char cf_p19_feature[BSF_P19_NODE_COUNT];
__constant__ short cf_p19_left[BSF_P19_NODE_COUNT];
__constant__ short cf_p19_right[BSF_P19_NODE_COUNT];
__constant__ double cf_p19_value[BSF_P19_NODE_COUNT];
__constant__ short cf_p19_root[BSF_P19_TREE_COUNT];

// One world's staged state (16-byte aligned: perm and axf are copied / read as uint4).
struct alignas(16) WorldSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    YF yf[OCT3][17];
    float axf[NOCT][2][NAX];   // FP32 fraction; after Lower, the 8 x 256 highest re-entry bytes
    float axd[NOCT][2][NAX];   // FP32 fade
    std::uint8_t axi[NOCT][2][NAX];  // lattice index & 255
    // 17-level sign masks of the world's distinct lattice columns: centre c's column
    // (ix, iz) is lattice column (ix + cx(c) + 15, iz + cz(c) + 15) of a 46 x 46 grid,
    // so the columns that adjacent centres share are computed once
    std::uint32_t maskL[NAX * NAX];
    std::uint32_t claimed[(NAX * NAX + 31) / 32];       // lattice columns with a P20 / Upper task
    std::uint32_t lowerClaimed[(NAX * NAX + 31) / 32];  // lattice columns with a Lower task
    float4 clim[10];  // climate generators' offsets as float pairs (climate_split)
    int p20[8], upper[8], high[8], gate[8];
};

// Column shapes of one wave of a phase's tasks (bsf_screen.cuh column_shape_f
// in two passes, see shape_wave).
constexpr int SHAPE_CAP = 1536;

struct FastSmem {
    WorldSmem w[PAIR];
    std::uint16_t tasks[PAIR * 8 * 256];  // lattice-column tasks (slot << 12 | lattice index)
    std::uint8_t units[PAIR * 8];         // centres through the P20 gate (slot << 3 | centre)
    int unitCount;
    float4 shape[SHAPE_CAP];              // d5, its bound, d7, its bound (d5 bound < 0: undecided)
    std::uint16_t climate[SHAPE_CAP];     // wave tasks whose d5 needs the climate and noise4
    std::uint16_t plain[SHAPE_CAP];       // the wave's other tasks
    int taskCount, screened, fallbacks, climateCount, plainCount;
    int cursor[3];                        // next unclaimed task of the P20, Upper and Lower phases
};
static_assert(sizeof(WorldSmem) % 16 == 0 && offsetof(WorldSmem, perm) == 0 && offsetof(WorldSmem, axf) % 16 == 0,
              "uint4 copies into perm and out of axf need 16-byte alignment");
static_assert(sizeof(FastSmem) <= 227 * 1024, "one CTA's shared memory");
static_assert(PAIR * NAX * NAX < (1 << 13) && NAX * NAX < (1 << 12), "task and fallback encodings");

__device__ __forceinline__ GenTable gtab(const WorldSmem& s) {
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

__device__ __forceinline__ AxisF axis_of(const WorldSmem& s, int o, int a, int k) {
    const float f = s.axf[o][a][k];
    return AxisF{f, f - 1.0f, s.axd[o][a][k], s.axi[o][a][k]};
}

// Lattice index of centre c's column col (ix = col >> 4, iz = col & 15).
__device__ __forceinline__ int lattice_index(int c, int col) {
    return ((col >> 4) + center_chunk_x(c) + 15) * NAX + (col & 15) + center_chunk_z(c) + 15;
}

// Coarse coordinates and axis-table indices of lattice column L (the same for
// every centre that reads it: cx = -28 + 4 ix + 4 cx(c) = 4 kx - 88).
__device__ __forceinline__ void lattice_coords(int L, int& cx, int& cz, int& kx, int& kz) {
    kx = L / NAX;
    kz = L % NAX;
    cx = 4 * kx - 88;
    cz = 4 * kz - 88;
}

// Claims lattice column L in a bitmap; true for the first claimant.
__device__ __forceinline__ bool claim(std::uint32_t* bits, int L) {
    const std::uint32_t m = 1u << (L & 31);
    return (atomicOr(&bits[L >> 5], m) & m) == 0u;
}

constexpr std::uint32_t UPPER_BITS = 0x1F800u;  // levels 11..16


// ---- screened FP32 path ---------------------------------------------------
// Column shape (BetaTerrain173.java:739-804) in two passes. The first takes
// noise5 and the d6/d7 half (shape_d7_f) of every task of a wave; in the
// reference's d6 < 0 branch (about 70% of Stage0 columns) d5 is 0.5 whatever
// the climate and noise4 are, so only the other columns go on to the second
// pass, which the CTA's threads share densely: the climate's ten simplex
// octaves are the most expensive part of a screened column.
__device__ __noinline__ bool shape_first(const WorldSmem& s, int L, float4& sh) {
    int cx, cz, kx, kz;
    lattice_coords(L, cx, cz, kx, kz);
    float n5 = 0.0f;
#pragma unroll 1
    for (int o = 0; o < 16; ++o) {
        const int st = ST_N5 + o;
        n5 = n5 + octave2f(s.perm + st * PERM_BYTES, axis_of(s, st, 0, kx), axis_of(s, st, 1, kz)) *
                      static_cast<float>(1 << o);  // 0.0f + first term is exact
    }
    Fe d7;
    bool zeroD5 = false;
    if (!shape_d7_f(Fe{n5, E_N5}, d7, zeroD5)) {
        sh = make_float4(0.0f, -1.0f, 0.0f, 0.0f);  // d5 branch undecided: the exact path decides
        return false;
    }
    sh = make_float4(0.5f, 0.0f, d7.v, d7.e);
    return !zeroD5;
}

// Second pass: the climate and noise4 part of d5 (shape_d5_f), as (d5, bound).
__device__ __noinline__ float2 shape_climate(const WorldSmem& s, int L) {
    int cx, cz, kx, kz;
    lattice_coords(L, cx, cz, kx, kz);
    Fe temp, rain;
    climate_f(gtab(s), s.clim, cx * 4 + 2, cz * 4 + 2, temp, rain);
    float n4 = 0.0f;
#pragma unroll 1
    for (int o = 0; o < 10; ++o) {
        const int st = ST_N4 + o;
        n4 = n4 + octave2f(s.perm + st * PERM_BYTES, axis_of(s, st, 0, kx), axis_of(s, st, 1, kz)) *
                      static_cast<float>(1 << o);
    }
    const Fe d5 = shape_d5_f(temp, rain, Fe{n4, E_N4});
    return make_float2(d5.v, d5.e);
}

// Screened signs of one column's levels [Y0, Y0+N) given its shape; false
// when undecided. The levels are compile-time: the top fade and the level bits
// fold into the hot loop.
template <int Y0, int N>
__device__ __noinline__ bool screened_range(const WorldSmem& s, int L, Fe d5, Fe d7, unsigned& bits) {
    int cx, cz, kx, kz;
    lattice_coords(L, cx, cz, kx, kz);
    auto oct = [&](int st, int o, float* v) {  // state st's octave o (st is also its Y-table index)
        octave3f<Y0, N>(s.perm + st * PERM_BYTES, axis_of(s, st, 0, kx), axis_of(s, st, 1, kz), s.yf[st],
                        static_cast<float>(1 << o), v, true);
    };
    return progressive_signs<N>(Y0, N, d5, d7, oct, bits);
}

// Level ranges of the column tasks: 0 -> 11..15 (P20 / Upper; 16 is air),
// 1 -> 0..5 and 2 -> 6..10 (the Lower groups).
__device__ __forceinline__ void range_levels(int r, int& y0, int& n) {
    y0 = r == 0 ? 11 : (r == 1 ? 0 : 6);
    n = r == 0 ? TOP_SOLID_LEVEL - 10 : (r == 1 ? 6 : 5);
}

// Column ranges a task's screen left undecided, for the exact path: up to two
// entries (range << 14 | slot << 13 | lattice index), NONE when unused.
constexpr std::uint32_t NONE = 0xFFFFFFFFu;
struct Pending {
    std::uint32_t e[2] = {NONE, NONE};
};
__device__ __forceinline__ std::uint32_t fallback_entry(FastSmem& s, int q, int L, int r) {
    atomicAdd(&s.fallbacks, 1);
    return static_cast<std::uint32_t>((r << 14) | (q << 13) | L);
}

// P20 / Upper column task of world slot q: levels 11..15 (16 is air).
__device__ __forceinline__ Pending upper_task(FastSmem& s, int q, int L, const float4& sh, bool forceExact) {
    WorldSmem& w = s.w[q];
    atomicAdd(&s.screened, 1);
    unsigned bits = 0;
    Pending p;
    if (!forceExact && sh.y >= 0.0f &&
        screened_range<11, TOP_SOLID_LEVEL - 10>(w, L, Fe{sh.x, sh.y}, Fe{sh.z, sh.w}, bits)) {
        w.maskL[L] = bits;
        return p;
    }
    p.e[0] = fallback_entry(s, q, L, 0);
    return p;
}

// Lower column task: levels 0..5 and 6..10 (two screened tasks) on one shape.
__device__ __forceinline__ Pending lower_task(FastSmem& s, int q, int L, const float4& sh, bool forceExact) {
    WorldSmem& w = s.w[q];
    atomicAdd(&s.screened, 2);
    const bool shaped = !forceExact && sh.y >= 0.0f;
    const Fe d5{sh.x, sh.y}, d7{sh.z, sh.w};
    unsigned lo = 0, hi = 0;
    const bool okLo = shaped && screened_range<0, 6>(w, L, d5, d7, lo);
    const bool okHi = shaped && screened_range<6, 5>(w, L, d5, d7, hi);
    const unsigned bits = (okLo ? lo : 0u) | (okHi ? hi : 0u);
    if (bits) atomicOr(&w.maskL[L], bits);
    Pending p;
    if (!okLo) p.e[0] = fallback_entry(s, q, L, 1);
    if (!okHi) p.e[1] = fallback_entry(s, q, L, 2);
    return p;
}

// Exact FP64 column task by one whole warp (bsf_exact_warp.cuh).
__device__ __noinline__ unsigned exact_task_w(const WorldSmem& s, int L, int r) {
    int cx, cz, kx, kz;
    lattice_coords(L, cx, cz, kx, kz);
    int y0, n;
    range_levels(r, y0, n);
    return exactwarp::exact_column_warp(s, cx, cz, y0, n);
}

// A phase's tasks [0, total) handed out 32 at a time to whichever warp asks
// next: a screened task stops as soon as its signs are certain, so task costs
// vary, and a fixed split would leave the CTA waiting at the phase's barrier for
// its slowest warp. Column ranges the chunk's screen left undecided are
// resolved right away by the same warp, all 32 lanes on one column
// (bsf_exact_warp.cuh), while the other warps go on claiming chunks. Every
// lane of the warp calls it; the phase's barrier follows.
template <typename F>
__device__ __forceinline__ void run_phase(FastSmem& s, int k, int total, F body) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&s.cursor[k], 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        const Pending p = base + lane < total ? body(base + lane) : Pending{};
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            unsigned todo = __ballot_sync(0xffffffffu, p.e[i] != NONE);
            while (todo) {
                const int src = __ffs(todo) - 1;
                todo &= todo - 1;
                const std::uint32_t e = __shfl_sync(0xffffffffu, p.e[i], src);
                const int r = e >> 14, q = (e >> 13) & 1, L = e & 8191;
                const unsigned bits = exact_task_w(s.w[q], L, r);
                if (lane == 0) atomicOr(&s.w[q].maskL[L], bits);
            }
        }
    }
    __syncthreads();
}

// First pass of the shapes of wave tasks [t0, t0 + n), n <= SHAPE_CAP, into
// s.shape[0, n) (spread over all threads), and the wave's task order for
// run_phase: first the m tasks whose d5 needs the climate and noise4
// (s.climate), then the others (s.plain), each list compacted by ballots. The
// climate part then runs inside the task that reads it (wave_task), on warps of
// climate tasks only, instead of as a pass of its own between two barriers:
// such a pass kept more than half of the CTA's threads waiting, the climate
// being needed by about 30% of the columns. The longest tasks also start first.
// coord(t) gives a task's (slot, lattice index). Resets the phase's task
// cursor k; returns m.
template <int FT, typename C>
__device__ __forceinline__ int shape_wave(FastSmem& s, int k, int t0, int n, bool forceExact, C coord) {
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) s.cursor[k] = 0;
    if (!forceExact) {
        for (int base = 0; base < n; base += FT) {
            const int i = base + tid;
            bool need = false;
            if (i < n) {
                int q, L;
                coord(t0 + i, q, L);
                need = shape_first(s.w[q], L, s.shape[i]);
            }
            const unsigned vote = __ballot_sync(0xffffffffu, need);
            const unsigned rest = __ballot_sync(0xffffffffu, i < n && !need);
            int slot = 0, slotRest = 0;
            if (lane == 0) {
                if (vote) slot = atomicAdd(&s.climateCount, __popc(vote));
                if (rest) slotRest = atomicAdd(&s.plainCount, __popc(rest));
            }
            slot = __shfl_sync(0xffffffffu, slot, 0);
            slotRest = __shfl_sync(0xffffffffu, slotRest, 0);
            const unsigned below = (1u << lane) - 1u;
            if (need) s.climate[slot + __popc(vote & below)] = static_cast<std::uint16_t>(i);
            else if (i < n) s.plain[slotRest + __popc(rest & below)] = static_cast<std::uint16_t>(i);
        }
    }
    __syncthreads();
    const int m = s.climateCount;
    __syncthreads();  // every thread holds m before the counts are reset for the next wave
    if (tid == 0) s.climateCount = s.plainCount = 0;
    return m;
}

// Task i of a wave in shape_wave's order: its (slot, lattice index) and its
// shape, the climate part computed here for the first m.
template <typename C>
__device__ __forceinline__ float4 wave_task(const FastSmem& s, int i, int m, int t0, bool forceExact, C coord, int& q,
                                            int& L) {
    const int t = forceExact ? i : (i < m ? s.climate[i] : s.plain[i - m]);
    coord(t0 + t, q, L);
    float4 sh = s.shape[t];
    if (!forceExact && i < m) {
        const float2 d5 = shape_climate(s.w[q], L);
        sh.x = d5.x;
        sh.y = d5.y;
    }
    return sh;
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

// FT threads per CTA, MINB CTAs per SM: launch shapes chosen by the autotuner.
// Each pass stages PAIR worlds; every phase's task list covers both, slot-major.
template <int FT, int MINB>
__global__ void __launch_bounds__(FT, MINB) k_stage0_fast(StateCache cache, int n, int centers, Profile prof,
                                                          RegionInfo* __restrict__ regions, Stage0FastScratch fs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FastSmem& s = *reinterpret_cast<FastSmem*>(smem_raw);
    const int tid = threadIdx.x;
    if (tid == 0) { s.screened = 0; s.fallbacks = 0; s.climateCount = 0; s.plainCount = 0; }
    for (int pair = blockIdx.x; pair * PAIR < n; pair += gridDim.x) {
        const int w0 = pair * PAIR;
        const int nw = min(PAIR, n - w0);
        __syncthreads();
        for (int q = 0; q < nw; ++q) {
            const uint4* src =
                reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(w0 + q) * WORLD_PERM_BYTES);
            uint4* dst = reinterpret_cast<uint4*>(s.w[q].perm);
            for (int k = tid; k < WORLD_PERM_BYTES / 16; k += FT) dst[k] = src[k];
            const double* o = cache.offsets + static_cast<std::size_t>(w0 + q) * WORLD_OFFSETS;
            // the lattice octaves' X (a) and Z (c) offsets also go to the axis phase as float
            // pairs, in the shape buffer, which the phases only use later
            float2* split = reinterpret_cast<float2*>(s.shape) + q * NOCT * 2;
            for (int k = tid; k < ST_COUNT * 3; k += FT) {
                const double v = o[(k / 3) * 4 + (k % 3)];
                s.w[q].off[k / 3][k % 3] = v;
                if (k / 3 < NOCT && k % 3 != 1) {
                    const DF d = df_of(v);
                    split[(k / 3) * 2 + (k % 3) / 2] = make_float2(d.h, d.l);
                }
            }
        }
        if (tid < 8 * nw) {
            WorldSmem& w = s.w[tid >> 3];
            const int c = tid & 7;
            w.p20[c] = 0; w.upper[c] = 0; w.high[c] = 0; w.gate[c] = 0;
        }
        if (tid == 0) {
            s.taskCount = 0;
            s.cursor[0] = s.cursor[1] = s.cursor[2] = 0;
        }
        constexpr int LCOLS = NAX * NAX, LWORDS = (NAX * NAX + 31) / 32;
        for (int k = tid; k < nw * LCOLS; k += FT) s.w[k / LCOLS].maskL[k % LCOLS] = 0;
        for (int k = tid; k < nw * LWORDS; k += FT) {
            s.w[k / LWORDS].claimed[k % LWORDS] = 0;
            s.w[k / LWORDS].lowerClaimed[k % LWORDS] = 0;
        }
        __syncthreads();
        if (tid < OCT3 * nw) {
            const int q = tid / OCT3, o = tid % OCT3;
            const int k = o < 16 ? o : (o < 32 ? o - 16 : o - 32);
            const double amp = exp2_neg(k);
            const double sy = o < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
            YEntry ya[17];
            build_yaxis(sy, s.w[q].off[o][1], ya);
            build_yf(ya, s.w[q].yf[o]);
        } else if (tid < OCT3 * nw + 10 * nw) {
            const int q = (tid - OCT3 * nw) / 10, i = (tid - OCT3 * nw) % 10;
            s.w[q].clim[i] = climate_split(s.w[q].off[ST_TEMP + i]);
        }
        // Axis table entries in double-float (FP64 only where a floor is too close to
        // call). One centre reads coordinates 15..30 only (kx = ix + 15).
        const int nk = centers == 1 ? 16 : NAX, k0 = centers == 1 ? 15 : 0;
        const int axes = NOCT * 2 * nk;
        for (int e = tid; e < nw * axes; e += FT) {
            const int q = e / axes, f = e % axes;
            WorldSmem& w = s.w[q];
            const int o = f / (2 * nk), a = (f / nk) & 1, k = k0 + f % nk;
            const float2 sc = cf_octave_scale[o];
            const float2 of = reinterpret_cast<const float2*>(s.shape)[(q * NOCT + o) * 2 + a];
            AxisF ax;
            if (!make_axis_df(-88 + 4 * k, DF{sc.x, sc.y}, DF{of.x, of.y}, ax))
                ax = make_axis(static_cast<double>(-88 + 4 * k) * octave_scale(o), w.off[o][a == 0 ? 0 : 2]);
            w.axf[o][a][k] = ax.f;
            w.axd[o][a][k] = ax.fd;
            w.axi[o][a][k] = static_cast<std::uint8_t>(ax.i);
        }
        __syncthreads();

        // Tasks are distinct lattice columns: a column two centres share is computed once.
        auto taskCoord = [&](int t, int& q, int& L) {
            const int e = s.tasks[t];
            q = e >> 12;
            L = e & 4095;
        };
        auto appendTask = [&](int q, int L) {
            const int slot = atomicAdd(&s.taskCount, 1);
            s.tasks[slot] = static_cast<std::uint16_t>((q << 12) | L);
        };
        // P20: the 8x8 axis columns of every centre (gpu_p20_benchmark.cpp:335-589).
        const int p20Tasks = centers * 64;
        auto p20Column = [&](int t, int& q, int& c, int& L) {
            q = t / p20Tasks;
            const int u = t % p20Tasks, k = u & 63;
            c = u >> 6;
            L = lattice_index(c, cf_axis[k >> 3] * 16 + cf_axis[k & 7]);
        };
        for (int t = tid; t < nw * p20Tasks; t += FT) {
            int q, c, L;
            p20Column(t, q, c, L);
            if (claim(s.w[q].claimed, L)) appendTask(q, L);
        }
        __syncthreads();
        const int p20N = s.taskCount;
        for (int t0 = 0; t0 < p20N; t0 += SHAPE_CAP) {
            const int wn = min(SHAPE_CAP, p20N - t0);
            const int m = shape_wave<FT>(s, 0, t0, wn, fs.forceExact, taskCoord);
            run_phase(s, 0, wn, [&](int i) {
                int q, L;
                const float4 sh = wave_task(s, i, m, t0, fs.forceExact, taskCoord, q, L);
                return upper_task(s, q, L, sh, fs.forceExact);
            });
        }
        __syncthreads();
        for (int t = tid; t < nw * p20Tasks; t += FT) {
            int q, c, L;
            p20Column(t, q, c, L);
            if (s.w[q].maskL[L]) atomicAdd(&s.w[q].p20[c], 1);
        }
        __syncthreads();
        if (tid == 0) {
            int nu = 0;
            for (int q = 0; q < nw; ++q) {
                WorldSmem& w = s.w[q];
                for (int c = 0; c < centers; ++c) {
                    const int g = prof.p20MinCount > 1 ? (w.p20[c] >= prof.p20MinCount ? w.p20[c] : 0) : w.p20[c];
                    w.gate[c] = g;
                    w.upper[c] = g;  // fullUpperCount starts from the gated P20 count (p33_shared_y.hpp:164)
                    if (g > 0) s.units[nu++] = static_cast<std::uint8_t>((q << 3) | c);
                }
            }
            s.unitCount = nu;
            s.taskCount = 0;
        }
        __syncthreads();
        // Upper: the 192 remaining columns of centres whose gated P20 count is positive,
        // less the lattice columns P20 already computed.
        const int upperUnits = s.unitCount;
        auto upperColumn = [&](int t, int& q, int& c, int& L) {
            const int e = s.units[t / 192];
            q = e >> 3;
            c = e & 7;
            L = lattice_index(c, cf_nonaxis_cols[t % 192]);
        };
        for (int t = tid; t < upperUnits * 192; t += FT) {
            int q, c, L;
            upperColumn(t, q, c, L);
            if (claim(s.w[q].claimed, L)) appendTask(q, L);
        }
        __syncthreads();
        const int upperN = s.taskCount;
        for (int t0 = 0; t0 < upperN; t0 += SHAPE_CAP) {
            const int wn = min(SHAPE_CAP, upperN - t0);
            const int m = shape_wave<FT>(s, 1, t0, wn, fs.forceExact, taskCoord);
            run_phase(s, 1, wn, [&](int i) {
                int q, L;
                const float4 sh = wave_task(s, i, m, t0, fs.forceExact, taskCoord, q, L);
                return upper_task(s, q, L, sh, fs.forceExact);
            });
        }
        __syncthreads();
        for (int t = tid; t < upperUnits * 192; t += FT) {
            int q, c, L;
            upperColumn(t, q, c, L);
            if (s.w[q].maskL[L]) atomicAdd(&s.w[q].upper[c], 1);
        }
        __syncthreads();
        if (tid == 0) s.taskCount = 0;
        __syncthreads();
        // Lower: levels 0..10 of the upper-positive columns of centres through the
        // Upper gate, in two halves (p30_compact_lower.hpp:29-239) that share the
        // column's shape; each distinct lattice column once.
        const int allCols = centers * 256;
        auto lowerColumn = [&](int t, int& q, int& c, int& col) {
            q = t / allCols;
            const int u = t % allCols;
            c = u >> 8;
            col = u & 255;
        };
        for (int t = tid; t < nw * allCols; t += FT) {
            int q, c, col;
            lowerColumn(t, q, c, col);
            const WorldSmem& w = s.w[q];
            const int L = lattice_index(c, col);
            if (w.gate[c] > 0 && w.upper[c] >= prof.upperMinCount && (w.maskL[L] & UPPER_BITS) != 0 &&
                claim(s.w[q].lowerClaimed, L))
                appendTask(q, L);
        }
        __syncthreads();
        const int lowerN = s.taskCount;
        for (int t0 = 0; t0 < lowerN; t0 += SHAPE_CAP) {
            const int wn = min(SHAPE_CAP, lowerN - t0);
            const int m = shape_wave<FT>(s, 2, t0, wn, fs.forceExact, taskCoord);
            run_phase(s, 2, wn, [&](int i) {
                int q, L;
                const float4 sh = wave_task(s, i, m, t0, fs.forceExact, taskCoord, q, L);
                return lower_task(s, q, L, sh, fs.forceExact);
            });
        }
        __syncthreads();
        // Highest re-entry per lower column of each centre through the Upper gate; each
        // world's axis table serves as its 8 x 256 byte grid now.
        for (int k = tid; k < nw * 8 * 256; k += FT)
            reinterpret_cast<std::uint8_t*>(&s.w[k >> 11].axf[0][0][0])[k & 2047] = 0xFF;
        __syncthreads();
        for (int t = tid; t < nw * allCols; t += FT) {
            int q, c, col;
            lowerColumn(t, q, c, col);
            WorldSmem& w = s.w[q];
            const std::uint32_t m = w.maskL[lattice_index(c, col)];
            if (w.gate[c] > 0 && w.upper[c] >= prof.upperMinCount && (m & UPPER_BITS) != 0) {
                const int h = highest_reentry(m);
                reinterpret_cast<std::uint8_t*>(&w.axf[0][0][0])[c * 256 + col] =
                    h < 0 ? 0xFF : static_cast<std::uint8_t>(h);
                if (h >= 11) atomicAdd(&w.high[c], 1);
            }
        }
        __syncthreads();
        // Region outcomes, one warp per (world, centre); P19 candidates go to the P19 queue with their grids.
        const int warp = tid >> 5, lane = tid & 31;
        for (int u = warp; u < nw * centers; u += FT / 32) {
            const int q = u / centers, c = u % centers;
            const WorldSmem& w = s.w[q];
            const bool eval = w.p20[c] >= prof.p20MinCount && w.upper[c] >= prof.upperMinCount &&
                              w.high[c] >= prof.highMinCount;
            int slot = -1;
            if (lane == 0) {
                RegionInfo r;
                r.p19Score = __longlong_as_double(0x7ff8000000000000LL);
                r.coarse = 0;
                r.p20 = static_cast<std::int16_t>(w.p20[c]);
                r.upper = static_cast<std::int16_t>(w.upper[c]);
                r.high = static_cast<std::int16_t>(w.high[c]);
                r.p19Evaluated = r.p19Pass = r.p19Extreme = r.megaReject = r.coarseEvaluated = r.pad0 = 0;
                r.fullY88 = r.fullY96 = r.fullY104 = r.fullY112 = r.y88Largest = r.y96Largest = 0;
                r.y88Width = r.y88Depth = r.y88Touches = r.y96Width = r.y96Depth = r.y96Touches = 0;
                r.pad1[0] = r.pad1[1] = 0;
                regions[static_cast<std::size_t>(w0 + q) * centers + c] = r;
                slot = eval ? atomicAdd(fs.p19Count, 1) : -1;
                if (eval && slot < fs.p19Capacity) fs.p19Queue[slot] = RegionRef{w0 + q, c};
            }
            slot = __shfl_sync(0xffffffffu, slot, 0);
            if (slot >= 0 && slot < fs.p19Capacity && lane < 16) {
                const uint4* src = reinterpret_cast<const uint4*>(&w.axf[0][0][0]) + c * 16;
                reinterpret_cast<uint4*>(fs.highest + static_cast<std::size_t>(slot) * 256)[lane] = src[lane];
            }
        }
    }
    __syncthreads();
    if (tid == 0 && fs.stats) {
        atomicAdd(&fs.stats[0], static_cast<unsigned long long>(s.screened));
        atomicAdd(&fs.stats[1], static_cast<unsigned long long>(s.fallbacks));
    }
}

// ---- P19 --------------------------------------------------------------------
// fillMonsterShapeStats (gpu_p20_benchmark.cpp:1022-1088): serial 4-connected BFS.
__device__ void shape_stats(const std::uint8_t* highest, int minH, std::uint8_t* visited, std::uint8_t* queue,
                            int& largestOut, int& widthOut, int& depthOut, int& touchesOut) {
    auto on = [&](int idx) {
        const int e = highest[idx];
        return e != 0xFF && e >= minH;
    };
    for (int i = 0; i < 256; ++i) visited[i] = 0;
    int largest = 0, minX = 16, maxX = -1, minZ = 16, maxZ = -1, touches = 0;
    for (int x = 0; x < 16; ++x) {
        for (int z = 0; z < 16; ++z) {
            const int index = x * 16 + z;
            if (!on(index)) continue;
            minX = min(minX, x);
            maxX = max(maxX, x);
            minZ = min(minZ, z);
            maxZ = max(maxZ, z);
            if (x == 0 || z == 0 || x == 15 || z == 15) touches = 1;
            if (visited[index]) continue;
            int head = 0, tail = 0, cluster = 0;
            visited[index] = 1;
            queue[tail++] = static_cast<std::uint8_t>(index);
            while (head < tail) {
                const int cur = queue[head++];
                ++cluster;
                const int cx = cur >> 4, cz = cur & 15;
                const int nx[4] = {cx - 1, cx + 1, cx, cx};
                const int nz[4] = {cz, cz, cz - 1, cz + 1};
                for (int k = 0; k < 4; ++k) {
                    if (nx[k] < 0 || nz[k] < 0 || nx[k] >= 16 || nz[k] >= 16) continue;
                    const int nb = nx[k] * 16 + nz[k];
                    if (!on(nb) || visited[nb]) continue;
                    visited[nb] = 1;
                    queue[tail++] = static_cast<std::uint8_t>(nb);
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
    // f: fullY88, fullY96, fullY104, fullY112, y88Largest, y88Width, y88Depth, y96Largest, y96Width, y96Depth
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

// Mean of the 16 trees summed in tree order (p19_monster_gate.hpp:48-67).
__device__ double p19_score(int scout, const int* f) {
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

constexpr int P19_WARPS = 8;

__global__ void __launch_bounds__(P19_WARPS * 32) k_p19(Stage0FastScratch fs, int centers, Profile prof,
                                                        RegionInfo* __restrict__ regions,
                                                        RegionRef* __restrict__ coarseQueue, int* coarseCount,
                                                        int coarseCapacity) {
    __shared__ std::uint8_t grids[P19_WARPS][256];
    __shared__ std::uint8_t scratch[P19_WARPS][2][512];
    __shared__ int feat[P19_WARPS][12];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = min(*fs.p19Count, fs.p19Capacity);
    for (int q = blockIdx.x * P19_WARPS + warp; q < total; q += gridDim.x * P19_WARPS) {
        const RegionRef ref = fs.p19Queue[q];
        const std::uint8_t* src = fs.highest + static_cast<std::size_t>(q) * 256;
        for (int i = lane; i < 256; i += 32) grids[warp][i] = src[i];
        __syncwarp();
        if (lane < 2) {
            int L, W, D, T;
            shape_stats(grids[warp], lane == 0 ? 11 : 12, scratch[warp][lane], scratch[warp][lane] + 256, L, W, D, T);
            int* f = feat[warp];
            if (lane == 0) { f[4] = L; f[5] = W; f[6] = D; f[10] = T; }
            else { f[7] = L; f[8] = W; f[9] = D; f[11] = T; }
        } else if (lane < 6) {
            const int minH = 11 + (lane - 2);
            int cnt = 0;
            for (int i = 0; i < 256; ++i) cnt += grids[warp][i] != 0xFF && grids[warp][i] >= minH;
            feat[warp][lane - 2] = cnt;
        }
        __syncwarp();
        if (lane == 0) {
            const int* f = feat[warp];
            RegionInfo& r = regions[static_cast<std::size_t>(ref.world) * centers + ref.center];
            const double score = p19_score(r.upper, f);
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
                if (slot < coarseCapacity) coarseQueue[slot] = ref;
            }
        }
        __syncwarp();
    }
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

// Launch-shape variants of k_stage0_fast the autotuner chooses from.
struct Variant {
    const char* name;
    int threads;
    void (*kernel)(StateCache, int, int, Profile, RegionInfo*, Stage0FastScratch);
    int grid;
};
Variant g_variants[] = {
    // 640 threads at 96 registers (some spills) hide latency better than 512 at
    // 128 (Stage0: 37.65 vs 38.72 ms per 16,384 worlds); it is the default
    {"640x1", 640, k_stage0_fast<640, 1>, 0},
    {"512x1", 512, k_stage0_fast<512, 1>, 0},
    {"256x2", 256, k_stage0_fast<256, 2>, 0},
    {"384x1", 384, k_stage0_fast<384, 1>, 0},
};
constexpr int kVariants = sizeof(g_variants) / sizeof(g_variants[0]);
int g_variant = 0;
int g_sms = 152;

}  // namespace

int stage0_fast_variants() { return kVariants; }
const char* stage0_fast_variant_name(int v) { return g_variants[v].name; }
void set_stage0_fast_variant(int v) { g_variant = (v >= 0 && v < kVariants) ? v : 0; }
int get_stage0_fast_variant() { return g_variant; }

// octave_scale(o) on the host, in the same IEEE operations as the device.
double octave_scale_host(int o) {
    if (o < 16) return NOISE_XZ * std::ldexp(1.0, -o);
    if (o < 32) return NOISE_XZ * std::ldexp(1.0, -(o - 16));
    if (o < 40) return (NOISE_XZ / 80.0) * std::ldexp(1.0, -(o - 32));
    if (o < 50) return 1.121 * std::ldexp(1.0, -(o - 40));
    return 200.0 * std::ldexp(1.0, -(o - 50));
}

void init_stage0_fast() {
    float2 scales[NOCT];
    for (int o = 0; o < NOCT; ++o) {
        const double v = octave_scale_host(o);
        const float h = static_cast<float>(v);
        scales[o] = make_float2(h, static_cast<float>(v - static_cast<double>(h)));
    }
    check(cudaMemcpyToSymbol(cf_octave_scale, scales, sizeof(scales)), "octave scales");
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
    int dev = 0;
    check(cudaGetDevice(&dev), "device");
    check(cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
    for (Variant& v : g_variants) {
        check(cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(FastSmem)),
              "stage0 fast smem");
        int perSm = 0;
        check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, v.kernel, v.threads, sizeof(FastSmem)),
              "occupancy");
        v.grid = g_sms * (perSm > 0 ? perSm : 1);
    }
}

std::size_t stage0_fast_smem() { return sizeof(FastSmem); }

void launch_stage0_fast(const StateCache& cache, int n, int centers, const Profile& prof, RegionInfo* dRegions,
                        RegionRef* dCoarseQueue, int* dCoarseCount, int coarseCapacity, const Stage0FastScratch& fs,
                        cudaStream_t stream, bool persistent) {
    if (n <= 0) return;
    check(cudaMemsetAsync(fs.p19Count, 0, sizeof(int), stream), "memset");
    const Variant& v = g_variants[g_variant];
    const int pairs = (n + PAIR - 1) / PAIR;  // a CTA takes PAIR worlds per pass
    const int grid = (!persistent || pairs < v.grid) ? pairs : v.grid;
    v.kernel<<<grid, v.threads, sizeof(FastSmem), stream>>>(cache, n, centers, prof, dRegions, fs);
    check(cudaGetLastError(), "k_stage0_fast");
    const int p19Grid = g_sms;
    k_p19<<<p19Grid, P19_WARPS * 32, 0, stream>>>(fs, centers, prof, dRegions, dCoarseQueue, dCoarseCount,
                                                  coarseCapacity);
    check(cudaGetLastError(), "k_p19");
}

}  // namespace bsf
