// Coarse stage (61x61x17 lattice signs + floating-component score) and the
// generic lattice-noise kernel used by the exact scan, for sm_103a.
//
// The coarse signs are fused: one CTA evaluates 64 lattice columns (3 Y-range
// tasks of the 40 3D octaves + 1 task of the 26 2D octaves and the climate
// per column) and combines them into 17-bit sign masks in shared memory, so
// the 1.5 MB of per-region noise the reference writes to global memory
// (p35_direct_coarse.hpp:60-343) never leaves the SM.
#include "bsf_device.cuh"
#include "bsf_internal.h"

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <stdexcept>

namespace bsf {
namespace {

constexpr int TILE = 64;  // lattice columns per CTA
constexpr int COARSE_SIDE = 61;
constexpr int COARSE_COLS = COARSE_SIDE * COARSE_SIDE;
constexpr int COARSE_CELLS = COARSE_COLS * 17;

struct LatticeSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    YEntry ytab[OCT3][17];
    double n1[TILE][17], n2[TILE][17], n3[TILE][17];
    double d5[TILE], d7[TILE];
    double n4[TILE], n5[TILE];
    std::uint32_t mask[TILE];
};

__device__ __forceinline__ GenTable table(const LatticeSmem& s) {
    GenTable t;
    t.perm = s.perm;
    t.off = &s.off[0][0];
    return t;
}

__device__ void load_gens(LatticeSmem& s, const StateCache& cache, int world) {
    const uint4* src = reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(world) * WORLD_PERM_BYTES);
    uint4* dst = reinterpret_cast<uint4*>(s.perm);
    for (int k = threadIdx.x; k < WORLD_PERM_BYTES / 16; k += blockDim.x) dst[k] = src[k];
    const double* o = cache.offsets + static_cast<std::size_t>(world) * WORLD_OFFSETS;
    for (int k = threadIdx.x; k < ST_COUNT * 3; k += blockDim.x) s.off[k / 3][k % 3] = o[(k / 3) * 4 + (k % 3)];
}

__device__ void build_ytabs(LatticeSmem& s) {
    const int o = threadIdx.x;
    if (o < OCT3) {
        const int k = o < 16 ? o : (o < 32 ? o - 16 : o - 32);
        const double amp = exp2_neg(k);
        const double sy = o < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
        build_yaxis(sy, s.off[o][1], s.ytab[o]);
    }
}

template <int Y0, int N>
__device__ __forceinline__ void lattice_task(const LatticeSmem& s, double X, double Z, int col, double (*n1)[17],
                                             double (*n2)[17], double (*n3)[17]) {
    const GenTable t = table(s);
    double a1[N], a2[N], a3[N];
    double amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double sc = NOISE_XZ * amp;
        octave3_column<Y0, N>(t(ST_N2 + o), X * sc, Z * sc, s.ytab[o], 1.0 / amp, a2, o == 0);
        amp /= 2.0;
    }
    amp = 1.0;
    for (int o = 0; o < 16; ++o) {
        const double sc = NOISE_XZ * amp;
        octave3_column<Y0, N>(t(ST_N3 + o), X * sc, Z * sc, s.ytab[16 + o], 1.0 / amp, a3, o == 0);
        amp /= 2.0;
    }
    amp = 1.0;
    for (int o = 0; o < 8; ++o) {
        const double sc = (NOISE_XZ / 80.0) * amp;
        octave3_column<Y0, N>(t(ST_N1 + o), X * sc, Z * sc, s.ytab[32 + o], 1.0 / amp, a1, o == 0);
        amp /= 2.0;
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
        n1[col][Y0 + k] = a1[k];
        n2[col][Y0 + k] = a2[k];
        n3[col][Y0 + k] = a3[k];
    }
}

// Runs the 4 tasks of the CTA's 64 columns (threads 0..191: 3D Y ranges,
// 192..255: 2D noise). Column (ix, iz) of the tile sits at coarse
// (originX + ix, originZ + iz).
// ABOVE_64: only levels 8..16, which the exact scan's fill reads (blocks at
// y >= 64); the legacy Y cells still come from the full 17-level tables.
template <bool ABOVE_64>
__device__ __forceinline__ void tile_noise(LatticeSmem& s, int originX, int originZ, int side, int tileBase) {
    const int tid = threadIdx.x;
    const int total = side * side;
    if (tid < 3 * TILE) {
        const int col = tid % TILE, grp = tid / TILE;
        const int g = tileBase + col;
        if (g < total) {
            const double X = static_cast<double>(originX + g / side);
            const double Z = static_cast<double>(originZ + g % side);
            if (ABOVE_64) {
                if (grp == 0) lattice_task<8, 3>(s, X, Z, col, s.n1, s.n2, s.n3);
                else if (grp == 1) lattice_task<11, 3>(s, X, Z, col, s.n1, s.n2, s.n3);
                else lattice_task<14, 3>(s, X, Z, col, s.n1, s.n2, s.n3);
            } else {
                if (grp == 0) lattice_task<0, 6>(s, X, Z, col, s.n1, s.n2, s.n3);
                else if (grp == 1) lattice_task<6, 6>(s, X, Z, col, s.n1, s.n2, s.n3);
                else lattice_task<12, 5>(s, X, Z, col, s.n1, s.n2, s.n3);
            }
        }
    } else {
        const int col = tid - 3 * TILE;
        const int g = tileBase + col;
        if (g < total) {
            const double X = static_cast<double>(originX + g / side);
            const double Z = static_cast<double>(originZ + g % side);
            noise45(table(s), X, Z, s.n4[col], s.n5[col]);
        }
    }
}

// Coarse signs for queued regions: lattice -28..32 (+ centre * 4), climate at
// block 4c+2 (coarse_exact_core.hpp:218-350 with the centre offset of
// p35_direct_coarse.hpp). signs[job][col] = 17-bit positive mask.
__global__ void __launch_bounds__(256) k_coarse_signs(StateCache cache, const RegionRef* __restrict__ queue,
                                                     const int* count, int maxCount,
                                                     std::uint32_t* __restrict__ signs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LatticeSmem& s = *reinterpret_cast<LatticeSmem*>(smem_raw);
    const int tilesPerJob = (COARSE_COLS + TILE - 1) / TILE;
    const int jobs = min(*count, maxCount);
    int loadedWorld = -1;
    // Persistent grid: each CTA walks (job, tile) items; the generators and Y
    // tables are restaged only when the item's world changes.
    for (int item = blockIdx.x; item < jobs * tilesPerJob; item += gridDim.x) {
        const int job = item / tilesPerJob;
        const int tile = item % tilesPerJob;
        const RegionRef ref = queue[job];
        const int originX = -28 + center_chunk_x(ref.center) * 4;
        const int originZ = -28 + center_chunk_z(ref.center) * 4;
        __syncthreads();
        if (ref.world != loadedWorld) {
            load_gens(s, cache, ref.world);
            __syncthreads();
            build_ytabs(s);
            loadedWorld = ref.world;
        }
        if (threadIdx.x < TILE) s.mask[threadIdx.x] = 0;
        __syncthreads();
        const int tileBase = tile * TILE;
        tile_noise<false>(s, originX, originZ, COARSE_SIDE, tileBase);
        if (threadIdx.x >= 3 * TILE) {
            const int col = threadIdx.x - 3 * TILE;
            const int g = tileBase + col;
            if (g < COARSE_COLS) {
                const int cx = originX + g / COARSE_SIDE, cz = originZ + g % COARSE_SIDE;
                double temp, rain;
                climate_at(table(s), cx * 4 + 2, cz * 4 + 2, temp, rain);
                column_shape(temp, rain, s.n4[col], s.n5[col], s.d5[col], s.d7[col]);
            }
        }
        __syncthreads();
        for (int k = threadIdx.x; k < TILE * 17; k += blockDim.x) {
            const int col = k / 17, y = k % 17;
            if (tileBase + col < COARSE_COLS &&
                density_at(y, s.d5[col], s.d7[col], s.n1[col][y], s.n2[col][y], s.n3[col][y]) > 0.0)
                atomicOr(&s.mask[col], 1u << y);
        }
        __syncthreads();
        if (threadIdx.x < TILE && tileBase + threadIdx.x < COARSE_COLS)
            signs[static_cast<std::size_t>(job) * COARSE_COLS + tileBase + threadIdx.x] = s.mask[threadIdx.x];
    }
}

// Lattice noise to global memory (exact scan): one job = one lattice, levels
// 8..16 of n1/n2/n3 (the fill of blocks y >= 64 reads no lower level).
__global__ void __launch_bounds__(256) k_lattice_noise(StateCache cache, const LatticeJob* __restrict__ jobs,
                                                      LatticeJob single, int side, LatticeBuffers buf) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LatticeSmem& s = *reinterpret_cast<LatticeSmem*>(smem_raw);
    const int total = side * side;
    const int tilesPerJob = (total + TILE - 1) / TILE;
    const int job = blockIdx.x / tilesPerJob;
    const int tile = blockIdx.x % tilesPerJob;
    const LatticeJob J = jobs ? jobs[job] : single;
    load_gens(s, cache, J.world);
    __syncthreads();
    build_ytabs(s);
    __syncthreads();
    const int tileBase = tile * TILE;
    tile_noise<true>(s, J.originX, J.originZ, side, tileBase);
    __syncthreads();
    const std::size_t base = static_cast<std::size_t>(job) * buf.columnsPerJob;
    for (int k = threadIdx.x; k < TILE * 9; k += blockDim.x) {
        const int col = k / 9, y = 8 + k % 9;  // levels 8..16 only
        const int g = tileBase + col;
        if (g < total) {
            const std::size_t idx = (base + g) * 17 + y;
            buf.n1[idx] = s.n1[col][y];
            buf.n2[idx] = s.n2[col][y];
            buf.n3[idx] = s.n3[col][y];
        }
    }
    if (threadIdx.x < TILE && tileBase + threadIdx.x < total) {
        buf.n4[base + tileBase + threadIdx.x] = s.n4[threadIdx.x];
        buf.n5[base + tileBase + threadIdx.x] = s.n5[threadIdx.x];
    }
}

// ---- coarse component score (coarsecore::scoreSigns, coarse_exact_core.hpp:83-169)
// Order-independent restatement: the score is the largest cell count over
// 6-connected positive components that reach level >= 8, touch neither level 0
// nor the lattice side, and have a lattice column with a positive cell below
// the component's lowest cell in that column (a re-entry).
constexpr int CC_THREADS = 1024;
constexpr int COARSE_SCORE_CTAS = 304;  // persistent grid: 2 per SM; scratch is per CTA
constexpr int FLAG_BAD = 1, FLAG_TALL = 2, FLAG_REENTRY = 4;

__device__ __forceinline__ int find_root(const int* L, int x) {
    for (int guard = 0; guard < (1 << 20); ++guard) {
        const int p = L[x];
        if (p == x) return x;
        x = p;
    }
    return x;
}

// Lock-free union by smaller root index; retries only when a concurrent
// union changed one of the roots, bounded defensively.
__device__ __forceinline__ void unite(int* L, int a, int b, int* err) {
    for (int guard = 0; guard < (1 << 20); ++guard) {
        a = find_root(L, a);
        b = find_root(L, b);
        if (a == b) return;
        if (a > b) { const int t = a; a = b; b = t; }
        const int old = atomicCAS(&L[b], b, a);
        if (old == b) return;
    }
    atomicOr(err, 1);
}

// First level of the run of set bits of column mask m that holds level y.
__device__ __forceinline__ int run_start(std::uint32_t m, int y) {
    const std::uint32_t zerosBelow = ~m & ((1u << y) - 1u);
    return zerosBelow ? 32 - __clz(zerosBelow) : 0;
}

// Components are unions of runs: a column's positive cells form at most 9
// runs along y (contiguous set bits of its 17-bit mask), and a run's cells are
// 6-connected, so the union-find works on run starts only. Neighbouring runs
// (z + 1, x + 1) are united once per overlapping pair, and counts, flags and
// the re-entry test are taken per run. One thread per column throughout.
__global__ void __launch_bounds__(CC_THREADS) k_coarse_score(const std::uint32_t* __restrict__ signs,
                                                            const RegionRef* __restrict__ queue, const int* count,
                                                            int maxCount, int* __restrict__ labelScratch,
                                                            int* __restrict__ statScratch, RegionInfo* regions,
                                                            int centers, int* err) {
    const int jobs = min(*count, maxCount);
    int* L = labelScratch + static_cast<std::size_t>(blockIdx.x) * COARSE_CELLS;
    int* cnt = statScratch + static_cast<std::size_t>(blockIdx.x) * COARSE_CELLS * 2;
    int* flg = cnt + COARSE_CELLS;
    __shared__ int best;
    for (int job = blockIdx.x; job < jobs; job += gridDim.x) {
        const std::uint32_t* sg = signs + static_cast<std::size_t>(job) * COARSE_COLS;
        __syncthreads();
        if (threadIdx.x == 0) best = 0;
        // run starts are their own roots, with empty statistics
        for (int col = threadIdx.x; col < COARSE_COLS; col += CC_THREADS) {
            std::uint32_t m = sg[col];
            while (m) {
                const int y = __ffs(m) - 1;
                const int len = __ffs(~(m >> y)) - 1;
                const int c = col * 17 + y;
                L[c] = c;
                cnt[c] = 0;
                flg[c] = 0;
                m &= ~(((1u << len) - 1u) << y);
            }
        }
        __syncthreads();
        for (int col = threadIdx.x; col < COARSE_COLS; col += CC_THREADS) {
            const std::uint32_t m = sg[col];
            if (!m) continue;
            const int x = col / COARSE_SIDE, z = col % COARSE_SIDE;
            for (int dir = 0; dir < 2; ++dir) {
                const bool inside = dir == 0 ? z + 1 < COARSE_SIDE : x + 1 < COARSE_SIDE;
                if (!inside) continue;
                const int ncol = col + (dir == 0 ? 1 : COARSE_SIDE);
                const std::uint32_t mn = sg[ncol];
                const std::uint32_t ov = m & mn;
                std::uint32_t segs = ov & ~(ov << 1);  // first level of each overlapping stretch
                while (segs) {
                    const int y = __ffs(segs) - 1;
                    unite(L, col * 17 + run_start(m, y), ncol * 17 + run_start(mn, y), err);
                    segs &= segs - 1;
                }
            }
        }
        __syncthreads();
        for (int col = threadIdx.x; col < COARSE_COLS; col += CC_THREADS) {
            std::uint32_t m = sg[col];
            while (m) {
                const int y = __ffs(m) - 1;
                const int len = __ffs(~(m >> y)) - 1;
                L[col * 17 + y] = find_root(L, col * 17 + y);
                m &= ~(((1u << len) - 1u) << y);
            }
        }
        __syncthreads();
        // per run: its cells, bottom / side contact, height >= 8; and the
        // re-entry test (IslandSearchEngine's lazy P17 and coarsecore::scoreSigns):
        // a component's lowest cell in a column with a positive cell below it
        for (int col = threadIdx.x; col < COARSE_COLS; col += CC_THREADS) {
            std::uint32_t m = sg[col];
            const int x = col / COARSE_SIDE, z = col % COARSE_SIDE;
            const bool side = x == 0 || z == 0 || x == COARSE_SIDE - 1 || z == COARSE_SIDE - 1;
            int seen[9];
            int nseen = 0;
            bool below = false;
            while (m) {
                const int y = __ffs(m) - 1;
                const int len = __ffs(~(m >> y)) - 1;
                const int r = L[col * 17 + y];
                atomicAdd(&cnt[r], len);
                int f = 0;
                if (y == 0 || side) f |= FLAG_BAD;
                if (y + len - 1 >= 8) f |= FLAG_TALL;
                bool first = true;
                for (int k = 0; k < nseen; ++k) first = first && seen[k] != r;
                if (first) {
                    if (nseen < 9) seen[nseen++] = r;
                    if (below) f |= FLAG_REENTRY;
                }
                if (f) atomicOr(&flg[r], f);
                below = true;
                m &= ~(((1u << len) - 1u) << y);
            }
        }
        __syncthreads();
        for (int col = threadIdx.x; col < COARSE_COLS; col += CC_THREADS) {
            std::uint32_t m = sg[col];
            while (m) {
                const int y = __ffs(m) - 1;
                const int len = __ffs(~(m >> y)) - 1;
                const int c = col * 17 + y;
                if (L[c] == c && flg[c] == (FLAG_TALL | FLAG_REENTRY)) atomicMax(&best, cnt[c]);
                m &= ~(((1u << len) - 1u) << y);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const RegionRef ref = queue[job];
            RegionInfo& r = regions[static_cast<std::size_t>(ref.world) * centers + ref.center];
            r.coarse = best;
            r.coarseEvaluated = 1;
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

std::once_flag g_attrs;  // handles on several threads launch these kernels
void ensure_attrs() {
    std::call_once(g_attrs, [] {
        check(cudaFuncSetAttribute(k_coarse_signs, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(LatticeSmem)),
              "coarse smem");
        check(cudaFuncSetAttribute(k_lattice_noise, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(LatticeSmem)),
              "lattice smem");
    });
}

}  // namespace

std::size_t coarse_scratch_bytes_per_region() {
    return static_cast<std::size_t>(COARSE_COLS) * 4 + static_cast<std::size_t>(COARSE_CELLS) * 4 * 3;
}

int coarse_score_ctas(int maxCount) { return std::min(maxCount, COARSE_SCORE_CTAS); }

void launch_coarse_score(const StateCache& cache, const RegionRef* dQueue, const int* dCount, int maxCount,
                         const LatticeBuffers&, std::uint32_t* dSignScratch, int* dLabelScratch, int* dStatScratch,
                         RegionInfo* dRegions, int centers, cudaStream_t stream) {
    if (maxCount <= 0) return;
    ensure_attrs();
    const int tilesPerJob = (COARSE_COLS + TILE - 1) / TILE;
    const int signGrid = std::min(maxCount * tilesPerJob, 152 * 4);
    k_coarse_signs<<<signGrid, 256, sizeof(LatticeSmem), stream>>>(cache, dQueue, dCount, maxCount, dSignScratch);
    check(cudaGetLastError(), "k_coarse_signs");
    // the retry-bound flag sits right after the per-CTA scratch of the grid
    int* err = dStatScratch + static_cast<std::size_t>(coarse_score_ctas(maxCount)) * COARSE_CELLS * 2;
    k_coarse_score<<<coarse_score_ctas(maxCount), CC_THREADS, 0, stream>>>(
        dSignScratch, dQueue, dCount, maxCount, dLabelScratch, dStatScratch, dRegions, centers, err);
    check(cudaGetLastError(), "k_coarse_score");
}

void launch_coarse_cc(const RegionRef* dQueue, const int* dCount, int maxCount, std::uint32_t* dSignScratch,
                      int* dLabelScratch, int* dStatScratch, RegionInfo* dRegions, int centers, cudaStream_t stream) {
    if (maxCount <= 0) return;
    // the retry-bound flag sits right after the per-CTA scratch of the grid
    int* err = dStatScratch + static_cast<std::size_t>(coarse_score_ctas(maxCount)) * COARSE_CELLS * 2;
    k_coarse_score<<<coarse_score_ctas(maxCount), CC_THREADS, 0, stream>>>(
        dSignScratch, dQueue, dCount, maxCount, dLabelScratch, dStatScratch, dRegions, centers, err);
    check(cudaGetLastError(), "k_coarse_score");
}

void launch_lattice_noise_one(const StateCache& cache, const LatticeJob& job, const LatticeBuffers& buf,
                              cudaStream_t stream) {
    ensure_attrs();
    const int tilesPerJob = (job.side * job.side + TILE - 1) / TILE;
    k_lattice_noise<<<tilesPerJob, 256, sizeof(LatticeSmem), stream>>>(cache, nullptr, job, job.side, buf);
    check(cudaGetLastError(), "k_lattice_noise");
}

}  // namespace bsf
