// MEGA exact scan on sm_103a: exact 16x128x16 terrain for (2r+1)^2 chunks
// around a region centre, floating-component labelling above the island floor
// (y >= 68), component statistics, the reference's match rule and tie order,
// and the preview column model.
//
// Restates IslandSearchEngine.findFloatingIslandInSeed's exact part
// (IslandSearchEngine.java:2861-2977), floodFillFlat (:4096-4202), isMatch
// (:3972-4003) and compareComponents (:4079-4094). The Java flood fill visits
// components from candidate starts in chunk-major order; every statistic it
// collects is a property of the whole 6-connected component of stone cells at
// y >= 68, so the GPU labels all components with a lock-free union-find and
// reproduces the scan order only where it matters: the first candidate start
// of a component (its flood order) breaks ties between equal components.
#include "bsf_device.cuh"
#include "bsf_internal.h"

#include <climits>
#include <cstdio>
#include <mutex>
#include <stdexcept>

namespace bsf {
namespace {

constexpr int SY = 61;  // stored levels: y = 67..127 (ys = y - 67)
constexpr int FLOOR_Y = 68;
constexpr int FLAG_SIDE = 1, FLAG_BOTTOM = 2;

struct Dims {
    int r, nc, SX, SZ, side;
    int ccx, ccz;
    int minWorldX, minWorldZ;
    long long cells;  // SY * SX * SZ
    int slotCap;
};

Dims make_dims(int r, int ccx, int ccz) {
    Dims d;
    d.r = r;
    d.nc = 2 * r + 1;
    d.SX = d.SZ = 16 * d.nc;
    d.side = 8 * r + 5;
    d.ccx = ccx;
    d.ccz = ccz;
    d.minWorldX = (ccx - r) * 16;
    d.minWorldZ = (ccz - r) * 16;
    d.cells = static_cast<long long>(SY) * d.SX * d.SZ;
    d.slotCap = d.nc * d.nc * 4 * (128 - FLOOR_Y);
    return d;
}

struct SlotStats {
    int* blocks;
    int* columns;
    int* minX;
    int* maxX;
    int* minZ;
    int* maxZ;
    int* minY;
    int* maxY;
    int* flags;
    int* firstCand;
    unsigned long long* sumX;
    unsigned long long* sumZ;
};

SlotStats carve_slots(int* base, int cap) {
    SlotStats s;
    s.blocks = base;
    s.columns = base + cap;
    s.minX = base + 2 * cap;
    s.maxX = base + 3 * cap;
    s.minZ = base + 4 * cap;
    s.maxZ = base + 5 * cap;
    s.minY = base + 6 * cap;
    s.maxY = base + 7 * cap;
    s.flags = base + 8 * cap;
    s.firstCand = base + 9 * cap;
    // 10 int arrays, then two 64-bit arrays (cap is even, so they stay 8-byte aligned)
    s.sumX = reinterpret_cast<unsigned long long*>(base + 10 * cap);
    s.sumZ = s.sumX + cap;
    return s;
}

std::size_t slot_bytes(int cap) { return static_cast<std::size_t>(cap) * (10 * 4 + 2 * 8); }

struct ChunkSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    double dens[25][17];
};

// One chunk: climate at its 25 lattice points (block offsets 3i+1), density
// from the shared region lattice, then the incremental trilinear fill of
// generateBareTerrain (BetaTerrain173.java:582-665) for y-cells 8..15
// (y 64..127); stone cells at y >= 67 are stored.
__global__ void __launch_bounds__(128) k_exact_chunks(StateCache cache, int world, Dims d, LatticeBuffers lat,
                                                     std::uint8_t* __restrict__ stone) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ChunkSmem& s = *reinterpret_cast<ChunkSmem*>(smem_raw);
    const int a = blockIdx.x / d.nc, b = blockIdx.x % d.nc;
    const int chunkX = d.ccx - d.r + a, chunkZ = d.ccz - d.r + b;
    const int tid = threadIdx.x;
    {
        const uint4* src = reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(world) * WORLD_PERM_BYTES);
        uint4* dst = reinterpret_cast<uint4*>(s.perm);
        for (int k = tid + ST_TEMP * 16; k < WORLD_PERM_BYTES / 16; k += blockDim.x) dst[k] = src[k];
        const double* o = cache.offsets + static_cast<std::size_t>(world) * WORLD_OFFSETS;
        for (int k = tid; k < ST_COUNT * 3; k += blockDim.x) s.off[k / 3][k % 3] = o[(k / 3) * 4 + (k % 3)];
    }
    __syncthreads();
    if (tid < 25) {
        const int i = tid / 5, j = tid % 5;
        GenTable t;
        t.perm = s.perm;
        t.off = &s.off[0][0];
        double temp, rain, d5, d7;
        climate_at(t, chunkX * 16 + i * 3 + 1, chunkZ * 16 + j * 3 + 1, temp, rain);
        const std::size_t col = static_cast<std::size_t>(a * 4 + i) * d.side + (b * 4 + j);
        column_shape(temp, rain, lat.n4[col], lat.n5[col], d5, d7);
        for (int y = 8; y < 17; ++y)  // the lattice holds levels 8..16: cells 8..15 read no lower level
            s.dens[tid][y] = density_at(y, d5, d7, lat.n1[col * 17 + y], lat.n2[col * 17 + y], lat.n3[col * 17 + y]);
    }
    __syncthreads();
    const int i1 = tid >> 5, j1 = (tid >> 3) & 3, k1 = 8 + (tid & 7);
    const double d0 = 0.125;
    double d1 = s.dens[(i1 + 0) * 5 + j1 + 0][k1];
    double d2 = s.dens[(i1 + 0) * 5 + j1 + 1][k1];
    double d3 = s.dens[(i1 + 1) * 5 + j1 + 0][k1];
    double d4 = s.dens[(i1 + 1) * 5 + j1 + 1][k1];
    const double d5 = (s.dens[(i1 + 0) * 5 + j1 + 0][k1 + 1] - d1) * d0;
    const double d6 = (s.dens[(i1 + 0) * 5 + j1 + 1][k1 + 1] - d2) * d0;
    const double d7 = (s.dens[(i1 + 1) * 5 + j1 + 0][k1 + 1] - d3) * d0;
    const double d8 = (s.dens[(i1 + 1) * 5 + j1 + 1][k1 + 1] - d4) * d0;
    const long long plane = static_cast<long long>(d.SX) * d.SZ;
    for (int l1 = 0; l1 < 8; ++l1) {
        double d10 = d1, d11 = d2;
        const double d12 = (d3 - d1) * 0.25;
        const double d13 = (d4 - d2) * 0.25;
        const int y = k1 * 8 + l1;
#pragma unroll
        for (int i2 = 0; i2 < 4; ++i2) {
            double d15 = d10;
            const double d16 = (d11 - d10) * 0.25;
            const int X = a * 16 + i1 * 4 + i2;
#pragma unroll
            for (int k2 = 0; k2 < 4; ++k2) {
                if (y >= FLOOR_Y - 1) {
                    const int Z = b * 16 + j1 * 4 + k2;
                    stone[(y - (FLOOR_Y - 1)) * plane + static_cast<long long>(X) * d.SZ + Z] = d15 > 0.0 ? 1 : 0;
                }
                d15 += d16;
            }
            d10 += d12;
            d11 += d13;
        }
        d1 += d5; d2 += d6; d3 += d7; d4 += d8;
    }
}

__device__ __forceinline__ int find_root(const int* L, int x) {
    for (int guard = 0; guard < (1 << 22); ++guard) {
        const int p = L[x];
        if (p == x) return x;
        x = p;
    }
    return x;
}

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

// Initial labels: each run of stone cells along z within a warp's 32 cells
// points to the run's first cell, which needs no atomics; a row start (z == 0)
// also starts a run. Planes are (16 nc)^2 = 256 nc^2 cells and the launches use
// 256-thread blocks, so every warp is full and its cells 32-aligned. Levels
// below the floor plane are not labelled.
__global__ void k_cc_init(const std::uint8_t* __restrict__ stone, int* __restrict__ L, int* __restrict__ aux, Dims d) {
    const long long plane = static_cast<long long>(d.SX) * d.SZ;
    const int lane = threadIdx.x & 31;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < d.cells;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const bool on = c >= plane && stone[c];
        const int z = static_cast<int>((c % plane) % d.SZ);
        const unsigned onMask = __ballot_sync(0xffffffffu, on);
        const bool first = on && (lane == 0 || z == 0 || !((onMask >> (lane - 1)) & 1u));
        const unsigned starts = __ballot_sync(0xffffffffu, first);
        const unsigned upTo = starts & (lane == 31 ? 0xffffffffu : ((2u << lane) - 1u));
        const int runStart = 31 - __clz(upTo);  // on => upTo != 0
        L[c] = on ? static_cast<int>(c) - (lane - runStart) : -1;
        aux[c] = -1;
    }
}

// Unions of 6-neighbouring stone cells. Along z only across warp segments
// (inside one, a run already shares its label); along x and y only where the
// previous cell of the run did not already link the same two runs (then its
// union, and the z-links on both sides, connect this pair too).
__global__ void k_cc_union(const std::uint8_t* __restrict__ stone, int* L, Dims d, int* err) {
    const long long plane = static_cast<long long>(d.SX) * d.SZ;
    const int lane = threadIdx.x & 31;
    for (long long c = plane + blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < d.cells;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (!stone[c]) continue;
        const long long rem = c % plane;
        const int x = static_cast<int>(rem / d.SZ), z = static_cast<int>(rem % d.SZ);
        const bool prev = z > 0 && stone[c - 1];
        if (lane == 31 && z + 1 < d.SZ && stone[c + 1]) unite(L, static_cast<int>(c), static_cast<int>(c + 1), err);
        if (x + 1 < d.SX && stone[c + d.SZ] && !(prev && stone[c - 1 + d.SZ]))
            unite(L, static_cast<int>(c), static_cast<int>(c + d.SZ), err);
        if (c + plane < d.cells && stone[c + plane] && !(prev && stone[c - 1 + plane]))
            unite(L, static_cast<int>(c), static_cast<int>(c + plane), err);
    }
}

__global__ void k_cc_flatten(int* L, Dims d) {
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < d.cells;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (L[c] >= 0) L[c] = find_root(L, static_cast<int>(c));
    }
}

// Candidate starts: local x, z in {4, 12}, y >= 68, stone with non-stone below
// (IslandSearchEngine.java:2909-2924, :4005-4007). Candidate i enumerates
// (chunk a*nc+b, column k, y) in the Java scan order.
__device__ __forceinline__ bool candidate_cell(const std::uint8_t* stone, const Dims& d, int i, long long& cell,
                                               int& key) {
    const int perChunk = 4 * (128 - FLOOR_Y);
    const int chunk = i / perChunk;
    const int rem = i % perChunk;
    const int k = rem / (128 - FLOOR_Y);
    const int y = FLOOR_Y + rem % (128 - FLOOR_Y);
    const int a = chunk / d.nc, b = chunk % d.nc;
    const int X = a * 16 + ((k >> 1) ? 12 : 4);
    const int Z = b * 16 + ((k & 1) ? 12 : 4);
    const long long plane = static_cast<long long>(d.SX) * d.SZ;
    cell = static_cast<long long>(y - (FLOOR_Y - 1)) * plane + static_cast<long long>(X) * d.SZ + Z;
    key = (chunk * 4 + k) * 128 + y;
    return stone[cell] && !stone[cell - plane];
}

__global__ void k_cc_mark(const std::uint8_t* __restrict__ stone, const int* __restrict__ L, int* aux, Dims d) {
    const int total = d.nc * d.nc * 4 * (128 - FLOOR_Y);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        long long cell;
        int key;
        if (candidate_cell(stone, d, i, cell, key)) aux[L[cell]] = -2;
    }
}

__global__ void k_cc_slots(int* aux, Dims d, int* nslots) {
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < d.cells;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (aux[c] == -2) aux[c] = atomicAdd(nslots, 1);
    }
}

__global__ void k_slot_init(SlotStats st, int cap) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        st.blocks[i] = 0;
        st.columns[i] = 0;
        st.minX[i] = INT_MAX;
        st.maxX[i] = INT_MIN;
        st.minZ[i] = INT_MAX;
        st.maxZ[i] = INT_MIN;
        st.minY[i] = INT_MAX;
        st.maxY[i] = INT_MIN;
        st.flags[i] = 0;
        st.firstCand[i] = INT_MAX;
        st.sumX[i] = 0;
        st.sumZ[i] = 0;
    }
}

__global__ void k_cc_cand(const std::uint8_t* __restrict__ stone, const int* __restrict__ L,
                          const int* __restrict__ aux, Dims d, SlotStats st) {
    const int total = d.nc * d.nc * 4 * (128 - FLOOR_Y);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        long long cell;
        int key;
        if (candidate_cell(stone, d, i, cell, key)) atomicMin(&st.firstCand[aux[L[cell]]], key);
    }
}

// Per-cell statistics of candidate components (floodFillFlat, :4131-4186).
// A warp's 32 consecutive cells run along z and mostly share one component, so
// the lanes are grouped by slot and each group's counts, extremes and flags are
// reduced in registers; one lane per group updates the slot. (One atomic per
// cell serialises on the slots of large components.)
__global__ void k_cc_stats(const std::uint8_t* __restrict__ stone, const int* __restrict__ L,
                           const int* __restrict__ aux, Dims d, SlotStats st) {
    const long long plane = static_cast<long long>(d.SX) * d.SZ;
    const int lane = threadIdx.x & 31;
    for (long long c = plane + blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < d.cells;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int r = L[c];
        const int slot = r < 0 ? -1 : aux[r];
        const unsigned group = __match_any_sync(__activemask(), slot);
        if (slot < 0) continue;
        const int ys = static_cast<int>(c / plane);
        const long long rem = c % plane;
        const int x = static_cast<int>(rem / d.SZ), z = static_cast<int>(rem % d.SZ);
        const int wx = d.minWorldX + x, wz = d.minWorldZ + z, y = ys + (FLOOR_Y - 1);
        int f = 0;
        if (x == 0 || x == d.SX - 1 || z == 0 || z == d.SZ - 1) f |= FLAG_SIDE;
        // At the flood floor a stone block directly below grounds the component (:4173-4179).
        if (y == FLOOR_Y && stone[c - plane]) f |= FLAG_BOTTOM;
        const int minX = __reduce_min_sync(group, wx), maxX = __reduce_max_sync(group, wx);
        const int minZ = __reduce_min_sync(group, wz), maxZ = __reduce_max_sync(group, wz);
        const int minY = __reduce_min_sync(group, y), maxY = __reduce_max_sync(group, y);
        const unsigned flags = __reduce_or_sync(group, static_cast<unsigned>(f));
        if (lane == __ffs(group) - 1) {
            atomicAdd(&st.blocks[slot], __popc(group));
            atomicMin(&st.minX[slot], minX);
            atomicMax(&st.maxX[slot], maxX);
            atomicMin(&st.minZ[slot], minZ);
            atomicMax(&st.maxZ[slot], maxZ);
            atomicMin(&st.minY[slot], minY);
            atomicMax(&st.maxY[slot], maxY);
            if (flags) atomicOr(&st.flags[slot], static_cast<int>(flags));
        }
    }
}

// Distinct (x, z) columns of each candidate component and their world-coordinate sums.
__global__ void k_cc_columns(const int* __restrict__ L, const int* __restrict__ aux, Dims d, SlotStats st) {
    const long long plane = static_cast<long long>(d.SX) * d.SZ;
    const int cols = d.SX * d.SZ;
    for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < cols; col += gridDim.x * blockDim.x) {
        const int x = col / d.SZ, z = col % d.SZ;
        int seen[32];
        int nseen = 0;
        for (int ys = 1; ys < SY; ++ys) {
            const int r = L[ys * plane + col];
            if (r < 0) continue;
            const int slot = aux[r];
            if (slot < 0) continue;
            bool first = true;
            for (int k = 0; k < nseen; ++k) first = first && seen[k] != slot;
            if (!first) continue;
            if (nseen < 32) seen[nseen++] = slot;
            atomicAdd(&st.columns[slot], 1);
            atomicAdd(&st.sumX[slot], static_cast<unsigned long long>(static_cast<long long>(d.minWorldX + x)));
            atomicAdd(&st.sumZ[slot], static_cast<unsigned long long>(static_cast<long long>(d.minWorldZ + z)));
        }
    }
}

struct Cand {
    int slot, blocks, columns, area, first;
};

__device__ __forceinline__ bool better(const Cand& a, const Cand& b) {
    // compareComponents(a, b) > 0, ties resolved by the earlier flood (first candidate start).
    if (a.slot < 0) return false;
    if (b.slot < 0) return true;
    if (a.blocks != b.blocks) return a.blocks > b.blocks;
    if (a.columns != b.columns) return a.columns > b.columns;
    if (a.area != b.area) return a.area > b.area;
    return a.first < b.first;
}

__device__ __forceinline__ int java_round_div(long long sum, int n) {
    const double v = static_cast<double>(sum) / static_cast<double>(n);
    const double f = floor(v);
    return static_cast<int>(v - f >= 0.5 ? f + 1.0 : f);
}

__global__ void __launch_bounds__(1024) k_cc_best(const int* nslots, SlotStats st, MatchSettings ms, Dims d,
                                                  Island* out, int* bestSlot) {
    __shared__ Cand red[1024];
    const int n = *nslots;
    Cand mine{-1, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int blocks = st.blocks[i], columns = st.columns[i];
        const int width = st.maxX[i] - st.minX[i] + 1, depth = st.maxZ[i] - st.minZ[i] + 1;
        // isMatch (IslandSearchEngine.java:3972-4003)
        bool ok = blocks >= ms.minBlocks && columns >= ms.minColumns && st.maxY[i] >= ms.minYForMatch &&
                  !(st.flags[i] & FLAG_BOTTOM) && width >= ms.minWidth && depth >= ms.minDepth;
        if (ok) {
            const double avg = static_cast<double>(blocks) / static_cast<double>(columns > 1 ? columns : 1);
            ok = avg >= ms.minAvgThickness;
        }
        if (!ok) continue;
        const Cand c{i, blocks, columns, width * depth, st.firstCand[i]};
        if (better(c, mine)) mine = c;
    }
    red[threadIdx.x] = mine;
    __syncthreads();
    for (int off = 512; off > 0; off >>= 1) {
        if (threadIdx.x < off && better(red[threadIdx.x + off], red[threadIdx.x])) red[threadIdx.x] = red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const Cand b = red[0];
        Island isl;
        isl.radiusUsed = d.r;
        isl.sumX = isl.sumZ = 0;
        if (b.slot < 0) {
            isl.found = 0;
            isl.blocks = isl.columns = isl.minX = isl.maxX = isl.minZ = isl.maxZ = isl.minY = isl.maxY = 0;
            isl.centerX = isl.centerZ = isl.touchesSide = isl.touchesBottom = 0;
        } else {
            const int i = b.slot;
            isl.found = 1;
            isl.blocks = st.blocks[i];
            isl.columns = st.columns[i];
            isl.minX = st.minX[i]; isl.maxX = st.maxX[i];
            isl.minZ = st.minZ[i]; isl.maxZ = st.maxZ[i];
            isl.minY = st.minY[i]; isl.maxY = st.maxY[i];
            isl.sumX = static_cast<long long>(st.sumX[i]);
            isl.sumZ = static_cast<long long>(st.sumZ[i]);
            isl.centerX = java_round_div(isl.sumX, isl.columns);
            isl.centerZ = java_round_div(isl.sumZ, isl.columns);
            isl.touchesSide = (st.flags[i] & FLAG_SIDE) ? 1 : 0;
            isl.touchesBottom = (st.flags[i] & FLAG_BOTTOM) ? 1 : 0;
        }
        *out = isl;
        *bestSlot = b.slot;
    }
}

// Per-column lowest / highest y of the chosen component over its bounding box
// (buildPreviewData + buildIsland3DData, IslandSearchEngine.java:389-436, 5496-5636).
__global__ void k_preview(const int* __restrict__ L, const int* __restrict__ aux, Dims d, const Island* isl,
                          const int* bestSlot, int* minY, int* maxY, int capacity) {
    const int slot = *bestSlot;
    if (slot < 0) return;
    const int width = isl->maxX - isl->minX + 1, depth = isl->maxZ - isl->minZ + 1;
    if (width * depth > capacity) return;
    const long long plane = static_cast<long long>(d.SX) * d.SZ;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < width * depth; t += gridDim.x * blockDim.x) {
        const int x = isl->minX - d.minWorldX + t / depth;
        const int z = isl->minZ - d.minWorldZ + t % depth;
        int lo = INT_MAX, hi = INT_MIN;
        for (int ys = 1; ys < SY; ++ys) {
            const int r = L[ys * plane + static_cast<long long>(x) * d.SZ + z];
            if (r >= 0 && aux[r] == slot) {
                const int y = ys + (FLOOR_Y - 1);
                lo = min(lo, y);
                hi = max(hi, y);
            }
        }
        minY[t] = lo;
        maxY[t] = hi;
    }
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

std::size_t align256(std::size_t v) { return (v + 255) & ~static_cast<std::size_t>(255); }

}  // namespace

int exact_lattice_side(int radius) { return 8 * radius + 5; }

std::size_t exact_scratch_bytes(int R) {
    const Dims d = make_dims(R, 0, 0);
    const std::size_t cols = static_cast<std::size_t>(d.side) * d.side;
    std::size_t total = 0;
    total += align256(cols * 17 * 8) * 3 + align256(cols * 8) * 2;      // lattice
    total += align256(static_cast<std::size_t>(d.cells));               // stone
    total += align256(static_cast<std::size_t>(d.cells) * 4) * 2;       // labels, aux
    total += align256(slot_bytes(d.slotCap));                           // slot stats
    total += align256(64) * 3;                                          // nslots, best slot, err
    return total;
}

void exact_scratch_carve(ExactScratch& s, void* base, int R) {
    const Dims d = make_dims(R, 0, 0);
    const std::size_t cols = static_cast<std::size_t>(d.side) * d.side;
    char* p = static_cast<char*>(base);
    auto take = [&](std::size_t bytes) { char* q = p; p += align256(bytes); return q; };
    s.lattice.n1 = reinterpret_cast<double*>(take(cols * 17 * 8));
    s.lattice.n2 = reinterpret_cast<double*>(take(cols * 17 * 8));
    s.lattice.n3 = reinterpret_cast<double*>(take(cols * 17 * 8));
    s.lattice.n4 = reinterpret_cast<double*>(take(cols * 8));
    s.lattice.n5 = reinterpret_cast<double*>(take(cols * 8));
    s.lattice.columnsPerJob = cols;
    s.stone = reinterpret_cast<std::uint8_t*>(take(static_cast<std::size_t>(d.cells)));
    s.labels = reinterpret_cast<int*>(take(static_cast<std::size_t>(d.cells) * 4));
    s.compStats = reinterpret_cast<int*>(take(static_cast<std::size_t>(d.cells) * 4));  // aux map
    s.chunkDensity = reinterpret_cast<double*>(take(slot_bytes(d.slotCap)));          // slot statistics
    s.best = reinterpret_cast<unsigned long long*>(take(64));                          // nslots, best slot
    s.err = reinterpret_cast<int*>(take(64));
    s.jobs = reinterpret_cast<LatticeJob*>(take(64));
    s.maxRadius = R;
}

void launch_exact_scan(const StateCache& cache, int world, int ccx, int ccz, int radius, const MatchSettings& ms,
                       ExactScratch& s, Island* dIsland, int* dPreviewMinY, int* dPreviewMaxY, int previewCapacity,
                       bool reuseLattice, cudaStream_t stream) {
    if (radius < 0 || radius > s.maxRadius) throw std::runtime_error("exact scan radius exceeds scratch");
    const Dims d = make_dims(radius, ccx, ccz);
    LatticeBuffers lat = s.lattice;
    lat.columnsPerJob = static_cast<std::size_t>(d.side) * d.side;
    if (!reuseLattice) {
        LatticeJob job{world, (ccx - radius) * 4, (ccz - radius) * 4, d.side};
        launch_lattice_noise_one(cache, job, lat, stream);
    }
    static std::once_flag attr;  // handles on several threads launch this kernel
    std::call_once(attr, [] {
        check(cudaFuncSetAttribute(k_exact_chunks, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(ChunkSmem)),
              "exact smem");
    });
    k_exact_chunks<<<d.nc * d.nc, 128, sizeof(ChunkSmem), stream>>>(cache, world, d, lat, s.stone);
    check(cudaGetLastError(), "k_exact_chunks");
    int* aux = s.compStats;
    int* nslots = reinterpret_cast<int*>(s.best);
    int* bestSlot = nslots + 1;
    SlotStats st = carve_slots(reinterpret_cast<int*>(s.chunkDensity), d.slotCap);
    const int grid = 152 * 8;
    check(cudaMemsetAsync(nslots, 0, 8, stream), "memset");
    k_cc_init<<<grid, 256, 0, stream>>>(s.stone, s.labels, aux, d);
    k_cc_union<<<grid, 256, 0, stream>>>(s.stone, s.labels, d, s.err);
    k_cc_flatten<<<grid, 256, 0, stream>>>(s.labels, d);
    k_cc_mark<<<grid, 256, 0, stream>>>(s.stone, s.labels, aux, d);
    k_cc_slots<<<grid, 256, 0, stream>>>(aux, d, nslots);
    k_slot_init<<<grid, 256, 0, stream>>>(st, d.slotCap);
    k_cc_cand<<<grid, 256, 0, stream>>>(s.stone, s.labels, aux, d, st);
    k_cc_stats<<<grid, 256, 0, stream>>>(s.stone, s.labels, aux, d, st);
    k_cc_columns<<<grid, 256, 0, stream>>>(s.labels, aux, d, st);
    k_cc_best<<<1, 1024, 0, stream>>>(nslots, st, ms, d, dIsland, bestSlot);
    if (dPreviewMinY && dPreviewMaxY)
        k_preview<<<grid, 256, 0, stream>>>(s.labels, aux, d, dIsland, bestSlot, dPreviewMinY, dPreviewMaxY,
                                            previewCapacity);
    check(cudaGetLastError(), "exact scan kernels");
}

}  // namespace bsf
