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
#include "bsf_screen.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
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

// The incremental trilinear fill of one cell (generateBareTerrain,
// BetaTerrain173.java:582-665) in the reference's FP64 operations: cell
// (i1, j1) of chunk (a, b) at y-cell k1 (y 8 k1 .. 8 k1 + 7) from its corner
// densities at levels k1 (lo) and k1 + 1 (hi), in the order (x, z), (x, z + 1),
// (x + 1, z), (x + 1, z + 1). Stone cells at y >= 67 are stored.
__device__ __forceinline__ void fill_cell_fp64(const double (&lo)[4], const double (&hi)[4], const Dims& d, int a,
                                               int b, int i1, int j1, int k1, std::uint8_t* __restrict__ stone) {
    const double d0 = 0.125;
    double d1 = lo[0], d2 = lo[1], d3 = lo[2], d4 = lo[3];
    const double d5 = (hi[0] - d1) * d0;
    const double d6 = (hi[1] - d2) * d0;
    const double d7 = (hi[2] - d3) * d0;
    const double d8 = (hi[3] - d4) * d0;
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
    const double lo[4] = {s.dens[i1 * 5 + j1][k1], s.dens[i1 * 5 + j1 + 1][k1], s.dens[(i1 + 1) * 5 + j1][k1],
                          s.dens[(i1 + 1) * 5 + j1 + 1][k1]};
    const double hi[4] = {s.dens[i1 * 5 + j1][k1 + 1], s.dens[i1 * 5 + j1 + 1][k1 + 1],
                          s.dens[(i1 + 1) * 5 + j1][k1 + 1], s.dens[(i1 + 1) * 5 + j1 + 1][k1 + 1]};
    fill_cell_fp64(lo, hi, d, a, b, i1, j1, k1, stone);
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

// ---- screened fill (the queued forms) -------------------------------------
// The FP64 fill above evaluates every lattice point of a scan in FP64; on
// GB300 a CTA of that lattice kernel holds an SM for about half a millisecond
// of FP64 work, which inside the pipelined range is SM time taken from the
// next batch's Stage0. The screened fill does the same scan with the FP64
// work confined to the points the result depends on:
//   k_lattice_fast: per lattice column noise1..3 at levels 8..15 in FP32
//     (bsf_screen.cuh: double-float axis entries, E_OCT3 per octave, the sums
//     in the reference's order with their octave_sum_bound), and noise4 and
//     noise5 in exact FP64 (26 2D octaves), so that d7 and the d5 branch are
//     the reference's values and d5 carries only the climate's FP32 bound;
//   k_chunks_screen: per chunk the climate (FP32) and the corner densities
//     with their bounds, then per cell the incremental fill in FP32. A cell
//     whose blocks at y >= 67 all lie outside their bound stores its stone
//     bytes; any other cell is listed, and its 8 corner (column, level) pairs
//     are marked;
//   k_pack_points, k_points_fp64: noise1..3 in FP64 at the marked pairs only,
//     packed densely (a few per cent of the lattice's points);
//   k_cells_fp64: the listed cells with the FP64 climate, shape, densities and
//     fill_cell_fp64 of k_exact_chunks.
// A stone byte is thus either certain from the screen or computed by the FP64
// operations of the FP64 fill, and equal to its byte either way.
using namespace screen;

constexpr int NOCT = 66;
constexpr int LAT_FIELDS = 3 * 8;                      // FP32 noise1, noise2, noise3 at levels 8..15
constexpr float E_N16 = octave_sum_bound(16, E_OCT3);  // noise2 / noise3 summed as the reference does

__constant__ float2 ce_octave_scale[NOCT];  // octave_scale(o) split into a float pair

// One lattice row's setup: generators, offsets (and as float pairs for the
// axis entries), the FP32 Y axes and the row's X axis entries.
struct RowSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];
    double off[ST_COUNT][3];
    float2 offSplit[NOCT][2];
    YF yf[OCT3][17];
    AxisF ax[NOCT];
};

__device__ __forceinline__ double octave_scale_dev(int o) {
    if (o < 16) return NOISE_XZ * exp2_neg(o);
    if (o < 32) return NOISE_XZ * exp2_neg(o - 16);
    if (o < 40) return (NOISE_XZ / 80.0) * exp2_neg(o - 32);
    if (o < 50) return 1.121 * exp2_neg(o - 40);
    return 200.0 * exp2_neg(o - 50);
}

// Axis entry of octave o at lattice coordinate `coord` on axis a (0: x, 1: z):
// double-float, or FP64 where a floor is too close to call.
__device__ __forceinline__ AxisF lattice_axis(const RowSmem& s, int o, int a, int coord) {
    const float2 sc = ce_octave_scale[o];
    const float2 of = s.offSplit[o][a];
    AxisF r;
    if (!make_axis_df(coord, DF{sc.x, sc.y}, DF{of.x, of.y}, r))
        r = make_axis(static_cast<double>(coord) * octave_scale_dev(o), s.off[o][a == 0 ? 0 : 2]);
    return r;
}

// Lattice row kx = blockIdx.x, one thread per column z: FP32 noise1..3 into
// lat32[field * side^2 + kx * side + z], FP64 noise4/5 into the FP64 lattice.
__global__ void __launch_bounds__(256) k_lattice_fast(StateCache cache, int world, int originX, int originZ, int side,
                                                      float* __restrict__ lat32, LatticeBuffers lat) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RowSmem& s = *reinterpret_cast<RowSmem*>(smem_raw);
    const int tid = threadIdx.x, kx = blockIdx.x;
    {
        const uint4* src = reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(world) * WORLD_PERM_BYTES);
        uint4* dst = reinterpret_cast<uint4*>(s.perm);
        for (int k = tid; k < ST_TEMP * PERM_BYTES / 16; k += blockDim.x) dst[k] = src[k];
        const double* o = cache.offsets + static_cast<std::size_t>(world) * WORLD_OFFSETS;
        for (int k = tid; k < ST_COUNT * 3; k += blockDim.x) {
            const double v = o[(k / 3) * 4 + (k % 3)];
            s.off[k / 3][k % 3] = v;
            if (k / 3 < NOCT && k % 3 != 1) {
                const DF dv = df_of(v);
                s.offSplit[k / 3][(k % 3) / 2] = make_float2(dv.h, dv.l);
            }
        }
    }
    __syncthreads();
    if (tid < OCT3) {
        const int k = tid < 16 ? tid : (tid < 32 ? tid - 16 : tid - 32);
        const double amp = exp2_neg(k);
        const double sy = tid < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
        YEntry ya[17];
        build_yaxis(sy, s.off[tid][1], ya);
        build_yf(ya, s.yf[tid]);
    } else if (tid >= 64 && tid < 64 + NOCT) {
        s.ax[tid - 64] = lattice_axis(s, tid - 64, 0, originX + kx);
    }
    __syncthreads();
    const int z = tid;
    if (z >= side) return;
    const int coordZ = originZ + z;
    float a1[8], a2[8], a3[8];
#pragma unroll 1
    for (int o = 0; o < 16; ++o) {
        const int st = ST_N2 + o;
        octave3f<8, 8>(s.perm + st * PERM_BYTES, s.ax[st], lattice_axis(s, st, 1, coordZ), s.yf[st],
                       static_cast<float>(1 << o), a2, o == 0);
    }
#pragma unroll 1
    for (int o = 0; o < 16; ++o) {
        const int st = ST_N3 + o;
        octave3f<8, 8>(s.perm + st * PERM_BYTES, s.ax[st], lattice_axis(s, st, 1, coordZ), s.yf[st],
                       static_cast<float>(1 << o), a3, o == 0);
    }
#pragma unroll 1
    for (int o = 0; o < 8; ++o) {
        const int st = ST_N1 + o;
        octave3f<8, 8>(s.perm + st * PERM_BYTES, s.ax[st], lattice_axis(s, st, 1, coordZ), s.yf[st],
                       static_cast<float>(1 << o), a1, o == 0);
    }
    const std::size_t cols = static_cast<std::size_t>(side) * side, c = static_cast<std::size_t>(kx) * side + z;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        lat32[k * cols + c] = a1[k];
        lat32[(8 + k) * cols + c] = a2[k];
        lat32[(16 + k) * cols + c] = a3[k];
    }
    GenTable t;
    t.perm = s.perm;
    t.off = &s.off[0][0];
    noise45(t, static_cast<double>(originX + kx), static_cast<double>(coordZ), lat.n4[c], lat.n5[c]);
}

// d7 and the d6 < 0 branch of column_shape (bsf_device.cuh) from noise5, in the
// same FP64 operations.
__device__ __forceinline__ double shape_d7_exact(double n5, bool& zeroD5) {
    double d6 = n5 / 8000.0;
    if (d6 < 0.0) d6 = -d6 * 0.3;
    d6 = d6 * 3.0 - 2.0;
    zeroD5 = d6 < 0.0;
    if (zeroD5) {
        d6 /= 2.0;
        if (d6 < -1.0) d6 = -1.0;
        d6 /= 1.4;
        d6 /= 2.0;
    } else {
        if (d6 > 1.0) d6 = 1.0;
        d6 /= 8.0;
    }
    d6 = d6 * 17.0 / 16.0;
    return 17.0 / 2.0 + d6 * 4.0;
}

// density_at (BetaTerrain173.java:808-830) in FP32 with its bound, levels 8..15.
// Where the selector d12 is within its bound of 0 or 1, the lerp with d12
// clamped to [0, 1] covers both of the reference's branches (clamping is
// 1-Lipschitz and the lerp at 0 / 1 is d10 / d11).
__device__ __forceinline__ Fe density_fe(int y, Fe d5, Fe d7, Fe n1, Fe n2, Fe n3) {
    const Fe d9 = level_d9(y, d5, d7);
    const Fe d10{n2.v * (1.0f / 512.0f), n2.e * (1.0f / 512.0f)};
    const Fe d11{n3.v * (1.0f / 512.0f), n3.e * (1.0f / 512.0f)};
    const Fe d12 = fe_scale(fe_add(fe_div(n1, Fe{10.0f, 0.0f}), Fe{1.0f, 0.0f}), 0.5f);
    Fe d8;
    if (d12.v + d12.e < 0.0f) {
        d8 = d10;
    } else if (d12.v - d12.e > 1.0f) {
        d8 = d11;
    } else {
        const Fe t = fe_clamp_hi(fe_clamp_lo(d12, 0.0f), 1.0f);
        d8 = fe_add(d10, fe_mul(fe_sub(d11, d10), t));
    }
    Fe d = fe_sub(d8, d9);
    if (y > 13) {
        const float d13 = static_cast<float>(y - 13) / 3.0f;  // exact as the reference's float division
        d = fe_add(fe_mul(d, Fe{1.0f - d13, 2.0f * U}), Fe{-10.0f * d13, 20.0f * U});
    }
    return d;
}

struct ScreenChunkSmem {
    std::uint8_t perm[ST_COUNT * PERM_BYTES];  // the climate generators' part is staged
    double off[ST_COUNT][3];
    float4 clim[10];
    float dv[25][9], de[25][9];  // corner densities at levels 8..16 and their bounds
};

// One chunk of the screened fill (see above). Cell list entries are
// chunk << 7 | cell, cell = i1 << 5 | j1 << 3 | (k1 - 8) as in k_exact_chunks;
// needBits has a bit per (lattice column, level 8..16): column * 9 + level - 8.
__global__ void __launch_bounds__(128) k_chunks_screen(StateCache cache, int world, Dims d,
                                                       const float* __restrict__ lat32, LatticeBuffers lat,
                                                       std::uint8_t* __restrict__ stone,
                                                       std::uint32_t* __restrict__ needBits,
                                                       int* __restrict__ cellList, int* __restrict__ cellCount) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScreenChunkSmem& s = *reinterpret_cast<ScreenChunkSmem*>(smem_raw);
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
    if (tid < 10) s.clim[tid] = climate_split(s.off[ST_TEMP + tid]);
    __syncthreads();
    const std::size_t cols = static_cast<std::size_t>(d.side) * d.side;
    if (tid < 25) {
        const int i = tid / 5, j = tid % 5;
        GenTable t;
        t.perm = s.perm;
        t.off = &s.off[0][0];
        const std::size_t col = static_cast<std::size_t>(a * 4 + i) * d.side + (b * 4 + j);
        bool zeroD5 = false;
        const double d7x = shape_d7_exact(lat.n5[col], zeroD5);
        const float d7f = static_cast<float>(d7x);
        const Fe d7{d7f, fabsf(d7f) * U};
        Fe d5{0.5f, 0.0f};
        if (!zeroD5) {
            Fe temp, rain;
            climate_f(t, s.clim, chunkX * 16 + i * 3 + 1, chunkZ * 16 + j * 3 + 1, temp, rain);
            const float n4f = static_cast<float>(lat.n4[col]);
            d5 = shape_d5_f(temp, rain, Fe{n4f, fabsf(n4f) * U});
        }
#pragma unroll 1
        for (int y = 8; y < 16; ++y) {
            const Fe v = density_fe(y, d5, d7, Fe{lat32[(y - 8) * cols + col], E_N1},
                                    Fe{lat32[y * cols + col], E_N16}, Fe{lat32[(y + 8) * cols + col], E_N16});
            s.dv[tid][y - 8] = v.v;
            s.de[tid][y - 8] = v.e;
        }
        s.dv[tid][8] = -10.0f;  // level 16: d8 * 0.0 + -10.0 * 1.0 for any finite d8
        s.de[tid][8] = 0.0f;
    }
    __syncthreads();
    const int i1 = tid >> 5, j1 = (tid >> 3) & 3, k1 = 8 + (tid & 7);
    const int p[4] = {i1 * 5 + j1, i1 * 5 + j1 + 1, (i1 + 1) * 5 + j1, (i1 + 1) * 5 + j1 + 1};
    float lo[4], hi[4], emax = 0.0f, vmax = 0.0f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        lo[c] = s.dv[p[c]][k1 - 8];
        hi[c] = s.dv[p[c]][k1 - 7];
        emax = fmaxf(emax, fmaxf(s.de[p[c]][k1 - 8], s.de[p[c]][k1 - 7]));
        vmax = fmaxf(vmax, fmaxf(fabsf(lo[c]), fabsf(hi[c])));
    }
    // Every block value of the fill is a convex blend of the 8 corners, so it is
    // within emax of the blend of the reference's corners. The FP32 steps below
    // (at most 8 + 4 + 4 adds of steps whose own roundings repeat) add under
    // 16 u M, M bounding every intermediate, taken as 32 u M; the reference's
    // own FP64 steps are inside the absolute 1e-6. The bound is doubled as in
    // the other screened tests.
    const float m = vmax + emax;
    const float bound = 2.0f * (emax + 32.0f * U * m) + 1.0e-6f;
    std::uint32_t bits[4] = {0u, 0u, 0u, 0u};
    bool certain = true;
    {
        float d1 = lo[0], d2 = lo[1], d3 = lo[2], d4 = lo[3];
        const float d5 = (hi[0] - d1) * 0.125f, d6 = (hi[1] - d2) * 0.125f;
        const float d7 = (hi[2] - d3) * 0.125f, d8 = (hi[3] - d4) * 0.125f;
#pragma unroll
        for (int l1 = 0; l1 < 8; ++l1) {
            float d10 = d1, d11 = d2;
            const float d12 = (d3 - d1) * 0.25f, d13 = (d4 - d2) * 0.25f;
            const bool stored = k1 * 8 + l1 >= FLOOR_Y - 1;
#pragma unroll
            for (int i2 = 0; i2 < 4; ++i2) {
                float d15 = d10;
                const float d16 = (d11 - d10) * 0.25f;
#pragma unroll
                for (int k2 = 0; k2 < 4; ++k2) {
                    if (stored) {
                        certain = certain && fabsf(d15) > bound;  // false for NaN and infinite bounds too
                        bits[l1 >> 1] |= (d15 > 0.0f ? 1u : 0u) << ((l1 & 1) * 16 + i2 * 4 + k2);
                    }
                    d15 += d16;
                }
                d10 += d12;
                d11 += d13;
            }
            d1 += d5; d2 += d6; d3 += d7; d4 += d8;
        }
    }
    if (certain) {
        const long long plane = static_cast<long long>(d.SX) * d.SZ;
#pragma unroll 1
        for (int l1 = 0; l1 < 8; ++l1) {
            const int y = k1 * 8 + l1;
            if (y < FLOOR_Y - 1) continue;
#pragma unroll
            for (int i2 = 0; i2 < 4; ++i2) {
                const int X = a * 16 + i1 * 4 + i2;
#pragma unroll
                for (int k2 = 0; k2 < 4; ++k2) {
                    const int Z = b * 16 + j1 * 4 + k2;
                    stone[(y - (FLOOR_Y - 1)) * plane + static_cast<long long>(X) * d.SZ + Z] =
                        static_cast<std::uint8_t>((bits[l1 >> 1] >> ((l1 & 1) * 16 + i2 * 4 + k2)) & 1u);
                }
            }
        }
        return;
    }
    cellList[atomicAdd(cellCount, 1)] = (blockIdx.x << 7) | tid;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int col = (a * 4 + i1 + (c >> 1)) * d.side + (b * 4 + j1 + (c & 1));
#pragma unroll
        for (int dk = 0; dk < 2; ++dk) {
            const int bit = col * 9 + (k1 + dk - 8);
            atomicOr(&needBits[bit >> 5], 1u << (bit & 31));
        }
    }
}

// The marked (column, level) pairs as a dense list (any order: each entry
// writes its own lattice slot).
__global__ void k_pack_points(const std::uint32_t* __restrict__ needBits, int words, int* __restrict__ points,
                              int* __restrict__ pointCount) {
    const int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w - lane < words; w += gridDim.x * blockDim.x) {
        const std::uint32_t m = w < words ? needBits[w] : 0u;
        const int n = __popc(m);
        int incl = n;  // inclusive prefix of n over the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int base = 0;
        if (lane == 31 && total) base = atomicAdd(pointCount, total);
        base = __shfl_sync(0xffffffffu, base, 31) + incl - n;
        std::uint32_t r = m;
        while (r) {
            const int bit = __ffs(r) - 1;
            r &= r - 1;
            points[base++] = w * 32 + bit;
        }
    }
}

struct PointSmem {
    std::uint8_t perm[ST_TEMP * PERM_BYTES];
    double off[ST_TEMP][3];
    YEntry ytab[OCT3][17];
};

// FP64 noise1..3 at the listed (column, level) pairs into the FP64 lattice,
// one thread per pair: octave3_column's operations for that one level (the
// same lattice corners, cell corners and sample, summed over octaves in the
// reference's order), so every value equals the FP64 lattice kernel's.
constexpr int POINT_THREADS = 64;  // >= OCT3: the CTA builds the 40 Y axes
constexpr int CELL_THREADS = 64;

__global__ void __launch_bounds__(POINT_THREADS) k_points_fp64(StateCache cache, int world, int originX, int originZ, int side,
                                                     const int* __restrict__ points, const int* __restrict__ pointCount,
                                                     LatticeBuffers lat) {
    __shared__ __align__(16) PointSmem s;
    const int tid = threadIdx.x;
    const int n = *pointCount;
    if (static_cast<int>(blockIdx.x * blockDim.x) >= n) return;  // the whole CTA: no barrier below is skipped
    {
        const uint4* src = reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(world) * WORLD_PERM_BYTES);
        uint4* dst = reinterpret_cast<uint4*>(s.perm);
        for (int k = tid; k < ST_TEMP * PERM_BYTES / 16; k += blockDim.x) dst[k] = src[k];
        const double* o = cache.offsets + static_cast<std::size_t>(world) * WORLD_OFFSETS;
        for (int k = tid; k < ST_TEMP * 3; k += blockDim.x) s.off[k / 3][k % 3] = o[(k / 3) * 4 + (k % 3)];
    }
    __syncthreads();
    if (tid < OCT3) {
        const int k = tid < 16 ? tid : (tid < 32 ? tid - 16 : tid - 32);
        const double amp = exp2_neg(k);
        const double sy = tid < 32 ? NOISE_Y * amp : (NOISE_Y / 160.0) * amp;
        build_yaxis(sy, s.off[tid][1], s.ytab[tid]);
    }
    __syncthreads();
    GenTable t;
    t.perm = s.perm;
    t.off = &s.off[0][0];
    for (int idx = blockIdx.x * blockDim.x + tid; idx < n; idx += gridDim.x * blockDim.x) {
        const int e = points[idx];
        const int col = e / 9, y = 8 + e % 9;
        const double X = static_cast<double>(originX + col / side), Z = static_cast<double>(originZ + col % side);
        double v2 = 0.0, v3 = 0.0, v1 = 0.0, amp = 1.0;
#pragma unroll 1
        for (int o = 0; o < 16; ++o) {
            const double sc = NOISE_XZ * amp;
            const Gen g2 = t(ST_N2 + o), g3 = t(ST_N3 + o);
            const YEntry e2 = s.ytab[o][y], e3 = s.ytab[16 + o][y];
            double c00, c01, c10, c11;
            const Lattice3 L2 = lattice3(g2, X * sc, Z * sc);
            cell_corners(g2, L2, e2, c00, c01, c10, c11);
            const double w2 = cell_sample(L2, e2, c00, c01, c10, c11, 1.0 / amp);
            v2 = o == 0 ? 0.0 + w2 : v2 + w2;
            const Lattice3 L3 = lattice3(g3, X * sc, Z * sc);
            cell_corners(g3, L3, e3, c00, c01, c10, c11);
            const double w3 = cell_sample(L3, e3, c00, c01, c10, c11, 1.0 / amp);
            v3 = o == 0 ? 0.0 + w3 : v3 + w3;
            amp /= 2.0;
        }
        amp = 1.0;
#pragma unroll 1
        for (int o = 0; o < 8; ++o) {
            const double sc = (NOISE_XZ / 80.0) * amp;
            const Gen g1 = t(ST_N1 + o);
            const YEntry e1 = s.ytab[32 + o][y];
            double c00, c01, c10, c11;
            const Lattice3 L1 = lattice3(g1, X * sc, Z * sc);
            cell_corners(g1, L1, e1, c00, c01, c10, c11);
            const double w1 = cell_sample(L1, e1, c00, c01, c10, c11, 1.0 / amp);
            v1 = o == 0 ? 0.0 + w1 : v1 + w1;
            amp /= 2.0;
        }
        lat.n1[static_cast<std::size_t>(col) * 17 + y] = v1;
        lat.n2[static_cast<std::size_t>(col) * 17 + y] = v2;
        lat.n3[static_cast<std::size_t>(col) * 17 + y] = v3;
    }
}

// The listed cells of the screened fill in FP64 (see above): one thread per cell.
__global__ void __launch_bounds__(CELL_THREADS) k_cells_fp64(StateCache cache, int world, Dims d, LatticeBuffers lat,
                                                    const int* __restrict__ cellList, const int* __restrict__ cellCount,
                                                    std::uint8_t* __restrict__ stone) {
    __shared__ __align__(16) std::uint8_t perm[ST_COUNT * PERM_BYTES];  // the climate part is staged
    __shared__ double off[ST_COUNT][3];
    const int tid = threadIdx.x;
    const int n = *cellCount;
    if (static_cast<int>(blockIdx.x * blockDim.x) >= n) return;  // the whole CTA: no barrier below is skipped
    {
        const uint4* src = reinterpret_cast<const uint4*>(cache.perms + static_cast<std::size_t>(world) * WORLD_PERM_BYTES);
        uint4* dst = reinterpret_cast<uint4*>(perm);
        for (int k = tid + ST_TEMP * 16; k < WORLD_PERM_BYTES / 16; k += blockDim.x) dst[k] = src[k];
        const double* o = cache.offsets + static_cast<std::size_t>(world) * WORLD_OFFSETS;
        for (int k = tid; k < ST_COUNT * 3; k += blockDim.x) off[k / 3][k % 3] = o[(k / 3) * 4 + (k % 3)];
    }
    __syncthreads();
    GenTable t;
    t.perm = perm;
    t.off = &off[0][0];
    for (int idx = blockIdx.x * blockDim.x + tid; idx < n; idx += gridDim.x * blockDim.x) {
        const int e = cellList[idx];
        const int chunk = e >> 7, cell = e & 127;
        const int a = chunk / d.nc, b = chunk % d.nc;
        const int chunkX = d.ccx - d.r + a, chunkZ = d.ccz - d.r + b;
        const int i1 = cell >> 5, j1 = (cell >> 3) & 3, k1 = 8 + (cell & 7);
        double lo[4], hi[4];
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
            const int i = i1 + (c >> 1), j = j1 + (c & 1);
            double temp, rain, d5, d7;
            climate_at(t, chunkX * 16 + i * 3 + 1, chunkZ * 16 + j * 3 + 1, temp, rain);
            const std::size_t col = static_cast<std::size_t>(a * 4 + i) * d.side + (b * 4 + j);
            column_shape(temp, rain, lat.n4[col], lat.n5[col], d5, d7);
            lo[c] = density_at(k1, d5, d7, lat.n1[col * 17 + k1], lat.n2[col * 17 + k1], lat.n3[col * 17 + k1]);
            hi[c] = density_at(k1 + 1, d5, d7, lat.n1[col * 17 + k1 + 1], lat.n2[col * 17 + k1 + 1],
                               lat.n3[col * 17 + k1 + 1]);
        }
        fill_cell_fp64(lo, hi, d, a, b, i1, j1, k1, stone);
    }
}

std::size_t align256(std::size_t v) { return (v + 255) & ~static_cast<std::size_t>(255); }

}  // namespace

// Per device (constant memory and function attributes are per device), once,
// before any exact scan on it.
void init_exact_tables() {
    check(cudaFuncSetAttribute(k_exact_chunks, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(ChunkSmem)),
          "exact smem");
    check(cudaFuncSetAttribute(k_lattice_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(RowSmem)),
          "lattice smem");
    check(cudaFuncSetAttribute(k_chunks_screen, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(ScreenChunkSmem)),
          "screen smem");
    float2 scales[NOCT];
    for (int o = 0; o < NOCT; ++o) {  // octave_scale_dev(o) in the same IEEE operations
        const double base = o < 32 ? NOISE_XZ : (o < 40 ? NOISE_XZ / 80.0 : (o < 50 ? 1.121 : 200.0));
        const int k = o < 16 ? o : (o < 32 ? o - 16 : (o < 40 ? o - 32 : (o < 50 ? o - 40 : o - 50)));
        const double v = base * std::ldexp(1.0, -k);
        const float h = static_cast<float>(v);
        scales[o] = make_float2(h, static_cast<float>(v - static_cast<double>(h)));
    }
    check(cudaMemcpyToSymbol(ce_octave_scale, scales, sizeof(scales)), "octave scales");
}

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
    total += align256(cols * LAT_FIELDS * 4);                           // FP32 lattice
    total += align256((cols * 9 + 31) / 32 * 4);                        // (column, level) bits
    total += align256(cols * 9 * 4);                                    // packed pairs
    total += align256(static_cast<std::size_t>(d.nc) * d.nc * 128 * 4);  // FP64 cell list
    total += align256(64);                                              // counts
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
    s.lat32 = reinterpret_cast<float*>(take(cols * LAT_FIELDS * 4));
    s.needBits = reinterpret_cast<std::uint32_t*>(take((cols * 9 + 31) / 32 * 4));
    s.points = reinterpret_cast<int*>(take(cols * 9 * 4));
    s.cellList = reinterpret_cast<int*>(take(static_cast<std::size_t>(d.nc) * d.nc * 128 * 4));
    s.counts = reinterpret_cast<int*>(take(64));
    s.maxRadius = R;
}

int launch_exact_scan(const StateCache& cache, int world, int ccx, int ccz, int radius, const MatchSettings& ms,
                      ExactScratch& s, Island* dIsland, int* dPreviewMinY, int* dPreviewMaxY, int previewCapacity,
                      bool screened, cudaStream_t stream) {
    if (radius < 0 || radius > s.maxRadius) throw std::runtime_error("exact scan radius exceeds scratch");
    const Dims d = make_dims(radius, ccx, ccz);
    LatticeBuffers lat = s.lattice;
    lat.columnsPerJob = static_cast<std::size_t>(d.side) * d.side;
    const LatticeJob job{world, (ccx - radius) * 4, (ccz - radius) * 4, d.side};
    int launches = 0;
    if (screened) {
        // k_lattice_fast takes a lattice row per CTA and a column per thread
        if (d.side > 256) throw std::length_error("screened exact scan: radius above 31");
        const std::size_t cols = lat.columnsPerJob;
        const int words = static_cast<int>((cols * 9 + 31) / 32);
        check(cudaMemsetAsync(s.needBits, 0, static_cast<std::size_t>(words) * 4, stream), "memset");
        check(cudaMemsetAsync(s.counts, 0, 2 * sizeof(int), stream), "memset");
        k_lattice_fast<<<d.side, 256, sizeof(RowSmem), stream>>>(cache, world, job.originX, job.originZ, d.side,
                                                                  s.lat32, lat);
        k_chunks_screen<<<d.nc * d.nc, 128, sizeof(ScreenChunkSmem), stream>>>(
            cache, world, d, s.lat32, lat, s.stone, s.needBits, s.cellList, s.counts);
        k_pack_points<<<std::min((words + 255) / 256, 152), 256, 0, stream>>>(s.needBits, words, s.points,
                                                                              s.counts + 1);
        // grid-stride loops over the device-side counts; CTAs past them return at once
        // small CTAs: a CTA's points share one SM's FP64 pipe, so they set the latency
        static_assert(POINT_THREADS >= OCT3, "Y axes");
        k_points_fp64<<<std::min(static_cast<int>((cols * 9 + POINT_THREADS - 1) / POINT_THREADS), 152 * 8),
                        POINT_THREADS, 0, stream>>>(
            cache, world, job.originX, job.originZ, d.side, s.points, s.counts + 1, lat);
        k_cells_fp64<<<std::min(d.nc * d.nc * 2, 152 * 8), CELL_THREADS, 0, stream>>>(cache, world, d, lat, s.cellList, s.counts,
                                                                          s.stone);
        check(cudaGetLastError(), "screened fill");
        launches += 5;
    } else {
        launch_lattice_noise_one(cache, job, lat, stream);
        k_exact_chunks<<<d.nc * d.nc, 128, sizeof(ChunkSmem), stream>>>(cache, world, d, lat, s.stone);
        check(cudaGetLastError(), "k_exact_chunks");
        launches += 2;
    }
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
    launches += 10;
    if (dPreviewMinY && dPreviewMaxY) {
        k_preview<<<grid, 256, 0, stream>>>(s.labels, aux, d, dIsland, bestSlot, dPreviewMinY, dPreviewMaxY,
                                            previewCapacity);
        ++launches;
    }
    check(cudaGetLastError(), "exact scan kernels");
    return launches;
}

}  // namespace bsf
