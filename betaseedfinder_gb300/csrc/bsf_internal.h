// Internal host/device interfaces between the translation units of libbsf.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace bsf {

// Per-region Stage0 / P19 / coarse outcome (one per (world, centre)).
struct RegionInfo {
    double p19Score;      // NaN unless P19 was evaluated
    std::int32_t coarse;  // coarse score, 0 unless evaluated
    std::int16_t p20, upper, high;
    std::uint8_t p19Evaluated, p19Pass, p19Extreme, megaReject, coarseEvaluated, pad0;
    std::uint16_t fullY88, fullY96, fullY104, fullY112, y88Largest, y96Largest;
    std::uint8_t y88Width, y88Depth, y88Touches, y96Width, y96Depth, y96Touches;
    std::uint8_t pad1[2];
};
static_assert(sizeof(RegionInfo) == 48, "RegionInfo layout");

struct Profile {
    int p20MinCount, upperMinCount, highMinCount;
    double p19MinScore;
    int coarseMinCells;
    int megaTopologyFilter;
};
Profile profile_by_id(int id);

// Stream centres in chunks (gpu_p20_benchmark.cpp:7316-7317, GpuStage0Scout.java:19-21).
__host__ __device__ inline int center_chunk_x(int c) {
    return c == 1 || c == 3 || c == 7 ? 15 : (c == 4 || c == 5 ? -15 : 0);
}
__host__ __device__ inline int center_chunk_z(int c) {
    return c == 2 || c == 3 || c == 5 ? 15 : (c == 6 || c == 7 ? -15 : 0);
}

// One queued region for the coarse / exact stages.
struct RegionRef {
    std::int32_t world;   // index into the batch's seed/state arrays
    std::int32_t center;  // 0..7
};

// Device-resident per-world generator cache (21,888 B per world).
struct StateCache {
    std::uint8_t* perms = nullptr;  // [world][76][256]
    double* offsets = nullptr;      // [world][76][4] (a, b, c, 0)
    int capacity = 0;
};

// Exact-scan match settings (SearchSettings.java:39-45 defaults).
struct MatchSettings {
    int minBlocks, minColumns, minYForMatch, minWidth, minDepth;
    double minAvgThickness;
};

// Island component as IslandSearchEngine.Component (:6516-6536).
struct Island {
    std::int32_t found;
    std::int32_t blocks, columns;
    std::int32_t minX, maxX, minZ, maxZ, minY, maxY;
    std::int32_t centerX, centerZ;
    std::int32_t touchesSide, touchesBottom;
    std::int32_t radiusUsed;
    std::int64_t sumX, sumZ;
};

// ---- launches (all asynchronous on `stream`) ------------------------------
void init_lcg_tables();
void launch_world_init(const std::int64_t* dSeeds, int n, StateCache& cache, int* dFallbackCount,
                       cudaStream_t stream);
void launch_chunk_bitmaps(const StateCache& cache, int n, int chunkX, int chunkZ, std::uint8_t* dBitmaps,
                          std::uint64_t* dHashes, cudaStream_t stream);
// Stage0 + P19 for n worlds x centers; appends P19 survivors to the coarse queue.
void launch_stage0(const StateCache& cache, int n, int centers, const Profile& prof, double* dShapeScratch,
                   RegionInfo* dRegions, RegionRef* dCoarseQueue, int* dCoarseCount, int coarseCapacity,
                   cudaStream_t stream);
std::size_t stage0_shape_scratch_bytes(int capacity);

// Lattice noise (noise1..3 at 17 levels, noise4/5) for `count` lattices of
// side `side` starting at coarse (originX[i], originZ[i]) of world worlds[i].
struct LatticeJob {
    std::int32_t world;
    std::int32_t originX, originZ;  // coarse coordinates of lattice column (0,0)
    std::int32_t side;              // columns per axis
};
struct LatticeBuffers {
    double* n1 = nullptr;  // [job][side*side][17]
    double* n2 = nullptr;
    double* n3 = nullptr;
    double* n4 = nullptr;  // [job][side*side]
    double* n5 = nullptr;
    std::size_t columnsPerJob = 0;
};
// Levels 8..16 of n1/n2/n3 and n4/n5 of one exact-scan lattice.
void launch_lattice_noise_one(const StateCache& cache, const LatticeJob& job, const LatticeBuffers& buf,
                              cudaStream_t stream);
// Coarse stage for `count` queued regions whose lattices are in `buf` (side 61).
void launch_coarse_score(const StateCache& cache, const RegionRef* dQueue, const int* dCount, int maxCount,
                         const LatticeBuffers& buf, std::uint32_t* dSignScratch, int* dLabelScratch,
                         int* dStatScratch, RegionInfo* dRegions, int centers, cudaStream_t stream);
std::size_t coarse_scratch_bytes_per_region();
// Component score of coarse sign masks already in dSignScratch.
void launch_coarse_cc(const RegionRef* dQueue, const int* dCount, int maxCount, std::uint32_t* dSignScratch,
                      int* dLabelScratch, int* dStatScratch, RegionInfo* dRegions, int centers, cudaStream_t stream);

// Screened (FP32 + exact fallback) kernels: identical outputs, far fewer FP64 operations.
struct Stage0FastScratch {
    RegionRef* p19Queue = nullptr;   // regions that passed the P20/Upper/High gates
    std::uint8_t* highest = nullptr; // [slot][256] highest re-entry level per column (0xFF none)
    int* p19Count = nullptr;
    int p19Capacity = 0;
    unsigned long long* stats = nullptr;  // [0] stage0 column tasks, [1] their FP64 fallbacks,
                                          // [2] coarse column tasks, [3] their FP64 fallbacks
    int forceExact = 0;  // verification: treat every screened column task as undecided
};
void init_stage0_fast();
// persistent: one CTA per resident slot looping over worlds (fastest alone);
// otherwise one CTA per world, so CTAs retire every world and a higher-priority
// stream's kernels get SM slots without waiting for the whole batch.
void launch_stage0_fast(const StateCache& cache, int n, int centers, const Profile& prof, RegionInfo* dRegions,
                        RegionRef* dCoarseQueue, int* dCoarseCount, int coarseCapacity, const Stage0FastScratch& fs,
                        cudaStream_t stream, bool persistent = true);
// Launch-shape variants (threads x CTAs per SM) of the screened kernels, set by the autotuner.
int stage0_fast_variants();
const char* stage0_fast_variant_name(int v);
void set_stage0_fast_variant(int v);
int get_stage0_fast_variant();
int coarse_fast_variants();
const char* coarse_fast_variant_name(int v);
void set_coarse_fast_variant(int v);
int get_coarse_fast_variant();
void init_coarse_fast();
void launch_coarse_signs_fast(const StateCache& cache, const RegionRef* dQueue, const int* dCount, int maxCount,
                              std::uint32_t* dSigns, unsigned long long* stats, cudaStream_t stream,
                              bool persistent = true, bool forceExact = false);
// Stage0 sweep state on the device (bsf_sweep.cu): a seed cursor, the running
// survivor total and list, per-block survivor counts of the current batch and
// the stage pass counters.
struct SweepState {
    unsigned long long* next = nullptr;    // first seed of the next batch
    unsigned long long* total = nullptr;   // survivors in `out` so far
    int* blockCounts = nullptr;            // [sweep_blocks(capacity)]
    unsigned long long* stage = nullptr;   // [0] P20, [1] +Upper, [2] +high (regions), [3] surviving worlds
    std::int64_t* out = nullptr;           // survivor seeds in seed order
    unsigned long long outCap = 0;
};
int sweep_blocks(int n);
void launch_sweep_seeds(std::int64_t* dSeeds, int n, const SweepState& st, cudaStream_t stream);
// Counts the batch's gate passes and appends its surviving worlds' seeds, in order.
void launch_sweep_compact(const RegionInfo* dRegions, const std::int64_t* dSeeds, int n, int centers,
                          const Profile& prof, const SweepState& st, cudaStream_t stream);
// Persistent coarse-score grid for a queue of maxCount regions: label/stat scratch
// is per CTA (COARSE_CELLS ints of labels, 2 * COARSE_CELLS of stats) and the
// union-find retry-bound flag (one int) follows the stat scratch.
int coarse_score_ctas(int maxCount);

// Exact scan of one region at one radius; result in *dIsland (device).
struct ExactScratch {
    LatticeBuffers lattice;
    LatticeJob* jobs = nullptr;
    double* chunkDensity = nullptr;  // [chunks][25][17]
    std::uint8_t* stone = nullptr;   // [X][61][Z] (y 67..127)
    int* labels = nullptr;           // [X][60][Z]
    int* compStats = nullptr;        // per-root statistics (see bsf_exact.cu)
    unsigned long long* best = nullptr;
    int* err = nullptr;
    float* lat32 = nullptr;             // screened fill: FP32 noise1..3 per lattice column and level
    std::uint32_t* needBits = nullptr;  // (column, level) pairs the FP64 cells read
    int* points = nullptr;              // the same pairs packed
    int* cellList = nullptr;            // cells the screen left to FP64 (chunk << 7 | cell)
    int* counts = nullptr;              // listed cells, packed pairs
    int maxRadius = 0;
};
std::size_t exact_scratch_bytes(int maxRadius);
void exact_scratch_carve(ExactScratch& s, void* base, int maxRadius);
// One exact scan: the stone field (screened: FP32 with the FP64 operations
// where the screen is not certain; else all FP64), components, statistics and
// the best island. Returns the number of kernels launched.
int launch_exact_scan(const StateCache& cache, int world, int centerChunkX, int centerChunkZ, int radius,
                      const MatchSettings& ms, ExactScratch& s, Island* dIsland, int* dPreviewMinY,
                      int* dPreviewMaxY, int previewCapacity, bool screened, cudaStream_t stream);
int exact_lattice_side(int radius);
void init_exact_tables();  // per device, before its first exact scan

}  // namespace bsf
