/*
 * CPU oracle for the Beta 1.7.3 floating-island seed-finder hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA product
 * path is compared against; nothing in the product links, loads or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use it.
 *
 * It is a plain-C restatement of the reference's algorithm (Java Beta 1.7.3
 * generator under src/beta173/ plus the worker's stage semantics in
 * native/src/). Every function cites the reference file:line it restates.
 * Build with -ffp-contract=off and without -ffast-math: every FP64 operation
 * must round exactly like Java's strict IEEE double arithmetic.
 */
#ifndef BSF_ORACLE_H
#define BSF_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- java.util.Random (48-bit LCG) ---------------------------------------- */
typedef struct { uint64_t s; } or_rand;
void or_rand_set_seed(or_rand* r, int64_t seed);
int32_t or_rand_next(or_rand* r, int bits);
double or_rand_next_double(or_rand* r);
int32_t or_rand_next_int(or_rand* r, int32_t bound);

/* ---- one Perlin / simplex generator (same constructor layout) ------------- */
typedef struct { int32_t p[512]; double a, b, c; } or_perlin;
void or_perlin_init(or_perlin* g, or_rand* r);
void or_perlin_consume(or_rand* r);

/* All octave generators of one world, in Java construction order. */
typedef struct {
    or_perlin n2[16], n3[16], n1[8], n4[10], n5[16];
    or_perlin temp[4], rain[4], blend[2];
} or_world;
void or_world_init(or_world* w, int64_t seed);

/* Exports used by tests: raw state of generator `index` in world order
 * (0..15 noise2, 16..31 noise3, 32..39 noise1, 40..49 noise4, 50..65 noise5,
 *  66..69 temperature, 70..73 rain, 74..75 blend). perm256 gets p[0..255]. */
int or_world_state(int64_t seed, int index, uint8_t* perm256, double* abc3);

/* Legacy NoiseGeneratorPerlin173.a(double[],...) with an integer sample stride. */
void or_perlin_add(const or_perlin* g, double* out, double fromX, double fromY, double fromZ,
                   int xLen, int yLen, int zLen, double stepX, double stepZ,
                   double sx, double sy, double sz, double amplitude);
/* NoiseGenerator2173.aStrided */
void or_simplex_add(const or_perlin* g, double* out, double x0, double z0, int xLen, int zLen,
                    int strideX, int strideZ, double sx, double sz, double weight);

/* One octave column (weight 1) from a raw state, outputs y >= yLo: test hook. */
void or_perlin_column17_test(const uint8_t* perm256, const double* abc, double xs, double sy, double zs,
                             int yLo, double* out17);
/* Single-point samplers (the first octave term, weight 1). */
double or_perlin3_point(const or_perlin* g, double x, double y, double z);
double or_perlin2_point(const or_perlin* g, double x, double z);
double or_simplex_point(const or_perlin* g, double x, double z);

/* Climate (temperature, rain) after normalisation at integer block coords. */
void or_climate(const or_world* w, int blockX, int blockZ, double* temperature, double* rain);

/* One 17-level lattice density column at coarse coords (cx, cz) with the
 * climate sampled at block (climX, climZ); outputs only y >= yLo (others 0). */
void or_density_column(const or_world* w, int cx, int cz, int climX, int climZ, int yLo, double* out17);

/* BetaTerrain173.generateChunkBaseTerrain: blocks[(x*16+z)*128+y] in {0 air,1 stone,2 water,3 ice}. */
void or_chunk_base_terrain(const or_world* w, int chunkX, int chunkZ, uint8_t* blocks);
/* Stone bitmap: bit (x*16+z)*128+y, LSB first; returns the 64-bit bitmap hash. */
uint64_t or_chunk_stone_bitmap(int64_t seed, int chunkX, int chunkZ, uint8_t* bitmap4096);
/* Test hook: the chunk path's noise1..5 sums at the 5x5 lattice columns of a chunk
 * (coarse (4*chunkX+i, 4*chunkZ+j), index i*5+j); n1..n3 [25][17], n4/n5 [25]. */
void or_chunk_noise_test(int64_t seed, int chunkX, int chunkZ, double* n1, double* n2, double* n3, double* n4,
                         double* n5);
uint64_t or_bitmap_hash(const uint8_t* bitmap4096);
/* Batch version for tests/baselines: n seeds, optional threads. */
void or_chunk_bitmaps(const int64_t* seeds, int n, int chunkX, int chunkZ,
                      uint8_t* bitmaps, uint64_t* hashes, int threads);

/* ---- Stage0 (P20 -> Upper -> Lower) + P19 + Mega + coarse per region ------ */
typedef struct {
    int p20MinCount, upperMinCount, highMinCount;
    double p19MinScore;
    int coarseMinCells;
    int megaTopologyFilter;
} or_profile;
/* profile ids: 0 general, 1 mega, 2 record60, 3 record80 */
void or_profile_get(int id, or_profile* out);

typedef struct {
    int fullY88, fullY96, fullY104, fullY112;
    int y88Largest, y88Width, y88Depth, y88Touches;
    int y96Largest, y96Width, y96Depth, y96Touches;
} or_features;

typedef struct {
    int32_t p20, upper, high;
    int32_t p19Evaluated, p19Pass, p19Extreme, megaReject;
    int32_t coarseEvaluated, coarse;
    double p19Score;
    or_features f;
    uint8_t upperMask[256];
    uint8_t highest[256];
} or_region;

void or_stage0_region(const or_world* w, int centerChunkX, int centerChunkZ,
                      const or_profile* prof, int runCoarse, or_region* out);
double or_p19_score(int scout, const or_features* f);
int or_p19_extreme(const or_features* f);
int or_mega_topology_reject(double score, int extreme, const or_features* f);
void or_monster_features(const uint8_t* highest256, or_features* f);

/* Coarse 61x61x17 sign grid (climate at 4c+2) and its component score. */
void or_coarse_signs(const or_world* w, int centerChunkX, int centerChunkZ, uint8_t* signs);
int or_coarse_score(const uint8_t* signs);
int or_coarse_score_seed(int64_t seed, int centerChunkX, int centerChunkZ);

/* The Java app's component-lazy coarse scorer (P17): the upper slice (levels
 * 8..16) everywhere, lower levels only for columns a component's search reaches.
 * A second restatement of the coarse score; it must equal or_coarse_score. */
typedef struct {
    int lowerColumns;   /* lower column slices generated */
    int rounds;         /* expansion rounds */
    int fallbackToFull; /* a limit was hit and the whole grid was scored */
} or_lazy_stats;
int or_coarse_score_lazy_seed(int64_t seed, int centerChunkX, int centerChunkZ, or_lazy_stats* stats);
void or_coarse_signs_seed(int64_t seed, int centerChunkX, int centerChunkZ, uint8_t* signs);

/* Worker record packing (lean 16 B / research 34 B). */
void or_pack_record(const or_region* r, int research, uint8_t* outRecord);
/* stage0stream batch: n worlds x centers records into out. */
void or_stage0_batch(const int64_t* seeds, int n, int centers, int profileId, int research,
                     uint8_t* out, int threads);

/* ---- MEGA exact scan ------------------------------------------------------ */
typedef struct {
    int minBlocks, minColumns, minYForMatch, minWidth, minDepth;
    double minAvgThickness;
} or_match_settings;
void or_match_defaults(or_match_settings* s);

typedef struct {
    int32_t found;
    int32_t blocks, columns;
    int32_t minX, maxX, minZ, maxZ, minY, maxY;
    int32_t centerX, centerZ;
    int32_t touchesSide, touchesBottom;
    int32_t radiusUsed;
    int64_t sumX, sumZ;
} or_island;

/* findFloatingIslandInSeed exact part at one radius (no border verify, no hot scan). */
int or_exact_scan(int64_t seed, int centerChunkX, int centerChunkZ, int radius,
                  const or_match_settings* s, or_island* out);
/* processGpuRegionAttempt: exact r + border verify + hot scan when coarse >= 120. */
int or_resolve_region(int64_t seed, int centerChunkX, int centerChunkZ, int radius, int coarse,
                      const or_match_settings* s, or_island* out);
/* Preview column model of the best component (minY/maxY per bbox column, INT_MAX/INT_MIN empty). */
int or_preview(int64_t seed, int centerChunkX, int centerChunkZ, int radius,
               const or_match_settings* s, or_island* out, int32_t* minY, int32_t* maxY, int capacity);

/* ---- whole MEGA pipeline for the CPU baseline ----------------------------- */
typedef struct {
    uint64_t worlds, regions, p20Passed, upperPassed, highPassed, p19Passed,
             megaRejected, coarseEvaluated, coarsePassed, islands;
} or_pipeline_counts;
/* Runs n worlds x 8 centres through every stage; island records (one per
 * coarse survivor, found or not) are written to islands[] in (world, centre)
 * order, up to islandCap. Returns the number written. */
int or_mega_pipeline(const int64_t* seeds, int n, int profileId, int radius,
                     const or_match_settings* s, int threads,
                     or_pipeline_counts* counts, or_island* islands, int64_t* islandRegion, int islandCap);

uint64_t or_splitmix_seed(uint64_t sequenceSeed, uint64_t attempt);

#ifdef __cplusplus
}
#endif
#endif
