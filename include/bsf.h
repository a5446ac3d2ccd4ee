/*
 * libbsf: GB300 (sm_103a) Beta 1.7.3 floating-island seed-finder worker, C ABI.
 *
 * Plain C types only; all buffers are caller-owned host memory unless the
 * name ends in _device (device pointers + a cudaStream_t passed as void*).
 * Every function returns BSF_OK (0) or a negative BSF_E_* status; the message
 * of the last failure on a handle is available from bsf_last_error(). No C++
 * exception crosses this boundary. A request of count == 0 is BSF_E_ARG here;
 * the worker's stream modes read a zero count as the end of the stream, as the
 * reference worker does. A handle serves one request at a time
 * (the reference worker is single-request too: GpuStage0Scout.filter is
 * synchronized, src/GpuStage0Scout.java:249); use one handle per thread.
 */
#ifndef BSF_H
#define BSF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BSF_OK 0
#define BSF_E_ARG (-1)     /* invalid argument (null pointer, bad size, count > capacity) */
#define BSF_E_CUDA (-2)    /* CUDA runtime failure */
#define BSF_E_STATE (-3)   /* handle unusable (open failed or a device fault occurred) */
#define BSF_E_LIMIT (-4)   /* request exceeds a provisioned limit (radius, preview size) */

/* Hunt profiles: gpu_p20_benchmark.cpp:7251-7298 (HuntProfileConfig). */
#define BSF_PROFILE_GENERAL 0
#define BSF_PROFILE_MEGA 1
#define BSF_PROFILE_RECORD60 2
#define BSF_PROFILE_RECORD80 3

/* Pipeline forms for the batch entry points. */
#define BSF_MODE_QUEUED 0 /* fused Stage0 kernel, device-side queues, one host sync per batch */
#define BSF_MODE_PLAIN 1  /* one launch per stage, host round trip after every stage (FP64 kernels) */
#define BSF_MODE_PLAIN_SCREENED 2 /* BSF_MODE_PLAIN's stage-by-stage driving of the queued form's kernels */

typedef struct bsf_config {
    int32_t device;           /* CUDA device ordinal */
    uint32_t capacity;        /* max worlds per request; worker argv "capacity" (default 32768) */
    int32_t profile;          /* BSF_PROFILE_* (worker argv profile) */
    int32_t research;         /* 1: 34-byte research records, 0: 16-byte lean records */
    int32_t centers;          /* regions per world: 1 or 8 (worker argv "centers") */
    int32_t max_exact_radius; /* largest exact-scan radius to provision (24 covers border verify) */
} bsf_config;

/* SearchSettings match thresholds (src/SearchSettings.java:39-45). */
typedef struct bsf_match_settings {
    int32_t min_blocks, min_columns, min_y_for_match, min_width, min_depth;
    double min_avg_thickness;
} bsf_match_settings;

/* IslandSearchEngine.Component (src/IslandSearchEngine.java:6516-6536) of the chosen island. */
typedef struct bsf_island {
    int32_t found;
    int32_t blocks, columns;
    int32_t min_x, max_x, min_z, max_z, min_y, max_y;
    int32_t center_x, center_z;
    int32_t touches_side, touches_bottom;
    int32_t radius_used;
    int64_t sum_x, sum_z;
} bsf_island;

/* One region that reached the exact stage in bsf_mega_search. */
typedef struct bsf_mega_record {
    int64_t seed;
    int32_t world_index;    /* index into the request's seed array */
    int32_t center_index;   /* 0..7 (GpuStage0Scout centres) */
    int32_t center_chunk_x, center_chunk_z;
    int32_t p20, upper, high, coarse;
    double p19_score;
    bsf_island island;      /* the chosen island (found == 0 when no island matched) */
    /* How it was chosen (processGpuRegionAttempt, src/IslandSearchEngine.java:1878-1971),
     * for the candidate log (hunter_candidates.csv): */
    bsf_island raw_island;  /* the scan at `radius` after side-border verification (found == 0: none) */
    bsf_island hot_island;  /* the radius-16 hot scan after verification (found == 0: none or not run) */
    int32_t hot_scanned;    /* 1 when the hot scan ran (coarse >= 120 and radius < 16) */
    int32_t final_source;   /* 0 no island, 1 the raw scan, 2 the hot scan */
    int32_t p19_pass, p19_extreme;
} bsf_mega_record;

typedef struct bsf_stage_counts {
    uint64_t worlds, regions, p20_passed, upper_passed, high_passed, p19_passed,
             mega_rejected, coarse_evaluated, coarse_passed, islands, rng_fallbacks,
             lower_columns, /* lattice columns evaluated by the Lower stage */
             screened_tasks, fallback_tasks; /* FP32-screened column tasks and those recomputed in FP64 */
} bsf_stage_counts;

/* Lifecycle. bsf_open returns NULL only when allocation of the handle itself fails;
 * check bsf_last_error(h) for an open failure (then every call returns BSF_E_STATE). */
void bsf_default_config(bsf_config* cfg);
void bsf_default_match_settings(bsf_match_settings* s);
void* bsf_open(const bsf_config* cfg);
void bsf_close(void* h);
const char* bsf_last_error(const void* h);
int bsf_set_mode(void* h, int32_t mode);

/* Stage0 scout batch: the worker's `stage0stream` response body for `count`
 * worlds (gpu_p20_benchmark.cpp:7310-7613 streamStage0Filter; Java caller
 * GpuStage0Scout.filter, src/GpuStage0Scout.java:249-335). Writes
 * count * centers records of 16 (lean) or 34 (research) bytes, world-major,
 * centre-minor, into out (out_len must hold them). */
int bsf_stage0_filter(void* h, const int64_t* seeds, uint32_t count, uint8_t* out, size_t out_len);

/* P20-only batch: the worker's `stream` response body, one clamped P20 count
 * byte per seed (gpu_p20_benchmark.cpp:7614-7685 streamFilter; Java caller
 * GpuP20Scout, src/GpuP20Scout.java:45-93). */
int bsf_p20_filter(void* h, const int64_t* seeds, uint32_t count, uint8_t* out, size_t out_len);

/* Stage0 scout sweep: `count` consecutive world seeds start_seed, start_seed+1, ...
 * (64-bit wrap-around), each at the handle's centres, through P20 -> Upper ->
 * Lower under the handle's profile. A world survives when one of its regions
 * passes the P20, Upper and high gates: the regions the app sends on to P19,
 * i.e. rejectStage 0 or >= 5 (src/IslandSearchEngine.java:1368-1376; the
 * per-region values are the stage0stream records' p20/upper/high,
 * gpu_p20_benchmark.cpp:7421-7454). The survivors' seeds are written in
 * increasing sweep order, at most `cap` of them; *n_survivors receives the total
 * (which may exceed cap). Runs in the queued form; count may exceed the handle's
 * capacity (the sweep runs in batches of capacity worlds). */
typedef struct bsf_sweep_counts {
    uint64_t worlds, regions;
    uint64_t p20_passed, upper_passed, high_passed; /* regions passing P20, P20+Upper, P20+Upper+high */
    uint64_t survivors;                             /* worlds with a region through all three gates */
    uint64_t rng_fallbacks, screened_tasks, fallback_tasks;
} bsf_sweep_counts;
int bsf_stage0_sweep(void* h, int64_t start_seed, uint64_t count, int64_t* survivors, uint64_t cap,
                     uint64_t* n_survivors, bsf_sweep_counts* counts);

/* BetaTerrain173.generateChunkBaseTerrain (src/beta173/BetaTerrain173.java:120-138)
 * reduced to a stone bitmap: bit (x*16+z)*128+y of 4096 bytes per seed, LSB
 * first, plus a 64-bit hash per bitmap (sum over the 512 little-endian words w_i
 * of splitmix64-finalizer(w_i + (i+1) * 0x9E3779B97F4A7C15)). */
int bsf_chunk_bitmaps(void* h, const int64_t* seeds, uint32_t count, int32_t chunk_x, int32_t chunk_z,
                      uint8_t* bitmaps, uint64_t* hashes);

/* Exact-only findFloatingIslandInSeed at one radius around a centre chunk
 * (src/IslandSearchEngine.java:2861-2977), no border verify or hot scan. */
int bsf_exact_scan(void* h, int64_t seed, int32_t center_chunk_x, int32_t center_chunk_z, int32_t radius,
                   const bsf_match_settings* s, bsf_island* out);

/* processGpuRegionAttempt (src/IslandSearchEngine.java:1878-1971): exact scan at
 * `radius` with side-border verification (radii 10,13,16,20,24) and the
 * radius-16 hot scan when coarse >= 120; returns the reference's chosen island. */
int bsf_resolve_region(void* h, int64_t seed, int32_t center_chunk_x, int32_t center_chunk_z, int32_t radius,
                       int32_t coarse, const bsf_match_settings* s, bsf_island* out);

/* buildIsland3DData (src/IslandSearchEngine.java:389-436; src/Island3DData.java):
 * the best island of an exact scan and its per-column lowest/highest stone Y over
 * its bounding box (index x*depth+z; INT32_MAX / INT32_MIN for empty columns).
 * capacity = entries available in min_y / max_y. */
int bsf_preview(void* h, int64_t seed, int32_t center_chunk_x, int32_t center_chunk_z, int32_t radius,
                const bsf_match_settings* s, bsf_island* out, int32_t* min_y, int32_t* max_y, uint32_t capacity);

/* Whole MEGA pipeline for a batch of worlds: Stage0 (P20 -> Upper -> Lower) ->
 * P19 + Mega topology -> coarse -> exact scan (+ border verify + hot scan) for
 * regions whose coarse score reaches the profile threshold. Writes one record
 * per exact-stage region (in world, centre order) up to records_cap. */
int bsf_mega_search(void* h, const int64_t* seeds, uint32_t count, int32_t radius, const bsf_match_settings* s,
                    bsf_mega_record* records, uint32_t records_cap, uint32_t* records_count,
                    bsf_stage_counts* counts);

/* Device-resident variant of bsf_mega_search's GPU stages for callers that keep
 * seeds in HBM: d_seeds is a device pointer, stream a cudaStream_t (NULL =
 * the handle's stream). Exact-stage regions are returned like bsf_mega_search. */
int bsf_mega_search_device(void* h, const int64_t* d_seeds, uint32_t count, int32_t radius,
                           const bsf_match_settings* s, bsf_mega_record* records, uint32_t records_cap,
                           uint32_t* records_count, bsf_stage_counts* counts, void* stream);

/* Pipelined MEGA search over `count` worlds (1 .. 2^31-1, any multiple of the
 * capacity): batches of capacity worlds alternate between this handle and a
 * second one it opens on first use with the same config (so twice the device
 * memory; bsf_handle_footprint counts both), and each batch's GPU stages are
 * enqueued before the previous batch's exact stage runs, so the exact stage
 * (host threads and exact-scan streams) overlaps the next batch's GPU work.
 * Records come in (world_index, center_index) order with world_index counted
 * from the start of the range; counts are summed over the batches. The reference
 * overlaps the same two parts across processes: the worker streams Stage0 and
 * coarse records while the Java app's exact-scan threads drain its survivor
 * queue (src/IslandSearchEngine.java:1225, 1437-1443). bsf_last_region_records
 * and bsf_last_stage_ms describe this handle's own last batch only. */
int bsf_mega_search_range(void* h, const int64_t* seeds, uint64_t count, int32_t radius, const bsf_match_settings* s,
                          bsf_mega_record* records, uint32_t records_cap, uint32_t* records_count,
                          bsf_stage_counts* counts);
/* bsf_mega_search_range on device-resident seeds; the pipeline's streams wait for
 * the work queued on `stream` (a cudaStream_t, NULL = none) before they start. */
int bsf_mega_search_range_device(void* h, const int64_t* d_seeds, uint64_t count, int32_t radius,
                                 const bsf_match_settings* s, bsf_mega_record* records, uint32_t records_cap,
                                 uint32_t* records_count, bsf_stage_counts* counts, void* stream);

/* Stage outcomes of every region of the last bsf_mega_search(_device) batch:
 * count * centers 34-byte research records (the stage0stream research layout,
 * world-major, centre-minor), e.g. to sample rejected regions for exact audits. */
int bsf_last_region_records(void* h, uint8_t* out, size_t out_len);

/* The device lines of the worker's startup banner (printDevice,
 * gpu_p20_benchmark.cpp:979-992): "GPU: <name>", "Architecture: sm_XY",
 * "Compute units: N", "Global memory: G GiB", one per line, into out. */
int bsf_device_summary(int32_t device, char* out, size_t out_len);

/* Number of GPU kernel launches issued by the handle (and the second handle of
 * its pipelined range search) so far (instrumentation). */
uint64_t bsf_kernel_launches(const void* h);

/* Device time of each stage of the last batch call, from CUDA events recorded
 * on the stream the kernels ran on (instrumentation): ms[0] generator setup,
 * ms[1] Stage0 + P19, ms[2] coarse, ms[3] exact stage (host wall time, it
 * includes its round trips). */
int bsf_last_stage_ms(const void* h, float* ms4);

/* Autotuner: times every launch-shape variant (threads per CTA x CTAs per SM)
 * of the screened Stage0 and coarse kernels on `worlds` calibration worlds
 * (capacity permitting) with CUDA events and keeps the fastest for this
 * process, then times the two grid shapes (bsf_set_persistent) with them and
 * keeps the faster for this handle. report (optional) receives
 * "kernel: variant=ms ... -> choice; grid: ... -> choice". */
int bsf_autotune(void* h, uint32_t worlds, char* report, size_t report_len);
/* Selects launch-shape variants explicitly (index order of the autotune report). */
int bsf_set_launch_variants(void* h, int32_t stage0_variant, int32_t coarse_variant);

/* Measured scalar FP64 and FP32 issue rates of the current device (instrumentation
 * for the roofline): independent add chains in every lane of every SM, timed
 * with CUDA events. ops_per_s[0] = FP64 DADD/s, ops_per_s[1] = FP32 FADD/s. */
int bsf_measure_peaks(double* ops_per_s2);

/* Screen-bound probe (instrumentation): for `worlds` seeds' real generator
 * states, evaluates every FP32 screening primitive beside its exact FP64 twin at
 * random lattice points (samples_per_thread samples in each of 77,824 threads)
 * and writes, per kind, the largest |FP32 - FP64| divided by the bound the
 * screen uses, and the samples taken. Kinds: 0/1 one 3D octave against
 * E_OCT3 with FP64 / double-float axis entries, 2/3 one 2D octave against
 * E_OCT2 (same), 4/5 one simplex sample against its tracked bound with
 * double-float / FP64 lattice geometry, 6 temperature and rain, 7 column shape
 * d5 and d7, against their tracked bounds. The screen is sound while every
 * ratio stays below 1. Allocates its own device memory. */
#define BSF_PROBE_KINDS 8
int bsf_screen_probe(const int64_t* seeds, uint32_t worlds, uint32_t samples_per_thread, uint64_t rng,
                     double* max_ratio, uint64_t* counts, char* err, size_t err_len);

/* Switches the hunt profile (BSF_PROFILE_*) of later batch calls on this handle
 * (the worker argv profile, chosen per request instead of per process). */
int bsf_set_profile(void* h, int32_t profile);

/* Verification switch for the queued form: on == 0 sends every column task of
 * the screened Stage0 and coarse kernels down their exact FP64 fallback path,
 * and exact scans (batches, bsf_exact_scan, bsf_resolve_region, bsf_preview)
 * through the all-FP64 fill instead of the screened one (slow; results must
 * not change). Default on. */
int bsf_set_screening(void* h, int32_t on);

/* Grid shape of the screened Stage0 and coarse kernels. on != 0 (default):
 * persistent grids, one CTA per resident slot looping over worlds (fastest when
 * the handle has the GPU to itself). on == 0: one CTA per world (Stage0) and per
 * half-region of the coarse queue, so CTAs retire every world and kernels of a
 * higher-priority stream start without waiting for the batch (served mode's
 * range lanes). Results are identical either way. */
int bsf_set_persistent(void* h, int32_t on);

/* Device memory (bytes) a handle opened with cfg allocates, computed without a
 * GPU from the same buffer list bsf_open allocates; BSF_E_ARG for a bad config. */
int bsf_config_footprint(const bsf_config* cfg, uint64_t* bytes);
/* Device memory (bytes) this handle holds. */
uint64_t bsf_handle_footprint(const void* h);
/* Moves the handle's work to a new stream of the device's highest (high != 0) or
 * default (high == 0) priority; the block scheduler starts pending CTAs of a
 * higher-priority stream first. Must not be called while the handle is in use. */
int bsf_set_stream_priority(void* h, int32_t high);

/* ---- Served mode (bsf_server_*) ------------------------------------------
 * Lanes run on separate streams; for their kernels to overlap without false
 * dependencies the process needs CUDA_DEVICE_MAX_CONNECTIONS above the number
 * of lanes. Loading libbsf sets it to 32 unless it is already set, which works
 * when the library is loaded before the process's first CUDA call.
 * A request loop that keeps generator caches, stage queues and scratch
 * resident on the device in "lanes" (one handle + stream each) and runs two
 * request classes concurrently:
 *   RANGE   a MEGA search over a list of seeds (IslandSearchEngine's GPU range
 *           scan, src/IslandSearchEngine.java:1252-1255 / 1878-1971), split
 *           into chunks of chunk_worlds worlds;
 *   PREVIEW one island preview (generate3DPreviewForIsland -> buildIsland3DData,
 *           src/IslandSearchEngine.java:284-436).
 * Continuous batching: a request is admitted as soon as a lane is idle, or a
 * new lane's device footprint (bsf_config_footprint) fits in the HBM budget
 * (idle lanes of the other class are closed to make room); range requests
 * are handed out one chunk at a time, so requests that arrive later start
 * while earlier ones are still on the GPU, previews first. Preview lanes run
 * on high-priority streams. Results do not depend on what else is running:
 * every lane computes with its own buffers. Records of a range request come
 * back in (world_index, center_index) order like bsf_mega_search. */
#define BSF_PENDING 1 /* bsf_server_poll: not finished within the wait */
#define BSF_REQ_RANGE 0
#define BSF_REQ_PREVIEW 1

typedef struct bsf_server_config {
    int32_t device;
    int32_t profile;             /* BSF_PROFILE_* of range searches */
    uint64_t hbm_budget_bytes;   /* device bytes all lanes may hold; 0 = half the free memory at open */
    uint32_t chunk_worlds;       /* range lane capacity = worlds per chunk (default 8192) */
    int32_t max_lanes;           /* range chunks running at once = range worker threads (default 4) */
    int32_t preview_lanes;       /* previews running at once = preview worker threads (default 2) */
    int32_t max_preview_radius;  /* largest preview radius (default 16, at most 24) */
} bsf_server_config;

typedef struct bsf_server_result {
    int32_t kind;                /* BSF_REQ_* */
    int32_t status;              /* BSF_OK or the failing call's BSF_E_* */
    double queue_ms;             /* submit -> first work on a lane */
    double latency_ms;           /* submit -> completion */
    uint32_t records;            /* RANGE: records available from bsf_server_records */
    bsf_stage_counts counts;     /* RANGE: summed over chunks */
    bsf_island island;           /* PREVIEW: the chosen island */
    uint32_t preview_columns;    /* PREVIEW: width * depth entries of bsf_server_preview_columns */
} bsf_server_result;

typedef struct bsf_server_stats {
    uint64_t submitted[2], completed[2], failed[2]; /* by BSF_REQ_* */
    double p50_ms[2], p99_ms[2], p999_ms[2];        /* latency of completed requests */
    uint64_t worlds_completed;                       /* RANGE worlds finished */
    uint64_t hbm_bytes_in_use, hbm_bytes_peak, hbm_budget;
    uint32_t lanes_open[2];
    uint32_t max_busy_lanes;                         /* most lanes running work at one time */
    uint64_t deferred;                               /* admissions that waited for memory or a lane */
    uint64_t evictions;                              /* idle lanes closed to admit the other class */
} bsf_server_stats;

void bsf_default_server_config(bsf_server_config* cfg);
void* bsf_server_open(const bsf_server_config* cfg);
void bsf_server_close(void* s); /* waits for running work; pending requests are dropped */
const char* bsf_server_last_error(const void* s);
/* Submit calls copy their inputs and return at once with a ticket. profile is a
 * BSF_PROFILE_* for this range request, or -1 for the server's profile. */
int bsf_server_submit_range(void* s, const int64_t* seeds, uint32_t count, int32_t radius, int32_t profile,
                            const bsf_match_settings* ms, uint64_t* ticket);
int bsf_server_submit_preview(void* s, int64_t seed, int32_t center_chunk_x, int32_t center_chunk_z,
                              int32_t radius, const bsf_match_settings* ms, uint64_t* ticket);
/* Waits up to wait_ms (0 = no wait, < 0 = forever) for the ticket: BSF_OK with
 * out filled when finished, BSF_PENDING when not yet, BSF_E_ARG for an unknown ticket. */
int bsf_server_poll(void* s, uint64_t ticket, int32_t wait_ms, bsf_server_result* out);
int bsf_server_records(void* s, uint64_t ticket, bsf_mega_record* out, uint32_t cap, uint32_t* n);
int bsf_server_preview_columns(void* s, uint64_t ticket, int32_t* min_y, int32_t* max_y, uint32_t cap);
int bsf_server_release(void* s, uint64_t ticket); /* frees a finished request's results */
int bsf_server_get_stats(void* s, bsf_server_stats* out);

/* Allocation-free variant of bsf_chunk_bitmaps. It has no counterpart in the
 * reference: it exists for callers that cannot allocate GPU memory (a host
 * that owns all device memory and passes in pre-allocated buffers, a serving
 * loop where cudaMalloc would synchronise the device, a fixed memory budget).
 * Inputs and outputs are caller-owned device buffers (d_seeds: count int64,
 * d_bitmaps: count * 4096 bytes, d_hashes: count uint64) and the work is
 * enqueued on `stream` (a cudaStream_t, NULL = default stream) without a
 * synchronisation. Its scratch is a fixed array of BSF_NOALLOC_MAX_WORLDS
 * generator caches (5.6 MB) compiled into the library, which every GPU that
 * loads the library keeps until the process exits; count beyond the maximum
 * returns BSF_E_LIMIT. The first call on each device does a one-time set-up
 * (constant tables, the scratch address) and should come before any stream
 * capture. That set-up is kept for the life of the process: the entry point
 * assumes the device (its primary context) is not reset after the first call,
 * since a reset would leave a stale scratch address and empty constant tables.
 * All calls share the one array: calls whose work overlaps on the GPU race.
 * err (optional, err_len bytes) receives a message on failure. */
#define BSF_NOALLOC_MAX_WORLDS 256u
int bsf_chunk_bitmaps_noalloc(const int64_t* d_seeds, uint32_t count, int32_t chunk_x, int32_t chunk_z,
                              uint8_t* d_bitmaps, uint64_t* d_hashes, void* stream, char* err, size_t err_len);

#ifdef __cplusplus
}
#endif
#endif
