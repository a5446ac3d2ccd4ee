// Host side of libbsf: the C ABI of include/bsf.h, device buffer ownership and
// the two batch pipeline forms (queued and plain stage-by-stage).
#include "../../include/bsf.h"
#include "bsf_device.cuh"
#include "bsf_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <shared_mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace bsf {
namespace {

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[320];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

// Response record packing (gpu_p20_benchmark.cpp:7504-7554): lean 16 bytes or
// research 34 bytes per region, world-major / centre-minor.
__global__ void k_pack_records(const RegionInfo* __restrict__ regions, int count, int research,
                               std::uint8_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const RegionInfo r = regions[i];
    const int rec = research ? 34 : 16;
    std::uint8_t* o = out + static_cast<std::size_t>(i) * rec;
    auto clamp8 = [](int v) { return static_cast<std::uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v)); };
    o[0] = clamp8(r.p20);
    o[1] = clamp8(r.upper);
    o[2] = clamp8(r.high);
    o[3] = r.p19Pass;
    o[4] = static_cast<std::uint8_t>(r.coarse & 0xFF);
    o[5] = static_cast<std::uint8_t>((r.coarse >> 8) & 0xFF);
    o[6] = r.p19Extreme;
    o[7] = r.megaReject;
    const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(r.p19Score));
    for (int k = 0; k < 8; ++k) o[8 + k] = static_cast<std::uint8_t>(bits >> (8 * k));
    if (!research) return;
    auto put16 = [&](int off, int v) {
        const unsigned u = static_cast<unsigned>(v < 0 ? 0 : (v > 65535 ? 65535 : v));
        o[off] = static_cast<std::uint8_t>(u & 0xFF);
        o[off + 1] = static_cast<std::uint8_t>((u >> 8) & 0xFF);
    };
    put16(16, r.fullY88);
    put16(18, r.fullY96);
    put16(20, r.fullY104);
    put16(22, r.fullY112);
    put16(24, r.y88Largest);
    o[26] = r.y88Width;
    o[27] = r.y88Depth;
    o[28] = r.y88Touches ? 1 : 0;
    put16(29, r.y96Largest);
    o[31] = r.y96Width;
    o[32] = r.y96Depth;
    o[33] = r.y96Touches ? 1 : 0;
}

// P20-only response byte (gpu_p20_benchmark.cpp:7660-7668).
__global__ void k_pack_p20(const RegionInfo* __restrict__ regions, int count, int centers, std::uint8_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int v = regions[static_cast<std::size_t>(i) * centers].p20;
    out[i] = static_cast<std::uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v));
}

// Stage pass counters (gpu_p20_benchmark.cpp:7556-7571) and the exact-stage queue.
__global__ void k_stage_counts(const RegionInfo* __restrict__ regions, int count, Profile prof,
                               unsigned long long* counts, RegionRef* exactQueue, int* exactCount, int exactCap,
                               int centers) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (i < count) {
        const RegionInfo r = regions[i];
        const bool p20 = r.p20 >= prof.p20MinCount;
        const bool up = p20 && r.upper >= prof.upperMinCount;
        const bool hi = up && r.high >= prof.highMinCount;
        c[0] = p20;
        c[1] = up;
        c[2] = hi;
        c[3] = hi && r.p19Pass;
        c[4] = hi && r.p19Pass && r.megaReject;
        c[5] = r.coarseEvaluated;
        c[6] = r.coarseEvaluated && r.coarse >= prof.coarseMinCells;
        c[7] = up ? static_cast<unsigned long long>(r.upper) : 0ULL;  // Lower-stage columns
        if (c[6]) {
            const int slot = atomicAdd(exactCount, 1);
            if (slot < exactCap) exactQueue[slot] = RegionRef{i / centers, i % centers};
        }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        unsigned long long v = c[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&counts[k], v);
    }
}

// One exact-stage region with everything the host needs to resolve and report it.
struct ExactItem {
    RegionRef ref;
    std::int64_t seed;
    RegionInfo info;
};
static_assert(sizeof(ExactItem) == 64, "ExactItem layout");

// Gathers the exact-stage queue's regions (outcome and world seed) into one
// contiguous array, so the host reads them with one copy instead of one per region.
__global__ void k_gather_exact(const RegionRef* __restrict__ queue, const int* count, int cap,
                               const RegionInfo* __restrict__ regions, const std::int64_t* __restrict__ seeds,
                               int centers, ExactItem* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(*count, cap)) return;
    const RegionRef r = queue[i];
    ExactItem e;
    e.ref = r;
    e.seed = seeds[r.world];
    e.info = regions[static_cast<std::size_t>(r.world) * centers + r.center];
    out[i] = e;
}

// Issue-rate probes: 8 independent dependent-add chains per thread.
template <typename T>
__global__ void k_add_chains(T* out, int iters, T inc) {
    T a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
        a0 += inc; a1 += inc; a2 += inc; a3 += inc; a4 += inc; a5 += inc; a6 += inc; a7 += inc;
    }
    const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == static_cast<T>(-1)) out[0] = s;  // keeps the chains alive
}

}  // namespace
}  // namespace bsf

using namespace bsf;

// Stream capture versus device-wide calls. While any thread captures a stream,
// calls that synchronise the device (cudaFree, cudaDeviceSynchronize) fail and
// break the capture, so handles open and close under the exclusive side of this
// lock and batch graphs are captured under the shared side: handles on several
// threads (the served mode's lanes) can capture at once but never while another
// thread allocates or frees a handle.
static std::shared_mutex& capture_guard() {
    static std::shared_mutex m;
    return m;
}

// Exact-stage regions copied back inside every batch (a 32,768-world MEGA batch
// has about 13); more cost one further copy.
constexpr int kExactPrefix = 256;

// One exact-scan context: a stream, exact-scan scratch and a result slot.
// Context 0 is the handle's own (its stream, scratch and preview buffers); the
// others let the batch exact stage resolve several regions at once.
struct ExactCtx {
    cudaStream_t stream = nullptr;  // nullptr: the handle's current stream
    void* base = nullptr;           // scratch allocation (contexts 1..)
    ExactScratch exact;
    Island* dIsland = nullptr;
};

struct BsfHandle {
    bsf_config cfg{};
    Profile prof{};
    int mode = BSF_MODE_QUEUED;
    bool persistent = true;  // grid shape of the screened kernels (bsf_set_persistent)
    bool ok = false;
    std::string err;
    cudaStream_t stream = nullptr;
    std::atomic<unsigned long long> launches{0};
    std::vector<ExactCtx> ectx;  // exact-scan contexts (0: the handle's own)
    int capacity = 0;
    int centers = 8;
    int lastBatch = 0;  // worlds in the last MEGA batch (their RegionInfo stays in dRegions)
    int coarseCap = 0;
    int exactCap = 0;

    std::int64_t* dSeeds = nullptr;
    StateCache cache;
    RegionInfo* dRegions = nullptr;
    RegionRef* dCoarseQueue = nullptr;
    int* dCounters = nullptr;  // [0] coarse count, [1] rng fallbacks, [2] exact count
    std::uint32_t* dSigns = nullptr;
    int* dLabels = nullptr;
    int* dStats = nullptr;
    int* dCoarseErr = nullptr;  // coarse union-find retry-bound flag (inside dStats)
    std::uint8_t* dOut = nullptr;
    std::uint64_t* dHashes = nullptr;
    unsigned long long* dStageCounts = nullptr;
    RegionRef* dExactQueue = nullptr;
    ExactItem* dExactItems = nullptr;  // gathered exact-stage regions (k_gather_exact)
    ExactItem* hExactItems = nullptr;  // pinned copy; the first kExactPrefix come back inside the batch
    void* dExactBase = nullptr;
    ExactScratch exact;
    Stage0FastScratch fs;
    Island* dIsland = nullptr;
    int* dPrevMin = nullptr;
    int* dPrevMax = nullptr;
    int prevCap = 0;
    SweepState sweep;                     // bsf_stage0_sweep (bsf_sweep.cu)
    void* dSweepBase = nullptr;
    std::int64_t* hSweepOut = nullptr;    // pinned copy of the survivor list
    unsigned long long* hSweep = nullptr; // pinned: [0] start seed, [1] list total, [2..5] stage counters,
                                          // [6..7] screen stats, [8] setup fallbacks
    std::int64_t* hSeeds = nullptr;  // pinned staging
    std::uint8_t* hOut = nullptr;
    std::size_t outBytes = 0;
    std::vector<RegionInfo> hRegions;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float stageMs[4] = {0, 0, 0, 0};
    unsigned long long* hPinned = nullptr;  // stage counters [0..7], screen stats [8..11], counters [12..13],
                                            // coarse retry flag [14]
    struct CachedGraph {
        cudaGraphExec_t exec;
        cudaStream_t stream;
        int variants;  // launch-shape variants the graph was captured with
    };
    std::vector<std::pair<long long, CachedGraph>> graphs;  // batch graphs by (worlds, seed source)
    BsfHandle* twin = nullptr;           // second handle of the pipelined range search (mega_range)
    bool exactHigh = false;              // exact-scan contexts 1.. on the highest-priority streams
    cudaEvent_t rangeEvent = nullptr;    // orders a range search after the caller's stream

    void drop_graphs() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second.exec);
        graphs.clear();
    }

    std::size_t footprint = 0;  // device bytes allocated by the handle
    bool dry = false;           // size the buffers without allocating them

    void alloc(void** p, std::size_t bytes, const char* what) {
        if (dry) *p = nullptr;
        else check(cudaMalloc(p, bytes), what);
        footprint += bytes;
    }
};

namespace {

void fail(BsfHandle* h, const std::string& msg) {
    if (h) h->err = msg;
}

template <typename F>
int guarded(void* hv, F&& f) {
    BsfHandle* h = static_cast<BsfHandle*>(hv);
    if (!h) return BSF_E_ARG;
    if (!h->ok) {
        if (h->err.empty()) h->err = "handle is not open";
        return BSF_E_STATE;
    }
    try {
        return f(h);
    } catch (const std::invalid_argument& e) {
        fail(h, e.what());
        return BSF_E_ARG;
    } catch (const std::length_error& e) {
        fail(h, e.what());
        return BSF_E_LIMIT;
    } catch (const std::exception& e) {
        fail(h, e.what());
        const cudaError_t sticky = cudaGetLastError();
        if (sticky != cudaSuccess) h->ok = false;
        return BSF_E_CUDA;
    }
}

MatchSettings to_ms(const bsf_match_settings* s) {
    bsf_match_settings d;
    if (!s) {
        bsf_default_match_settings(&d);
        s = &d;
    }
    return MatchSettings{s->min_blocks, s->min_columns, s->min_y_for_match, s->min_width, s->min_depth,
                         s->min_avg_thickness};
}

void to_island(const Island& i, bsf_island* o) {
    o->found = i.found;
    o->blocks = i.blocks;
    o->columns = i.columns;
    o->min_x = i.minX; o->max_x = i.maxX; o->min_z = i.minZ; o->max_z = i.maxZ;
    o->min_y = i.minY; o->max_y = i.maxY;
    o->center_x = i.centerX; o->center_z = i.centerZ;
    o->touches_side = i.touchesSide; o->touches_bottom = i.touchesBottom;
    o->radius_used = i.radiusUsed;
    o->sum_x = i.sumX; o->sum_z = i.sumZ;
}

// H2D seeds and build every generator of the batch.
void stage_seeds(BsfHandle* h, const std::int64_t* seeds, int n, bool hostSeeds) {
    if (hostSeeds) {
        std::memcpy(h->hSeeds, seeds, static_cast<std::size_t>(n) * 8);
        check(cudaMemcpyAsync(h->dSeeds, h->hSeeds, static_cast<std::size_t>(n) * 8, cudaMemcpyHostToDevice, h->stream),
              "seed upload");
        launch_world_init(h->dSeeds, n, h->cache, h->dCounters + 1, h->stream);
    } else {
        launch_world_init(seeds, n, h->cache, h->dCounters + 1, h->stream);
    }
    ++h->launches;
}

// Queued form: fused Stage0 kernel appends P19 survivors to the device coarse
// queue; the coarse kernels consume it by its device-side count.
void run_gpu_stages_queued(BsfHandle* h, int n, bool timed = false);

// External event records: under stream capture they become event-record nodes
// of the batch graph, so replays still time every stage.
void record(BsfHandle* h, int i) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    check(cudaStreamIsCapturing(h->stream, &st), "capture status");
    if (st == cudaStreamCaptureStatusActive)
        check(cudaEventRecordWithFlags(h->ev[i], h->stream, cudaEventRecordExternal), "event");
    else
        check(cudaEventRecord(h->ev[i], h->stream), "event");
}

// Queued form: the screened Stage0 kernel appends P19 survivors to the device
// coarse queue; the screened coarse kernels consume it by its device-side count.
void run_gpu_stages_queued(BsfHandle* h, int n, bool timed) {
    check(cudaMemsetAsync(h->dCounters, 0, sizeof(int), h->stream), "memset");
    launch_stage0_fast(h->cache, n, h->centers, h->prof, h->dRegions, h->dCoarseQueue, h->dCounters,
                       h->capacity * h->centers, h->fs, h->stream, h->persistent);
    if (timed) record(h, 2);
    launch_coarse_signs_fast(h->cache, h->dCoarseQueue, h->dCounters, h->coarseCap, h->dSigns, h->fs.stats,
                             h->stream, h->persistent, h->fs.forceExact != 0);
    launch_coarse_cc(h->dCoarseQueue, h->dCounters, h->coarseCap, h->dSigns, h->dLabels, h->dStats, h->dRegions,
                     h->centers, h->stream);
    if (timed) record(h, 3);
    h->launches += 4;
}

// Plain form: stage by stage with a host round trip after each; the host
// rebuilds the coarse work list and feeds it in micro-batches of 1024 regions
// (the reference worker's structure, gpu_p20_benchmark.cpp:7421-7502, 1188-1218).
void run_gpu_stages_plain(BsfHandle* h, int n) {
    check(cudaStreamSynchronize(h->stream), "world init");
    launch_stage0(h->cache, n, h->centers, h->prof, nullptr, h->dRegions, nullptr, h->dCounters, 0, h->stream);
    ++h->launches;
    const int regions = n * h->centers;
    h->hRegions.resize(regions);
    check(cudaMemcpyAsync(h->hRegions.data(), h->dRegions, sizeof(RegionInfo) * regions, cudaMemcpyDeviceToHost,
                          h->stream),
          "region download");
    check(cudaStreamSynchronize(h->stream), "stage0");
    std::vector<RegionRef> list;
    for (int i = 0; i < regions; ++i) {
        const RegionInfo& r = h->hRegions[i];
        if (r.p19Evaluated && r.p19Pass && !r.megaReject) list.push_back(RegionRef{i / h->centers, i % h->centers});
    }
    const int micro = std::min(1024, h->coarseCap);
    for (std::size_t off = 0; off < list.size(); off += micro) {
        const int chunk = static_cast<int>(std::min<std::size_t>(micro, list.size() - off));
        check(cudaMemcpyAsync(h->dCoarseQueue, list.data() + off, sizeof(RegionRef) * chunk, cudaMemcpyHostToDevice,
                              h->stream),
              "coarse list upload");
        check(cudaMemcpyAsync(h->dCounters, &chunk, sizeof(int), cudaMemcpyHostToDevice, h->stream), "count");
        // maxCount = the queue's capacity (the device-side count bounds the work): the
        // score kernel's grid, and with it the place of its retry-bound flag, is then
        // the one the batch resets and reads
        launch_coarse_score(h->cache, h->dCoarseQueue, h->dCounters, h->coarseCap, LatticeBuffers{}, h->dSigns,
                            h->dLabels, h->dStats, h->dRegions, h->centers, h->stream);
        h->launches += 2;
        check(cudaStreamSynchronize(h->stream), "coarse micro-batch");
    }
}

// Plain form on the screened kernels: the same FP32-screened Stage0 and coarse
// kernels as the queued form, driven stage by stage like run_gpu_stages_plain
// (region records downloaded, the coarse list built on the host and fed in
// micro-batches of 1024 with a sync each). Against the queued form it isolates
// what the device queues and batch graphs contribute; against the FP64 plain
// form, what the screen contributes.
void run_gpu_stages_plain_screened(BsfHandle* h, int n) {
    check(cudaStreamSynchronize(h->stream), "world init");
    check(cudaMemsetAsync(h->dCounters, 0, sizeof(int), h->stream), "memset");
    launch_stage0_fast(h->cache, n, h->centers, h->prof, h->dRegions, nullptr, h->dCounters, 0, h->fs, h->stream,
                       h->persistent);
    h->launches += 2;
    const int regions = n * h->centers;
    h->hRegions.resize(regions);
    check(cudaMemcpyAsync(h->hRegions.data(), h->dRegions, sizeof(RegionInfo) * regions, cudaMemcpyDeviceToHost,
                          h->stream),
          "region download");
    check(cudaStreamSynchronize(h->stream), "stage0");
    std::vector<RegionRef> list;
    for (int i = 0; i < regions; ++i) {
        const RegionInfo& r = h->hRegions[i];
        if (r.p19Evaluated && r.p19Pass && !r.megaReject) list.push_back(RegionRef{i / h->centers, i % h->centers});
    }
    const int micro = std::min(1024, h->coarseCap);
    for (std::size_t off = 0; off < list.size(); off += micro) {
        const int chunk = static_cast<int>(std::min<std::size_t>(micro, list.size() - off));
        check(cudaMemcpyAsync(h->dCoarseQueue, list.data() + off, sizeof(RegionRef) * chunk, cudaMemcpyHostToDevice,
                              h->stream),
              "coarse list upload");
        check(cudaMemcpyAsync(h->dCounters, &chunk, sizeof(int), cudaMemcpyHostToDevice, h->stream), "count");
        launch_coarse_signs_fast(h->cache, h->dCoarseQueue, h->dCounters, chunk, h->dSigns, h->fs.stats, h->stream,
                                 h->persistent, h->fs.forceExact != 0);
        launch_coarse_cc(h->dCoarseQueue, h->dCounters, h->coarseCap, h->dSigns, h->dLabels, h->dStats, h->dRegions,
                         h->centers, h->stream);  // maxCount: as in run_gpu_stages_plain
        h->launches += 2;
        check(cudaStreamSynchronize(h->stream), "coarse micro-batch");
    }
}

void run_gpu_stages(BsfHandle* h, int n) {
    if (h->mode == BSF_MODE_PLAIN) run_gpu_stages_plain(h, n);
    else if (h->mode == BSF_MODE_PLAIN_SCREENED) run_gpu_stages_plain_screened(h, n);
    else run_gpu_stages_queued(h, n);
}

// Stage0 and coarse bracketed by events (event 2 sits between them in the
// queued form; in the plain forms the host round trips fall inside stage 1/2).
void run_gpu_stages_timed(BsfHandle* h, int n) {
    if (h->mode == BSF_MODE_PLAIN || h->mode == BSF_MODE_PLAIN_SCREENED) {
        if (h->mode == BSF_MODE_PLAIN) run_gpu_stages_plain(h, n);
        else run_gpu_stages_plain_screened(h, n);
        record(h, 2);
        record(h, 3);
        return;
    }
    run_gpu_stages_queued(h, n, true);
}

// Blocking device-to-host read on the handle's own stream (never the legacy
// default stream, which handles on other threads must not wait on).
void d2h(BsfHandle* h, void* dst, const void* src, std::size_t bytes, const char* what) {
    check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream), what);
    check(cudaStreamSynchronize(h->stream), what);
}

void read_stage_times(BsfHandle* h) {
    for (int i = 0; i < 2; ++i) check(cudaEventElapsedTime(&h->stageMs[i], h->ev[i], h->ev[i + 1]), "event time");
    check(cudaEventElapsedTime(&h->stageMs[2], h->ev[2], h->ev[3]), "event time");
}

Island exact_once(BsfHandle* h, ExactCtx& x, int world, int ccx, int ccz, int radius, const MatchSettings& ms,
                  bool preview) {
    if (radius > x.exact.maxRadius) throw std::length_error("exact radius exceeds the provisioned max_exact_radius");
    cudaStream_t st = x.stream ? x.stream : h->stream;
    // the plain form keeps the all-FP64 scan, as its other stages do
    const bool screened = h->mode != BSF_MODE_PLAIN && !h->fs.forceExact;
    h->launches += launch_exact_scan(h->cache, world, ccx, ccz, radius, ms, x.exact, x.dIsland,
                                     preview ? h->dPrevMin : nullptr, preview ? h->dPrevMax : nullptr, h->prevCap,
                                     screened, st);
    Island isl;
    int err = 0;
    check(cudaMemcpyAsync(&isl, x.dIsland, sizeof(Island), cudaMemcpyDeviceToHost, st), "island download");
    check(cudaMemcpyAsync(&err, x.exact.err, sizeof(int), cudaMemcpyDeviceToHost, st), "err");
    check(cudaStreamSynchronize(st), "exact scan");
    if (err) throw std::runtime_error("exact scan union-find exceeded its retry bound");
    return isl;
}

Island exact_once(BsfHandle* h, int world, int ccx, int ccz, int radius, const MatchSettings& ms, bool preview) {
    return exact_once(h, h->ectx[0], world, ccx, ccz, radius, ms, preview);
}

int compare_island(const Island& a, const Island& b) {
    if (a.blocks != b.blocks) return a.blocks < b.blocks ? -1 : 1;
    if (a.columns != b.columns) return a.columns < b.columns ? -1 : 1;
    const int areaA = (a.maxX - a.minX + 1) * (a.maxZ - a.minZ + 1);
    const int areaB = (b.maxX - b.minX + 1) * (b.maxZ - b.minZ + 1);
    if (areaA != areaB) return areaA < areaB ? -1 : 1;
    return 0;
}

// verifySideBorderMatch (IslandSearchEngine.java:3188-3260).
bool border_verify(BsfHandle* h, ExactCtx& x, int world, int ccx, int ccz, const MatchSettings& ms, Island& best) {
    static const int radii[5] = {10, 13, 16, 20, 24};
    for (int r : radii) {
        if (r <= best.radiusUsed) continue;
        const Island e = exact_once(h, x, world, ccx, ccz, r, ms, false);
        if (!e.found) return false;
        best = e;
        if (!best.touchesSide) return true;
    }
    return true;
}

// The steps of one region's resolution, for the candidate log.
struct ResolveDetail {
    Island raw{}, hot{};  // found == 0: none (raw after border verify; hot after border verify)
    bool hotScanned = false;
    int finalSource = 0;  // 0 none, 1 raw, 2 hot
};

// processGpuRegionAttempt (IslandSearchEngine.java:1878-1971).
Island resolve(BsfHandle* h, ExactCtx& x, int world, int ccx, int ccz, int radius, int coarse,
              const MatchSettings& ms, ResolveDetail* detail = nullptr) {
    Island normal = exact_once(h, x, world, ccx, ccz, radius, ms, false);
    bool have = normal.found != 0;
    if (have && normal.touchesSide && radius < 24) have = border_verify(h, x, world, ccx, ccz, ms, normal);
    Island match = normal;
    int source = have ? 1 : 0;
    if (detail) {
        detail->raw = have ? normal : Island{};
        detail->hot = Island{};
    }
    if (radius < 16 && coarse >= 120) {
        Island hot = exact_once(h, x, world, ccx, ccz, 16, ms, false);
        bool haveHot = hot.found != 0;
        if (haveHot && hot.touchesSide && hot.radiusUsed < 24) haveHot = border_verify(h, x, world, ccx, ccz, ms, hot);
        if (detail) {
            detail->hotScanned = true;
            if (haveHot) detail->hot = hot;
        }
        if (haveHot && (!have || compare_island(hot, match) > 0)) {
            match = hot;
            have = true;
            source = 2;
        }
    }
    if (detail) detail->finalSource = source;
    if (!have) {
        Island none{};
        none.radiusUsed = radius;
        return none;
    }
    return match;
}

// The GPU part of one batch, all on h->stream and free of host-side work, so it
// can be captured into a graph: seed upload (seedSource 2: from the handle's
// pinned staging; 1: from host `seeds` via the staging; 0: already in dSeeds
// or given as device `seeds`), generator setup, stages, stage counters and the
// download of the counters into pinned host memory.
void enqueue_batch(BsfHandle* h, int n, int seedSource, const std::int64_t* seeds) {
    check(cudaMemsetAsync(h->dCounters, 0, 4 * sizeof(int), h->stream), "memset");
    check(cudaMemsetAsync(h->dStageCounts, 0, 8 * sizeof(unsigned long long), h->stream), "memset");
    check(cudaMemsetAsync(h->fs.stats, 0, 4 * sizeof(unsigned long long), h->stream), "memset");
    check(cudaMemsetAsync(h->dCoarseErr, 0, sizeof(int), h->stream), "memset");
    record(h, 0);
    if (seedSource == 2) {
        check(cudaMemcpyAsync(h->dSeeds, h->hSeeds, static_cast<std::size_t>(n) * 8, cudaMemcpyHostToDevice,
                              h->stream), "seed upload");
        launch_world_init(h->dSeeds, n, h->cache, h->dCounters + 1, h->stream);
        ++h->launches;
    } else if (seedSource == 1) {
        stage_seeds(h, seeds, n, true);
    } else {
        launch_world_init(seeds ? seeds : h->dSeeds, n, h->cache, h->dCounters + 1, h->stream);
        ++h->launches;
    }
    record(h, 1);
    run_gpu_stages_timed(h, n);
    const int regions = n * h->centers;
    k_stage_counts<<<(regions + 255) / 256, 256, 0, h->stream>>>(h->dRegions, regions, h->prof, h->dStageCounts,
                                                                h->dExactQueue, h->dCounters + 2, h->exactCap,
                                                                h->centers);
    ++h->launches;
    check(cudaGetLastError(), "k_stage_counts");
    check(cudaMemcpyAsync(h->hPinned, h->dStageCounts, 8 * 8, cudaMemcpyDeviceToHost, h->stream), "counts");
    check(cudaMemcpyAsync(h->hPinned + 8, h->fs.stats, 4 * 8, cudaMemcpyDeviceToHost, h->stream), "screen stats");
    check(cudaMemcpyAsync(h->hPinned + 12, h->dCounters, 4 * sizeof(int), cudaMemcpyDeviceToHost, h->stream),
          "counts");
    check(cudaMemcpyAsync(h->hPinned + 14, h->dCoarseErr, sizeof(int), cudaMemcpyDeviceToHost, h->stream),
          "coarse flag");
    // the seeds the setup read: the caller's device array (seed source 0 with seeds given) or the handle's
    const std::int64_t* seedSrc = (seedSource == 0 && seeds) ? seeds : h->dSeeds;
    k_gather_exact<<<(h->exactCap + 127) / 128, 128, 0, h->stream>>>(h->dExactQueue, h->dCounters + 2, h->exactCap,
                                                                     h->dRegions, seedSrc, h->centers,
                                                                     h->dExactItems);
    ++h->launches;
    check(cudaGetLastError(), "k_gather_exact");
    check(cudaMemcpyAsync(h->hExactItems, h->dExactItems, sizeof(ExactItem) * kExactPrefix, cudaMemcpyDeviceToHost,
                          h->stream),
          "exact items");
}

// Kernels in one batch graph: setup, Stage0, P19, coarse signs, coarse score, counters, exact gather.
constexpr int kBatchGraphKernels = 7;

// Batches of a Stage0 sweep between two host reads of the survivor list (the
// list holds this many batches' worth, so it never overflows in between).
constexpr int kSweepFlush = 8;
// Kernels in one sweep-batch graph: seeds, setup, Stage0, P19, count, write, advance.
constexpr int kSweepGraphKernels = 7;

// Launch-shape, grid-shape, verification and profile state a graph was captured
// with (the profile's gates are kernel parameters of the graph).
int graph_variants(const BsfHandle* h) {
    return (((get_stage0_fast_variant() * 64 + get_coarse_fast_variant()) * 2 + (h->persistent ? 1 : 0)) * 2 +
            h->fs.forceExact) * 4 + h->cfg.profile;
}

// The cached graph of `key` on the handle's stream, captured from `enqueue` on a miss.
template <typename F>
cudaGraphExec_t cached_graph(BsfHandle* h, long long key, F&& enqueue) {
    const int variants = graph_variants(h);
    for (const auto& g : h->graphs)
        if (g.first == key && g.second.stream == h->stream && g.second.variants == variants) return g.second.exec;
    const unsigned long long launchesBefore = h->launches.load();
    cudaGraph_t graph = nullptr;
    std::shared_lock<std::shared_mutex> captureLock(capture_guard());
    check(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
    try {
        enqueue();
    } catch (...) {
        cudaStreamEndCapture(h->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    check(cudaStreamEndCapture(h->stream, &graph), "graph capture");
    cudaGraphExec_t exec = nullptr;
    const cudaError_t rc = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    check(rc, "graph instantiate");
    h->launches = launchesBefore;  // capture issued nothing; replays are counted per launch
    if (h->graphs.size() >= 8) {
        cudaGraphExecDestroy(h->graphs.front().second.exec);
        h->graphs.erase(h->graphs.begin());
    }
    h->graphs.push_back({key, BsfHandle::CachedGraph{exec, h->stream, variants}});
    return exec;
}

cudaGraphExec_t batch_graph(BsfHandle* h, int n, bool hostSeeds) {
    const long long key = static_cast<long long>(n) * 2 + (hostSeeds ? 1 : 0);
    return cached_graph(h, key, [&]() { enqueue_batch(h, n, hostSeeds ? 2 : 0, nullptr); });
}

// One Stage0 sweep batch of n worlds: seeds from the device cursor, generator
// setup, screened Stage0 (+ P19 fields), and the ordered survivor append.
cudaGraphExec_t sweep_graph(BsfHandle* h, int n) {
    const long long key = -1 - static_cast<long long>(n);  // batch graphs use keys >= 0
    return cached_graph(h, key, [&]() {
        launch_sweep_seeds(h->dSeeds, n, h->sweep, h->stream);
        launch_world_init(h->dSeeds, n, h->cache, h->dCounters + 1, h->stream);
        launch_stage0_fast(h->cache, n, h->centers, h->prof, h->dRegions, nullptr, h->dCounters, 0, h->fs, h->stream,
                           h->persistent);
        launch_sweep_compact(h->dRegions, h->dSeeds, n, h->centers, h->prof, h->sweep, h->stream);
    });
}

// Stage0 scout sweep over `count` consecutive seeds from `start`, in batches of
// the handle's capacity. The survivor list is read back every kSweepFlush
// batches; the list is in seed order, so the host only appends.
void stage0_sweep(BsfHandle* h, std::int64_t start, std::uint64_t count, std::int64_t* out, std::uint64_t cap,
                  std::uint64_t* nOut, bsf_sweep_counts* counts) {
    if (!nOut || count == 0 || (!out && cap)) throw std::invalid_argument("bsf_stage0_sweep: bad count/output");
    if (h->mode != BSF_MODE_QUEUED) throw std::invalid_argument("bsf_stage0_sweep runs in the queued form only");
    unsigned long long* hs = h->hSweep;
    hs[0] = static_cast<unsigned long long>(start);
    check(cudaMemcpyAsync(h->sweep.next, hs, 8, cudaMemcpyHostToDevice, h->stream), "sweep start");
    check(cudaMemsetAsync(h->sweep.total, 0, 8 * 5, h->stream), "memset");  // total + 4 stage counters
    check(cudaMemsetAsync(h->dCounters, 0, 4 * sizeof(int), h->stream), "memset");
    check(cudaMemsetAsync(h->fs.stats, 0, 4 * sizeof(unsigned long long), h->stream), "memset");
    std::uint64_t remaining = count, written = 0, survivors = 0;
    while (remaining) {
        for (int b = 0; b < kSweepFlush && remaining; ++b) {
            const int n = static_cast<int>(std::min<std::uint64_t>(remaining, static_cast<std::uint64_t>(h->capacity)));
            check(cudaGraphLaunch(sweep_graph(h, n), h->stream), "sweep graph");
            h->launches += kSweepGraphKernels;
            remaining -= static_cast<std::uint64_t>(n);
        }
        check(cudaMemcpyAsync(hs + 1, h->sweep.total, 8, cudaMemcpyDeviceToHost, h->stream), "sweep total");
        check(cudaStreamSynchronize(h->stream), "sweep");
        const std::uint64_t total = hs[1];
        if (total > h->sweep.outCap) throw std::runtime_error("sweep survivor list overflowed");
        const std::uint64_t take = written < cap ? std::min<std::uint64_t>(total, cap - written) : 0;
        if (take) {
            check(cudaMemcpyAsync(h->hSweepOut, h->sweep.out, take * 8, cudaMemcpyDeviceToHost, h->stream),
                  "survivors");
            check(cudaStreamSynchronize(h->stream), "survivors");
            std::memcpy(out + written, h->hSweepOut, take * 8);
            written += take;
        }
        survivors += total;
        check(cudaMemsetAsync(h->sweep.total, 0, 8, h->stream), "memset");
    }
    check(cudaMemcpyAsync(hs + 2, h->sweep.stage, 4 * 8, cudaMemcpyDeviceToHost, h->stream), "sweep counters");
    check(cudaMemcpyAsync(hs + 6, h->fs.stats, 2 * 8, cudaMemcpyDeviceToHost, h->stream), "screen stats");
    check(cudaMemcpyAsync(hs + 8, h->dCounters + 1, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "fallbacks");
    check(cudaStreamSynchronize(h->stream), "sweep counters");
    const int fallbacks = *reinterpret_cast<const int*>(hs + 8);
    if (hs[5] != survivors) throw std::runtime_error("sweep survivor count mismatch");
    h->lastBatch = 0;  // the region outcomes on the device are the sweep's now, not a MEGA batch's
    *nOut = survivors;
    if (counts) {
        counts->worlds = count;
        counts->regions = count * static_cast<std::uint64_t>(h->centers);
        counts->p20_passed = hs[2];
        counts->upper_passed = hs[3];
        counts->high_passed = hs[4];
        counts->survivors = survivors;
        counts->rng_fallbacks = static_cast<std::uint64_t>(fallbacks);
        counts->screened_tasks = hs[6];
        counts->fallback_tasks = hs[7];
    }
}

// Enqueues the GPU part of a batch of n worlds on h->stream, without a host sync.
void mega_begin(BsfHandle* h, const std::int64_t* seeds, bool hostSeeds, int n) {
    if (h->mode == BSF_MODE_QUEUED) {
        // Queued form: one CUDA graph per (batch size, seed source) replays the
        // whole GPU part of the batch; the seeds reach the handle's buffers first.
        if (hostSeeds) std::memcpy(h->hSeeds, seeds, static_cast<std::size_t>(n) * 8);
        else check(cudaMemcpyAsync(h->dSeeds, seeds, static_cast<std::size_t>(n) * 8, cudaMemcpyDeviceToDevice,
                                   h->stream), "seed copy");
        check(cudaGraphLaunch(batch_graph(h, n, hostSeeds), h->stream), "batch graph");
        h->launches += kBatchGraphKernels;
    } else {
        enqueue_batch(h, n, hostSeeds ? 1 : 0, seeds);
    }
}

void mega_end(BsfHandle* h, uint32_t count, int32_t radius, const MatchSettings& ms, bsf_mega_record* records,
              uint32_t recordsCap, uint32_t* recordsCount, bsf_stage_counts* counts);

int mega_batch(BsfHandle* h, const std::int64_t* seeds, bool hostSeeds, cudaStream_t userStream, uint32_t count,
               int32_t radius, const bsf_match_settings* s, bsf_mega_record* records, uint32_t recordsCap,
               uint32_t* recordsCount, bsf_stage_counts* counts) {
    if (!seeds || count == 0 || count > static_cast<uint32_t>(h->capacity) || (!records && recordsCap))
        throw std::invalid_argument("bsf_mega_search: bad seeds/count/records");
    if (radius < 0 || radius > h->exact.maxRadius) throw std::length_error("radius exceeds max_exact_radius");
    const MatchSettings ms = to_ms(s);
    struct StreamRestore {
        BsfHandle* h;
        cudaStream_t saved;
        ~StreamRestore() { h->stream = saved; }
    } restore{h, h->stream};
    if (userStream) h->stream = userStream;
    mega_begin(h, seeds, hostSeeds, static_cast<int>(count));
    mega_end(h, count, radius, ms, records, recordsCap, recordsCount, counts);
    return BSF_OK;
}

// Waits for the GPU part of the batch mega_begin enqueued, runs its exact stage
// and writes its records (world_index within the batch) and stage counts.
void mega_end(BsfHandle* h, uint32_t count, int32_t radius, const MatchSettings& ms, bsf_mega_record* records,
              uint32_t recordsCap, uint32_t* recordsCount, bsf_stage_counts* counts) {
    const int n = static_cast<int>(count);
    const int regions = n * h->centers;
    unsigned long long* hc = h->hPinned;
    unsigned long long* hs = h->hPinned + 8;
    const int* hcount = reinterpret_cast<const int*>(h->hPinned + 12);
    check(cudaStreamSynchronize(h->stream), "mega batch");
    if (hcount[0] > h->coarseCap) throw std::runtime_error("coarse queue exceeded its provisioned capacity");
    if (*reinterpret_cast<const int*>(h->hPinned + 14))
        throw std::runtime_error("coarse union-find exceeded its retry bound");
    read_stage_times(h);
    const auto exactStart = std::chrono::steady_clock::now();
    const int exactN = std::min(hcount[2], h->exactCap);
    if (exactN > kExactPrefix)
        d2h(h, h->hExactItems + kExactPrefix, h->dExactItems + kExactPrefix,
            sizeof(ExactItem) * (exactN - kExactPrefix), "exact items");
    // queue order varies between runs; records go out in (world, centre) order
    std::vector<ExactItem> items(h->hExactItems, h->hExactItems + exactN);
    std::sort(items.begin(), items.end(), [](const ExactItem& a, const ExactItem& b) {
        return a.ref.world != b.ref.world ? a.ref.world < b.ref.world : a.ref.center < b.ref.center;
    });
    std::vector<RegionRef> ex(exactN);
    std::vector<RegionInfo> info(exactN);
    for (int k = 0; k < exactN; ++k) {
        ex[k] = items[k].ref;
        info[k] = items[k].info;
    }
    // Exact stage: the regions are independent, so up to ectx.size() of them are
    // resolved at once, each by a host thread on its own stream and scratch.
    std::vector<Island> resolved(exactN);
    std::vector<ResolveDetail> details(exactN);
    const int lanes = std::min<int>(static_cast<int>(h->ectx.size()), exactN);
    if (lanes <= 1) {
        for (int k = 0; k < exactN; ++k)
            resolved[k] = resolve(h, h->ectx[0], ex[k].world, center_chunk_x(ex[k].center),
                                  center_chunk_z(ex[k].center), radius, info[k].coarse, ms, &details[k]);
    } else {
        std::atomic<int> next{0};
        std::vector<std::string> errors(lanes);
        auto work = [&](int t) {
            try {
                check(cudaSetDevice(h->cfg.device), "cudaSetDevice");
                for (int k = next.fetch_add(1); k < exactN; k = next.fetch_add(1))
                    resolved[k] = resolve(h, h->ectx[t], ex[k].world, center_chunk_x(ex[k].center),
                                          center_chunk_z(ex[k].center), radius, info[k].coarse, ms, &details[k]);
            } catch (const std::exception& e) {
                errors[t] = e.what();
                next.store(exactN);
            }
        };
        std::vector<std::thread> helpers;
        for (int t = 1; t < lanes; ++t) helpers.emplace_back(work, t);
        work(0);
        for (auto& t : helpers) t.join();
        for (const auto& e : errors)
            if (!e.empty()) throw std::runtime_error(e);
    }
    unsigned long long islands = 0;
    uint32_t written = 0;
    for (int k = 0; k < exactN; ++k) {
        const int ccx = center_chunk_x(ex[k].center), ccz = center_chunk_z(ex[k].center);
        const Island& isl = resolved[k];
        if (isl.found) ++islands;
        if (written < recordsCap) {
            bsf_mega_record& r = records[written++];
            r.seed = items[k].seed;
            r.world_index = ex[k].world;
            r.center_index = ex[k].center;
            r.center_chunk_x = ccx;
            r.center_chunk_z = ccz;
            r.p20 = info[k].p20;
            r.upper = info[k].upper;
            r.high = info[k].high;
            r.coarse = info[k].coarse;
            r.p19_score = info[k].p19Score;
            to_island(isl, &r.island);
            to_island(details[k].raw, &r.raw_island);
            to_island(details[k].hot, &r.hot_island);
            r.hot_scanned = details[k].hotScanned ? 1 : 0;
            r.final_source = details[k].finalSource;
            r.p19_pass = info[k].p19Pass;
            r.p19_extreme = info[k].p19Extreme;
        }
    }
    h->stageMs[3] = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - exactStart).count();
    h->lastBatch = n;
    if (recordsCount) *recordsCount = written;
    if (counts) {
        counts->worlds = count;
        counts->regions = static_cast<uint64_t>(regions);
        counts->p20_passed = hc[0];
        counts->upper_passed = hc[1];
        counts->high_passed = hc[2];
        counts->p19_passed = hc[3];
        counts->mega_rejected = hc[4];
        counts->coarse_evaluated = hc[5];
        counts->coarse_passed = hc[6];
        counts->islands = islands;
        counts->rng_fallbacks = static_cast<uint64_t>(hcount[1]);
        counts->lower_columns = hc[7];
        counts->screened_tasks = h->mode == BSF_MODE_PLAIN ? 0 : hs[0] + hs[2];
        counts->fallback_tasks = h->mode == BSF_MODE_PLAIN ? 0 : hs[1] + hs[3];
    }
}

// The pipeline's second handle: same config and settings, its own buffers,
// streams, graphs and exact-scan contexts. Opened on first use.
BsfHandle* twin_of(BsfHandle* h) {
    if (!h->twin) {
        void* t = bsf_open(&h->cfg);
        if (!t) throw std::runtime_error("out of memory opening the pipeline's second handle");
        BsfHandle* tw = static_cast<BsfHandle*>(t);
        if (!tw->ok) {
            const std::string msg = "opening the pipeline's second handle: " + tw->err;
            bsf_close(t);
            throw std::runtime_error(msg);
        }
        h->twin = tw;
    }
    BsfHandle* t = h->twin;
    t->mode = h->mode;
    t->persistent = h->persistent;
    t->prof = h->prof;
    t->cfg.profile = h->cfg.profile;
    t->fs.forceExact = h->fs.forceExact;
    return t;
}

// Exact-scan streams of the batch exact stage (contexts 1..) at the device's
// highest priority (or the default): in a pipelined range the next batch's
// Stage0 CTAs hold nearly all of each SM's shared memory, so an exact-scan
// kernel only starts when one of them retires, and at equal priority the block
// scheduler would start the next queued Stage0 CTA instead.
void set_exact_priority(BsfHandle* h, bool high) {
    if (h->exactHigh == high) return;
    int least = 0, greatest = 0;
    check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "priority range");
    for (std::size_t t = 1; t < h->ectx.size(); ++t) {
        ExactCtx& x = h->ectx[t];
        cudaStream_t s = nullptr;
        check(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, high ? greatest : least), "stream");
        if (x.stream) {
            check(cudaStreamSynchronize(x.stream), "stream");
            cudaStreamDestroy(x.stream);
        }
        x.stream = s;
    }
    h->exactHigh = high;
}

// Pipelined MEGA search over `count` worlds: batches of the handle's capacity
// alternate between h and its twin, and each batch's GPU part is enqueued
// before the previous batch's exact stage runs, so that exact stage (host
// threads, exact-context streams) overlaps the next batch's GPU stages.
void mega_range(BsfHandle* h, const std::int64_t* seeds, bool hostSeeds, cudaStream_t userStream, std::uint64_t count,
                int32_t radius, const bsf_match_settings* s, bsf_mega_record* records, uint32_t recordsCap,
                uint32_t* recordsCount, bsf_stage_counts* counts) {
    if (!seeds || count == 0 || count >= (1ull << 31) || (!records && recordsCap))
        throw std::invalid_argument("bsf_mega_search_range: bad seeds/count/records (count must be 1..2^31-1)");
    if (radius < 0 || radius > h->exact.maxRadius) throw std::length_error("radius exceeds max_exact_radius");
    const MatchSettings ms = to_ms(s);
    BsfHandle* hs[2] = {h, twin_of(h)};
    for (BsfHandle* x : hs) set_exact_priority(x, true);
    if (userStream) {
        // work the caller queued before the call (e.g. writing the seeds) comes first
        if (!h->rangeEvent) check(cudaEventCreateWithFlags(&h->rangeEvent, cudaEventDisableTiming), "event");
        check(cudaEventRecord(h->rangeEvent, userStream), "event");
        for (BsfHandle* x : hs) check(cudaStreamWaitEvent(x->stream, h->rangeEvent, 0), "stream wait");
    }
    const std::uint64_t cap = static_cast<std::uint64_t>(h->capacity);
    auto batchAt = [&](std::uint64_t off) { return static_cast<int>(std::min<std::uint64_t>(cap, count - off)); };
    bsf_stage_counts total{};
    uint32_t written = 0;
    std::uint64_t off = 0;
    int k = 0;
    try {
        mega_begin(hs[0], seeds, hostSeeds, batchAt(0));
        while (off < count) {
            BsfHandle* cur = hs[k & 1];
            const int n = batchAt(off);
            const std::uint64_t next = off + static_cast<std::uint64_t>(n);
            if (next < count) mega_begin(hs[(k + 1) & 1], seeds + next, hostSeeds, batchAt(next));
            uint32_t w = 0;
            bsf_stage_counts c{};
            mega_end(cur, static_cast<uint32_t>(n), radius, ms, records ? records + written : nullptr,
                     recordsCap - written, &w, &c);
            for (uint32_t i = 0; i < w; ++i) records[written + i].world_index += static_cast<int32_t>(off);
            written += w;
            std::uint64_t* dst = &total.worlds;
            const std::uint64_t* src = &c.worlds;
            for (std::size_t f = 0; f < sizeof(bsf_stage_counts) / sizeof(std::uint64_t); ++f) dst[f] += src[f];
            off = next;
            ++k;
        }
    } catch (...) {
        for (BsfHandle* x : hs) cudaStreamSynchronize(x->stream);  // no batch left in flight
        throw;
    }
    if (recordsCount) *recordsCount = written;
    if (counts) *counts = total;
}

// Every device buffer of a handle, sized from its config. With h->dry set this
// only sums the sizes (bsf_config_footprint); otherwise it allocates them.
void open_buffers(BsfHandle* h, const bsf_config& cfg) {
    h->capacity = static_cast<int>(cfg.capacity);
    h->centers = cfg.centers;
    h->prof = profile_by_id(cfg.profile);
    const std::size_t n = static_cast<std::size_t>(h->capacity);
    const std::size_t regions = n * h->centers;
    h->coarseCap = static_cast<int>(std::min<std::size_t>(regions, 1u << 14));
    h->exactCap = 4096;
    h->alloc(reinterpret_cast<void**>(&h->dSeeds), n * 8, "seeds");
    h->alloc(reinterpret_cast<void**>(&h->cache.perms), n * WORLD_PERM_BYTES, "state cache");
    h->alloc(reinterpret_cast<void**>(&h->cache.offsets), n * WORLD_OFFSETS * 8, "state cache");
    h->cache.capacity = h->capacity;
    h->alloc(reinterpret_cast<void**>(&h->dRegions), regions * sizeof(RegionInfo), "regions");
    h->alloc(reinterpret_cast<void**>(&h->dCoarseQueue), regions * sizeof(RegionRef), "coarse queue");
    h->alloc(reinterpret_cast<void**>(&h->dCounters), 16 * sizeof(int), "counters");
    const std::size_t cc = static_cast<std::size_t>(h->coarseCap);
    h->alloc(reinterpret_cast<void**>(&h->dSigns), cc * 61 * 61 * 4, "coarse signs");
    const std::size_t ctas = static_cast<std::size_t>(coarse_score_ctas(h->coarseCap));
    h->alloc(reinterpret_cast<void**>(&h->dLabels), ctas * 61 * 61 * 17 * 4, "coarse labels");
    h->alloc(reinterpret_cast<void**>(&h->dStats), ctas * 61 * 61 * 17 * 8 + 64, "coarse stats");
    if (!h->dry) h->dCoarseErr = h->dStats + ctas * 61 * 61 * 17 * 2;
    h->outBytes = regions * (cfg.research ? 34 : 16) + 64;
    h->alloc(reinterpret_cast<void**>(&h->dOut), std::max<std::size_t>(h->outBytes, n * 4096), "output");
    h->alloc(reinterpret_cast<void**>(&h->dHashes), n * 8, "hashes");
    h->alloc(reinterpret_cast<void**>(&h->dStageCounts), 8 * sizeof(unsigned long long), "stage counts");
    h->alloc(reinterpret_cast<void**>(&h->dExactQueue), h->exactCap * sizeof(RegionRef), "exact queue");
    h->alloc(reinterpret_cast<void**>(&h->dExactItems), h->exactCap * sizeof(ExactItem), "exact items");
    h->fs.p19Capacity = static_cast<int>(regions);
    h->alloc(reinterpret_cast<void**>(&h->fs.p19Queue), regions * sizeof(RegionRef), "p19 queue");
    h->alloc(reinterpret_cast<void**>(&h->fs.highest), regions * 256, "p19 grids");
    h->alloc(reinterpret_cast<void**>(&h->fs.p19Count), 64, "p19 count");
    h->alloc(reinterpret_cast<void**>(&h->fs.stats), 8 * sizeof(unsigned long long), "screen stats");
    if (!h->dry) check(cudaMemsetAsync(h->fs.stats, 0, 8 * sizeof(unsigned long long), h->stream), "memset");
    const std::size_t eb = exact_scratch_bytes(cfg.max_exact_radius);
    h->alloc(&h->dExactBase, eb, "exact scratch");
    if (!h->dry) {
        exact_scratch_carve(h->exact, h->dExactBase, cfg.max_exact_radius);
        check(cudaMemsetAsync(h->exact.err, 0, 64, h->stream), "memset");
    }
    h->alloc(reinterpret_cast<void**>(&h->dIsland), sizeof(Island), "island");
    // exact-scan contexts: the handle's own, plus seven more for batch handles
    // (capacity >= 1024) so that a batch's exact stage resolves regions at once
    // (measured per 16k-world batch: 2 contexts 12.3 ms, 4: 11.2 ms, 8: 10.2 ms)
    const int lanes = cfg.capacity >= 1024 ? 8 : 1;
    h->ectx.assign(lanes, ExactCtx{});
    h->ectx[0].exact = h->exact;
    h->ectx[0].dIsland = h->dIsland;
    for (int t = 1; t < lanes; ++t) {
        ExactCtx& x = h->ectx[t];
        h->alloc(&x.base, eb, "exact scratch");
        h->alloc(reinterpret_cast<void**>(&x.dIsland), sizeof(Island), "island");
        if (!h->dry) {
            exact_scratch_carve(x.exact, x.base, cfg.max_exact_radius);
            check(cudaMemsetAsync(x.exact.err, 0, 64, h->stream), "memset");
            check(cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking), "stream");
        }
    }
    h->prevCap = 16 * (2 * cfg.max_exact_radius + 1) * 16 * (2 * cfg.max_exact_radius + 1);
    h->alloc(reinterpret_cast<void**>(&h->dPrevMin), static_cast<std::size_t>(h->prevCap) * 4, "preview");
    h->alloc(reinterpret_cast<void**>(&h->dPrevMax), static_cast<std::size_t>(h->prevCap) * 4, "preview");
    // Stage0 sweep: cursor, total and stage counters (64 B), per-block counts, and a
    // survivor list that holds kSweepFlush batches (a batch has at most n survivors)
    const std::size_t blocks = static_cast<std::size_t>(sweep_blocks(h->capacity));
    h->sweep.outCap = static_cast<unsigned long long>(kSweepFlush) * n;
    const std::size_t sweepBytes = 64 + ((blocks * 4 + 255) / 256) * 256 + h->sweep.outCap * 8;
    h->alloc(&h->dSweepBase, sweepBytes, "sweep");
    if (!h->dry) {
        unsigned char* b = static_cast<unsigned char*>(h->dSweepBase);
        h->sweep.next = reinterpret_cast<unsigned long long*>(b);
        h->sweep.total = h->sweep.next + 1;
        h->sweep.stage = h->sweep.next + 2;  // 4 counters
        h->sweep.blockCounts = reinterpret_cast<int*>(b + 64);
        h->sweep.out = reinterpret_cast<std::int64_t*>(b + 64 + ((blocks * 4 + 255) / 256) * 256);
    }
}

// Constant tables and kernel attributes, once per device: handles opened later
// (from any thread) must not rewrite constant memory under running kernels.
void init_device_once(int device) {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), device) != done.end()) return;
    init_lcg_tables();
    init_stage0_fast();
    init_coarse_fast();
    init_exact_tables();
    done.push_back(device);
}

void validate_config(const bsf_config& cfg) {
    if (cfg.capacity < 1 || cfg.capacity > (1u << 22)) throw std::invalid_argument("capacity must be 1..4194304");
    if (cfg.centers != 1 && cfg.centers != 8) throw std::invalid_argument("centers must be 1 or 8");
    if (cfg.profile < 0 || cfg.profile > 3) throw std::invalid_argument("profile must be 0..3");
    if (cfg.max_exact_radius < 1 || cfg.max_exact_radius > 24)
        throw std::invalid_argument("max_exact_radius must be 1..24");
}

}  // namespace

extern "C" {

void bsf_default_config(bsf_config* c) {
    if (!c) return;
    c->device = 0;
    c->capacity = 32768;
    c->profile = BSF_PROFILE_MEGA;
    c->research = 0;
    c->centers = 8;
    c->max_exact_radius = 24;
}

void bsf_default_match_settings(bsf_match_settings* s) {
    if (!s) return;
    s->min_blocks = 1000;
    s->min_columns = 100;
    s->min_y_for_match = 60;
    s->min_width = 10;
    s->min_depth = 10;
    s->min_avg_thickness = 2.0;
}

void* bsf_open(const bsf_config* cfgIn) {
    BsfHandle* h = new (std::nothrow) BsfHandle();
    if (!h) return nullptr;
    bsf_config cfg;
    bsf_default_config(&cfg);
    if (cfgIn) cfg = *cfgIn;
    h->cfg = cfg;
    std::unique_lock<std::shared_mutex> allocLock(capture_guard());
    try {
        validate_config(cfg);
        check(cudaSetDevice(cfg.device), "cudaSetDevice");
        check(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
        init_device_once(cfg.device);
        open_buffers(h, cfg);
        const std::size_t n = static_cast<std::size_t>(h->capacity);
        for (auto& e : h->ev) check(cudaEventCreate(&e), "event");
        check(cudaMallocHost(reinterpret_cast<void**>(&h->hSeeds), n * 8), "pinned seeds");
        check(cudaMallocHost(reinterpret_cast<void**>(&h->hPinned), 16 * sizeof(unsigned long long)), "pinned counters");
        check(cudaMallocHost(reinterpret_cast<void**>(&h->hOut), std::max<std::size_t>(h->outBytes, n * 4096)),
              "pinned output");
        check(cudaMallocHost(reinterpret_cast<void**>(&h->hSweep), 16 * sizeof(unsigned long long)), "pinned sweep");
        check(cudaMallocHost(reinterpret_cast<void**>(&h->hExactItems), sizeof(ExactItem) * h->exactCap),
              "pinned exact items");
        check(cudaMallocHost(reinterpret_cast<void**>(&h->hSweepOut), h->sweep.outCap * 8), "pinned sweep list");
        check(cudaStreamSynchronize(h->stream), "open");
        h->ok = true;
    } catch (const std::exception& e) {
        h->err = e.what();
        h->ok = false;
    }
    return h;
}

void bsf_close(void* hv) {
    BsfHandle* h = static_cast<BsfHandle*>(hv);
    if (!h) return;
    if (h->twin) bsf_close(h->twin);
    if (h->rangeEvent) cudaEventDestroy(h->rangeEvent);
    if (h->stream) cudaStreamSynchronize(h->stream);
    std::unique_lock<std::shared_mutex> allocLock(capture_guard());
    h->drop_graphs();
    void* dev[] = {h->dSeeds, h->cache.perms, h->cache.offsets, h->dRegions, h->dCoarseQueue, h->dCounters,
                   h->dSigns, h->dLabels, h->dStats, h->dOut, h->dHashes, h->dStageCounts, h->dExactQueue,
                   h->dExactBase, h->dIsland, h->dPrevMin, h->dPrevMax, h->fs.p19Queue, h->fs.highest,
                   h->fs.p19Count, h->fs.stats, h->dSweepBase, h->dExactItems};
    for (void* p : dev)
        if (p) cudaFree(p);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    for (std::size_t t = 1; t < h->ectx.size(); ++t) {
        if (h->ectx[t].stream) cudaStreamDestroy(h->ectx[t].stream);
        if (h->ectx[t].base) cudaFree(h->ectx[t].base);
        if (h->ectx[t].dIsland) cudaFree(h->ectx[t].dIsland);
    }
    if (h->hSeeds) cudaFreeHost(h->hSeeds);
    if (h->hOut) cudaFreeHost(h->hOut);
    if (h->hPinned) cudaFreeHost(h->hPinned);
    if (h->hSweep) cudaFreeHost(h->hSweep);
    if (h->hExactItems) cudaFreeHost(h->hExactItems);
    if (h->hSweepOut) cudaFreeHost(h->hSweepOut);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int bsf_config_footprint(const bsf_config* cfg, uint64_t* bytes) {
    if (!cfg || !bytes) return BSF_E_ARG;
    try {
        validate_config(*cfg);
        BsfHandle h;
        h.dry = true;
        open_buffers(&h, *cfg);
        *bytes = h.footprint;
        return BSF_OK;
    } catch (const std::exception&) {
        return BSF_E_ARG;
    }
}

uint64_t bsf_handle_footprint(const void* hv) {
    const BsfHandle* h = static_cast<const BsfHandle*>(hv);
    return h ? h->footprint + (h->twin ? h->twin->footprint : 0) : 0;
}

int bsf_last_region_records(void* hv, uint8_t* out, size_t outLen) {
    return guarded(hv, [&](BsfHandle* h) {
        const int regions = h->lastBatch * h->centers;
        const std::size_t need = static_cast<std::size_t>(regions) * 34;
        if (!out || outLen < need || regions == 0)
            throw std::invalid_argument("bsf_last_region_records: no MEGA batch yet, or out_len too small");
        // dOut holds max(records, capacity * 4096) bytes: 34-byte records of every region always fit
        if (need > std::max<std::size_t>(h->outBytes, static_cast<std::size_t>(h->capacity) * 4096))
            throw std::length_error("bsf_last_region_records: output staging too small");
        k_pack_records<<<(regions + 255) / 256, 256, 0, h->stream>>>(h->dRegions, regions, 1, h->dOut);
        ++h->launches;
        check(cudaGetLastError(), "k_pack_records");
        d2h(h, out, h->dOut, need, "region records");
        return BSF_OK;
    });
}

int bsf_set_profile(void* hv, int32_t profile) {
    return guarded(hv, [&](BsfHandle* h) {
        if (profile < 0 || profile > 3) throw std::invalid_argument("profile must be 0..3");
        h->cfg.profile = profile;
        h->prof = profile_by_id(profile);
        return BSF_OK;
    });
}

int bsf_set_screening(void* hv, int32_t on) {
    return guarded(hv, [&](BsfHandle* h) {
        h->fs.forceExact = on ? 0 : 1;
        return BSF_OK;
    });
}

int bsf_set_persistent(void* hv, int32_t on) {
    return guarded(hv, [&](BsfHandle* h) {
        h->persistent = on != 0;
        return BSF_OK;
    });
}

int bsf_set_stream_priority(void* hv, int32_t high) {
    return guarded(hv, [&](BsfHandle* h) {
        int least = 0, greatest = 0;
        check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "priority range");
        cudaStream_t s = nullptr;
        std::unique_lock<std::shared_mutex> allocLock(capture_guard());
        check(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, high ? greatest : least), "stream");
        check(cudaStreamSynchronize(h->stream), "stream");
        h->drop_graphs();
        cudaStreamDestroy(h->stream);
        h->stream = s;
        return BSF_OK;
    });
}

const char* bsf_last_error(const void* hv) {
    const BsfHandle* h = static_cast<const BsfHandle*>(hv);
    if (!h) return "null handle";
    return h->err.c_str();
}

int bsf_set_mode(void* hv, int32_t mode) {
    return guarded(hv, [&](BsfHandle* h) {
        if (mode != BSF_MODE_QUEUED && mode != BSF_MODE_PLAIN && mode != BSF_MODE_PLAIN_SCREENED)
            throw std::invalid_argument("mode must be 0, 1 or 2");
        h->mode = mode;
        return BSF_OK;
    });
}

int bsf_stage0_filter(void* hv, const int64_t* seeds, uint32_t count, uint8_t* out, size_t outLen) {
    return guarded(hv, [&](BsfHandle* h) {
        const std::size_t rec = h->cfg.research ? 34 : 16;
        if (!seeds || !out || count == 0 || count > static_cast<uint32_t>(h->capacity))
            throw std::invalid_argument("bsf_stage0_filter: bad seeds/out/count (count must be 1..capacity)");
        const std::size_t need = static_cast<std::size_t>(count) * h->centers * rec;
        if (outLen < need) throw std::invalid_argument("bsf_stage0_filter: out_len too small");
        const int n = static_cast<int>(count);
        check(cudaMemsetAsync(h->dCounters, 0, 4 * sizeof(int), h->stream), "memset");
        stage_seeds(h, seeds, n, true);
        run_gpu_stages(h, n);
        const int regions = n * h->centers;
        k_pack_records<<<(regions + 255) / 256, 256, 0, h->stream>>>(h->dRegions, regions, h->cfg.research, h->dOut);
        ++h->launches;
        check(cudaGetLastError(), "k_pack_records");
        check(cudaMemcpyAsync(h->hOut, h->dOut, need, cudaMemcpyDeviceToHost, h->stream), "record download");
        int cnt[4];
        check(cudaMemcpyAsync(cnt, h->dCounters, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream), "counters");
        check(cudaStreamSynchronize(h->stream), "stage0 filter");
        if (cnt[0] > h->coarseCap) throw std::runtime_error("coarse queue exceeded its provisioned capacity");
        std::memcpy(out, h->hOut, need);
        return BSF_OK;
    });
}

int bsf_p20_filter(void* hv, const int64_t* seeds, uint32_t count, uint8_t* out, size_t outLen) {
    return guarded(hv, [&](BsfHandle* h) {
        if (!seeds || !out || count == 0 || count > static_cast<uint32_t>(h->capacity) || outLen < count)
            throw std::invalid_argument("bsf_p20_filter: bad seeds/out/count");
        const int n = static_cast<int>(count);
        stage_seeds(h, seeds, n, true);
        // The P20 count of centre 0 comes out of the fused Stage0 kernel; the
        // stream protocol reports it for the world's first region only.
        check(cudaMemsetAsync(h->dCounters, 0, sizeof(int), h->stream), "memset");
        if (h->mode == BSF_MODE_PLAIN)
            launch_stage0(h->cache, n, h->centers, h->prof, nullptr, h->dRegions, nullptr, h->dCounters, 0, h->stream);
        else
            launch_stage0_fast(h->cache, n, h->centers, h->prof, h->dRegions, nullptr, h->dCounters, 0, h->fs,
                               h->stream);
        k_pack_p20<<<(n + 255) / 256, 256, 0, h->stream>>>(h->dRegions, n, h->centers, h->dOut);
        h->launches += 2;
        check(cudaGetLastError(), "k_pack_p20");
        check(cudaMemcpyAsync(h->hOut, h->dOut, count, cudaMemcpyDeviceToHost, h->stream), "download");
        check(cudaStreamSynchronize(h->stream), "p20 filter");
        std::memcpy(out, h->hOut, count);
        return BSF_OK;
    });
}

int bsf_chunk_bitmaps(void* hv, const int64_t* seeds, uint32_t count, int32_t chunkX, int32_t chunkZ,
                      uint8_t* bitmaps, uint64_t* hashes) {
    return guarded(hv, [&](BsfHandle* h) {
        if (!seeds || !bitmaps || count == 0 || count > static_cast<uint32_t>(h->capacity))
            throw std::invalid_argument("bsf_chunk_bitmaps: bad seeds/bitmaps/count");
        if (chunkX < -(1 << 20) || chunkX > (1 << 20) || chunkZ < -(1 << 20) || chunkZ > (1 << 20))
            throw std::invalid_argument("bsf_chunk_bitmaps: chunk coordinate out of range");
        const int n = static_cast<int>(count);
        stage_seeds(h, seeds, n, true);
        launch_chunk_bitmaps(h->cache, n, chunkX, chunkZ, h->dOut, h->dHashes, h->stream);
        ++h->launches;
        check(cudaMemcpyAsync(h->hOut, h->dOut, static_cast<std::size_t>(n) * 4096, cudaMemcpyDeviceToHost, h->stream),
              "bitmap download");
        check(cudaStreamSynchronize(h->stream), "chunk bitmaps");
        std::memcpy(bitmaps, h->hOut, static_cast<std::size_t>(n) * 4096);
        if (hashes) d2h(h, hashes, h->dHashes, static_cast<std::size_t>(n) * 8, "hashes");
        return BSF_OK;
    });
}

static int single_world(BsfHandle* h, int64_t seed) {
    stage_seeds(h, &seed, 1, true);
    return 0;
}

int bsf_exact_scan(void* hv, int64_t seed, int32_t ccx, int32_t ccz, int32_t radius, const bsf_match_settings* s,
                   bsf_island* out) {
    return guarded(hv, [&](BsfHandle* h) {
        if (!out || radius < 0) throw std::invalid_argument("bsf_exact_scan: bad out/radius");
        const int w = single_world(h, seed);
        to_island(exact_once(h, w, ccx, ccz, radius, to_ms(s), false), out);
        return BSF_OK;
    });
}

int bsf_resolve_region(void* hv, int64_t seed, int32_t ccx, int32_t ccz, int32_t radius, int32_t coarse,
                       const bsf_match_settings* s, bsf_island* out) {
    return guarded(hv, [&](BsfHandle* h) {
        if (!out || radius < 0) throw std::invalid_argument("bsf_resolve_region: bad out/radius");
        if (h->exact.maxRadius < 24) throw std::length_error("bsf_resolve_region needs max_exact_radius 24");
        const int w = single_world(h, seed);
        to_island(resolve(h, h->ectx[0], w, ccx, ccz, radius, coarse, to_ms(s)), out);
        return BSF_OK;
    });
}

int bsf_preview(void* hv, int64_t seed, int32_t ccx, int32_t ccz, int32_t radius, const bsf_match_settings* s,
                bsf_island* out, int32_t* minY, int32_t* maxY, uint32_t capacity) {
    return guarded(hv, [&](BsfHandle* h) {
        if (!out || !minY || !maxY || radius < 0) throw std::invalid_argument("bsf_preview: bad arguments");
        const int w = single_world(h, seed);
        const Island isl = exact_once(h, w, ccx, ccz, radius, to_ms(s), true);
        to_island(isl, out);
        if (!isl.found) return BSF_OK;
        const std::size_t cells = static_cast<std::size_t>(isl.maxX - isl.minX + 1) * (isl.maxZ - isl.minZ + 1);
        if (cells > capacity) throw std::length_error("bsf_preview: capacity smaller than the island footprint");
        d2h(h, minY, h->dPrevMin, cells * 4, "preview");
        d2h(h, maxY, h->dPrevMax, cells * 4, "preview");
        return BSF_OK;
    });
}

int bsf_mega_search(void* hv, const int64_t* seeds, uint32_t count, int32_t radius, const bsf_match_settings* s,
                    bsf_mega_record* records, uint32_t recordsCap, uint32_t* recordsCount, bsf_stage_counts* counts) {
    return guarded(hv, [&](BsfHandle* h) {
        return mega_batch(h, seeds, true, nullptr, count, radius, s, records, recordsCap, recordsCount, counts);
    });
}

int bsf_mega_search_device(void* hv, const int64_t* dSeeds, uint32_t count, int32_t radius,
                           const bsf_match_settings* s, bsf_mega_record* records, uint32_t recordsCap,
                           uint32_t* recordsCount, bsf_stage_counts* counts, void* stream) {
    return guarded(hv, [&](BsfHandle* h) {
        return mega_batch(h, dSeeds, false, static_cast<cudaStream_t>(stream), count, radius, s, records, recordsCap,
                          recordsCount, counts);
    });
}

int bsf_stage0_sweep(void* hv, int64_t startSeed, uint64_t count, int64_t* survivors, uint64_t cap,
                     uint64_t* nSurvivors, bsf_sweep_counts* counts) {
    return guarded(hv, [&](BsfHandle* h) {
        stage0_sweep(h, startSeed, count, survivors, cap, nSurvivors, counts);
        return BSF_OK;
    });
}

int bsf_mega_search_range(void* hv, const int64_t* seeds, uint64_t count, int32_t radius, const bsf_match_settings* s,
                          bsf_mega_record* records, uint32_t recordsCap, uint32_t* recordsCount,
                          bsf_stage_counts* counts) {
    return guarded(hv, [&](BsfHandle* h) {
        mega_range(h, seeds, true, nullptr, count, radius, s, records, recordsCap, recordsCount, counts);
        return BSF_OK;
    });
}

int bsf_mega_search_range_device(void* hv, const int64_t* dSeeds, uint64_t count, int32_t radius,
                                 const bsf_match_settings* s, bsf_mega_record* records, uint32_t recordsCap,
                                 uint32_t* recordsCount, bsf_stage_counts* counts, void* stream) {
    return guarded(hv, [&](BsfHandle* h) {
        mega_range(h, dSeeds, false, static_cast<cudaStream_t>(stream), count, radius, s, records, recordsCap,
                   recordsCount, counts);
        return BSF_OK;
    });
}

int bsf_last_stage_ms(const void* hv, float* ms4) {
    const BsfHandle* h = static_cast<const BsfHandle*>(hv);
    if (!h || !ms4) return BSF_E_ARG;
    for (int i = 0; i < 4; ++i) ms4[i] = h->stageMs[i];
    return BSF_OK;
}

int bsf_autotune(void* hv, uint32_t worlds, char* report, size_t reportLen) {
    return guarded(hv, [&](BsfHandle* h) {
        const int n = static_cast<int>(std::min<uint32_t>(std::max<uint32_t>(worlds, 64u), h->capacity));
        std::vector<std::int64_t> seeds(n);
        for (int i = 0; i < n; ++i) seeds[i] = 0x5DEECE66DLL * 7919 + i;  // fixed calibration range
        std::string rep;
        char buf[96];
        cudaEvent_t e0 = h->ev[0], e1 = h->ev[1];
        stage_seeds(h, seeds.data(), n, true);
        auto time_it = [&](auto&& fn) {
            fn();  // warm-up (module load, caches)
            check(cudaEventRecord(e0, h->stream), "event");
            fn();
            check(cudaEventRecord(e1, h->stream), "event");
            check(cudaEventSynchronize(e1), "autotune");
            float ms = 0.0f;
            check(cudaEventElapsedTime(&ms, e0, e1), "event");
            return ms;
        };
        auto stage0 = [&]() {
            check(cudaMemsetAsync(h->dCounters, 0, sizeof(int), h->stream), "memset");
            launch_stage0_fast(h->cache, n, h->centers, h->prof, h->dRegions, h->dCoarseQueue, h->dCounters,
                               h->capacity * h->centers, h->fs, h->stream, h->persistent);
        };
        int best = 0;
        float bestMs = 1e30f;
        rep += "stage0:";
        for (int v = 0; v < stage0_fast_variants(); ++v) {
            set_stage0_fast_variant(v);
            const float ms = time_it(stage0);
            std::snprintf(buf, sizeof(buf), " %s=%.2fms", stage0_fast_variant_name(v), ms);
            rep += buf;
            if (ms < bestMs) { bestMs = ms; best = v; }
        }
        set_stage0_fast_variant(best);
        rep += std::string(" -> ") + stage0_fast_variant_name(best) + "; coarse:";
        stage0();  // leaves the coarse queue of the calibration batch on the device
        best = 0;
        bestMs = 1e30f;
        for (int v = 0; v < coarse_fast_variants(); ++v) {
            set_coarse_fast_variant(v);
            const float ms = time_it([&]() {
                launch_coarse_signs_fast(h->cache, h->dCoarseQueue, h->dCounters, h->coarseCap, h->dSigns, nullptr,
                                         h->stream, h->persistent);
            });
            std::snprintf(buf, sizeof(buf), " %s=%.2fms", coarse_fast_variant_name(v), ms);
            rep += buf;
            if (ms < bestMs) { bestMs = ms; best = v; }
        }
        set_coarse_fast_variant(best);
        rep += std::string(" -> ") + coarse_fast_variant_name(best);
        // grid shape with the chosen variants: persistent CTAs looping over worlds and
        // half-regions, or one CTA per world pair and per half-region
        float gridMs[2];
        for (int persistent = 1; persistent >= 0; --persistent) {
            h->persistent = persistent != 0;
            gridMs[persistent] = time_it([&]() {
                stage0();
                launch_coarse_signs_fast(h->cache, h->dCoarseQueue, h->dCounters, h->coarseCap, h->dSigns, nullptr,
                                         h->stream, h->persistent);
            });
        }
        h->persistent = gridMs[1] <= gridMs[0];
        std::snprintf(buf, sizeof(buf), "; grid: persistent=%.2fms per-item=%.2fms -> %s", gridMs[1], gridMs[0],
                      h->persistent ? "persistent" : "per-item");
        rep += buf;
        check(cudaStreamSynchronize(h->stream), "autotune");
        if (report && reportLen) {
            std::strncpy(report, rep.c_str(), reportLen - 1);
            report[reportLen - 1] = '\0';
        }
        return BSF_OK;
    });
}

int bsf_set_launch_variants(void* hv, int32_t s0, int32_t co) {
    return guarded(hv, [&](BsfHandle*) {
        if (s0 < 0 || s0 >= stage0_fast_variants() || co < 0 || co >= coarse_fast_variants())
            throw std::invalid_argument("bsf_set_launch_variants: variant index out of range");
        set_stage0_fast_variant(s0);
        set_coarse_fast_variant(co);
        return BSF_OK;
    });
}

int bsf_measure_peaks(double* ops) {
    if (!ops) return BSF_E_ARG;
    try {
        int dev = 0, sms = 0;
        check(cudaGetDevice(&dev), "device");
        check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
        void* out = nullptr;
        check(cudaMalloc(&out, 64), "probe buffer");
        cudaEvent_t e0, e1;
        check(cudaEventCreate(&e0), "event");
        check(cudaEventCreate(&e1), "event");
        const int blocks = sms * 8, threads = 256;
        for (int kind = 0; kind < 2; ++kind) {
            const int iters = kind == 0 ? 4096 : 262144;
            float best = 1e30f;
            for (int rep = 0; rep < 4; ++rep) {
                check(cudaEventRecord(e0), "event");
                if (kind == 0) k_add_chains<double><<<blocks, threads>>>(static_cast<double*>(out), iters, 1e-9);
                else k_add_chains<float><<<blocks, threads>>>(static_cast<float*>(out), iters, 1e-9f);
                check(cudaEventRecord(e1), "event");
                check(cudaEventSynchronize(e1), "probe");
                float ms = 0;
                check(cudaEventElapsedTime(&ms, e0, e1), "event");
                if (rep > 0 && ms < best) best = ms;
            }
            ops[kind] = static_cast<double>(blocks) * threads * 8.0 * iters / (best / 1e3);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(out);
        return BSF_OK;
    } catch (const std::exception&) {
        return BSF_E_CUDA;
    }
}

int bsf_device_summary(int32_t device, char* out, size_t outLen) {
    if (!out || outLen == 0) return BSF_E_ARG;
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BSF_E_CUDA;
    std::snprintf(out, outLen, "GPU: %s\nArchitecture: sm_%d%d\nCompute units: %d\nGlobal memory: %g GiB\n",
                  prop.name, prop.major, prop.minor, prop.multiProcessorCount,
                  static_cast<double>(prop.totalGlobalMem) / (1024.0 * 1024.0 * 1024.0));
    return BSF_OK;
}

uint64_t bsf_kernel_launches(const void* hv) {
    const BsfHandle* h = static_cast<const BsfHandle*>(hv);
    if (!h) return 0;
    return h->launches.load() + (h->twin ? h->twin->launches.load() : 0);
}

}  // extern "C"
