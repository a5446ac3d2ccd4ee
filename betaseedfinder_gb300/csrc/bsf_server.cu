// Served mode of libbsf (bsf_server_* in include/bsf.h): a request loop over
// device-resident lanes with continuous batching and admission by HBM footprint.
//
// A lane is one libbsf handle (its own stream, generator cache, stage queues
// and exact-scan scratch) of one request class: RANGE lanes hold chunk_worlds
// worlds of MEGA pipeline state, PREVIEW lanes one world and exact-scan scratch
// up to max_preview_radius. Lanes stay open between requests, so generator
// tables, queues and CUDA graphs are reused. max_lanes range worker threads each
// run one chunk of a range request at a time on a lane, and preview_lanes
// preview worker threads one preview each, so a preview never waits on the
// host for a range chunk. On the device, preview lanes use the highest stream
// priority and range lanes launch their screened kernels one CTA per world, so
// preview CTAs take SM slots as soon as any world finishes. A unit is admitted
// when an idle lane of its class exists, or when a new lane's footprint
// (bsf_config_footprint) fits in the HBM budget, closing idle lanes of the other
// class if that makes room; otherwise it waits until a lane comes free. Because range requests are handed out a chunk
// at a time, a request that arrives while others run starts at the next chunk
// boundary, and the lanes' streams overlap on the device.
//
// The reference serves these two classes from the Java app: range scans through
// IslandSearchEngine's GPU worker path (src/IslandSearchEngine.java:1878-1971)
// and previews through generate3DPreviewForIsland -> buildIsland3DData
// (src/IslandSearchEngine.java:284-436), one request at a time per worker.
#include "../../include/bsf.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

// The GPU runs the streams of a process on CUDA_DEVICE_MAX_CONNECTIONS hardware
// queues (8 unless set); streams beyond that share queues, and a kernel then
// waits for every earlier kernel of any stream on its queue. A preview lane's
// stream sharing a queue with a range lane's stream would wait for that lane's
// Stage0 kernel (hundreds of ms under load) however high its priority. The
// library raises the queue count to the maximum when it is loaded, unless the
// process set it; it takes effect only if no CUDA context exists yet.
__attribute__((constructor)) void raise_hardware_queues() { setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0); }

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

constexpr std::uint32_t kChunkRecords = 4096;  // exact-stage regions one chunk can return

struct Request {
    std::uint64_t ticket = 0;
    int kind = BSF_REQ_RANGE;
    bsf_match_settings ms{};
    std::int32_t radius = 7;
    std::int32_t profile = BSF_PROFILE_MEGA;  // RANGE: hunt profile of the request
    Clock::time_point submitted{};
    bool started = false;
    bool deferredCounted = false;
    // RANGE
    std::vector<std::int64_t> seeds;
    std::uint32_t next = 0, inflight = 0, done = 0;
    bool aborted = false;
    std::vector<bsf_mega_record> records;
    bsf_stage_counts counts{};
    // PREVIEW
    std::int64_t seed = 0;
    std::int32_t cx = 0, cz = 0;
    std::vector<std::int32_t> minY, maxY;
    // result
    bool finished = false;
    bsf_server_result res{};
};

struct Lane {
    int kind = BSF_REQ_RANGE;
    void* h = nullptr;
    std::uint64_t bytes = 0;
    bool busy = false;
};

struct Work {
    Request* req = nullptr;
    Lane* lane = nullptr;
    bool openLane = false;
    std::vector<void*> evicted;  // handles of idle lanes closed to make room
    std::uint32_t begin = 0, end = 0;
};

struct Server {
    bsf_server_config cfg{};
    bsf_config laneCfg[2]{};
    std::uint64_t laneBytes[2] = {0, 0};
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<Request*> previews;
    std::deque<Request*> ranges;  // requests with chunks left to hand out, round robin
    std::map<std::uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<std::unique_ptr<Lane>> lanes;
    std::vector<std::thread> workers;
    bool stopping = false;
    std::uint64_t nextTicket = 1;
    std::uint64_t bytesInUse = 0, bytesPeak = 0;
    std::uint32_t busyLanes = 0, maxBusy = 0;
    std::uint64_t submitted[2] = {0, 0}, completed[2] = {0, 0}, failed[2] = {0, 0};
    std::uint64_t worldsCompleted = 0, deferred = 0, evictions = 0;
    std::vector<double> latency[2];
    std::string err;
};

void add_counts(bsf_stage_counts& into, const bsf_stage_counts& c) {
    static_assert(sizeof(bsf_stage_counts) % sizeof(uint64_t) == 0, "bsf_stage_counts holds uint64_t fields only");
    uint64_t* a = reinterpret_cast<uint64_t*>(&into);
    const uint64_t* b = reinterpret_cast<const uint64_t*>(&c);
    for (std::size_t i = 0; i < sizeof(bsf_stage_counts) / sizeof(uint64_t); ++i) a[i] += b[i];
}

// A lane for one unit of `kind`, under the lock: an idle lane, else a new one if
// its footprint fits the budget, else a new one after closing idle lanes of the
// other class. The new lane is reserved (busy, bytes counted) and opened by the
// worker outside the lock.
bool try_lane(Server& S, int kind, Work& w) {
    for (auto& l : S.lanes)
        if (l->kind == kind && !l->busy && l->h) {
            w.lane = l.get();
            return true;
        }
    const std::uint64_t need = S.laneBytes[kind];
    const std::uint64_t budget = S.cfg.hbm_budget_bytes;
    std::vector<std::size_t> victims;
    std::uint64_t freed = 0;
    if (S.bytesInUse + need > budget) {
        for (std::size_t i = 0; i < S.lanes.size() && S.bytesInUse - freed + need > budget; ++i) {
            const Lane& l = *S.lanes[i];
            if (l.kind != kind && !l.busy && l.h) {
                victims.push_back(i);
                freed += l.bytes;
            }
        }
        if (S.bytesInUse - freed + need > budget) return false;
    }
    for (auto it = victims.rbegin(); it != victims.rend(); ++it) {
        w.evicted.push_back(S.lanes[*it]->h);
        S.bytesInUse -= S.lanes[*it]->bytes;
        S.lanes.erase(S.lanes.begin() + static_cast<std::ptrdiff_t>(*it));
        ++S.evictions;
    }
    auto lane = std::make_unique<Lane>();
    lane->kind = kind;
    lane->bytes = need;
    w.lane = lane.get();
    w.openLane = true;
    S.lanes.push_back(std::move(lane));
    S.bytesInUse += need;
    S.bytesPeak = std::max(S.bytesPeak, S.bytesInUse);
    return true;
}

void note_deferred(Server& S, Request* r) {
    if (!r->deferredCounted) {
        r->deferredCounted = true;
        ++S.deferred;
    }
}

// Next unit of work of one class, under the lock: a preview, or one chunk of the
// range request at the head of the round robin.
bool pick(Server& S, Work& w, int cls) {
    if (cls == BSF_REQ_PREVIEW && !S.previews.empty()) {
        if (try_lane(S, BSF_REQ_PREVIEW, w)) {
            w.req = S.previews.front();
            S.previews.pop_front();
        } else {
            note_deferred(S, S.previews.front());
        }
    }
    if (cls == BSF_REQ_RANGE && !S.ranges.empty()) {
        if (try_lane(S, BSF_REQ_RANGE, w)) {
            Request* r = S.ranges.front();
            S.ranges.pop_front();
            const std::uint32_t n = static_cast<std::uint32_t>(r->seeds.size());
            w.req = r;
            w.begin = r->next;
            w.end = std::min<std::uint32_t>(n, r->next + S.cfg.chunk_worlds);
            r->next = w.end;
            ++r->inflight;
            if (r->next < n) S.ranges.push_back(r);
        } else {
            note_deferred(S, S.ranges.front());
        }
    }
    if (!w.req) return false;
    if (!w.req->started) {
        w.req->started = true;
        w.req->res.queue_ms = ms_between(w.req->submitted, Clock::now());
    }
    w.lane->busy = true;
    ++S.busyLanes;
    S.maxBusy = std::max(S.maxBusy, S.busyLanes);
    return true;
}

void finish(Server& S, Request* r) {
    r->res.latency_ms = ms_between(r->submitted, Clock::now());
    r->finished = true;
    if (r->res.status == BSF_OK) {
        ++S.completed[r->kind];
        S.latency[r->kind].push_back(r->res.latency_ms);
    } else {
        ++S.failed[r->kind];
    }
}

std::string lane_error(void* h, const char* what) {
    const char* e = h ? bsf_last_error(h) : "handle allocation failed";
    return std::string(what) + ": " + (e ? e : "");
}

void run_unit(Server* S, Work& w, int& status, std::string& err, std::vector<bsf_mega_record>& recs,
              std::uint32_t& nrec, bsf_stage_counts& counts, bsf_island& isl, std::vector<std::int32_t>& mn,
              std::vector<std::int32_t>& mx) {
    Request* r = w.req;
    void* h = w.lane->h;
    if (r->kind == BSF_REQ_RANGE) {
        recs.resize(kChunkRecords);
        status = bsf_set_profile(h, r->profile);
        if (status == BSF_OK)
            status = bsf_mega_search(h, r->seeds.data() + w.begin, w.end - w.begin, r->radius, &r->ms, recs.data(),
                                     kChunkRecords, &nrec, &counts);
        if (status != BSF_OK) err = lane_error(h, "range chunk");
        return;
    }
    const std::uint32_t side = 2u * static_cast<std::uint32_t>(r->radius) + 1u;
    const std::uint32_t cap = 256u * side * side;
    mn.resize(cap);
    mx.resize(cap);
    status = bsf_preview(h, r->seed, r->cx, r->cz, r->radius, &r->ms, &isl, mn.data(), mx.data(), cap);
    if (status != BSF_OK) err = lane_error(h, "preview");
}

// Preview lanes: highest stream priority. Range lanes: one CTA per world in the
// screened kernels, so they yield SM slots to preview kernels every world.
void configure_lane(void* h, int kind) {
    if (kind == BSF_REQ_PREVIEW) bsf_set_stream_priority(h, 1);
    else bsf_set_persistent(h, 0);
}

void worker_loop(Server* S, int cls) {
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        Work w;
        while (!S->stopping && !pick(*S, w, cls)) S->cvWork.wait(lk);
        if (!w.req) return;
        lk.unlock();
        for (void* h : w.evicted) bsf_close(h);
        int status = BSF_OK;
        std::string err;
        bool laneDead = false;
        if (w.openLane) {
            void* h = bsf_open(&S->laneCfg[w.lane->kind]);
            const char* e = h ? bsf_last_error(h) : "handle allocation failed";
            if (!h || (e && e[0])) {
                status = BSF_E_CUDA;
                err = std::string("opening a lane: ") + (e ? e : "");
                if (h) bsf_close(h);
                laneDead = true;
            } else {
                configure_lane(h, w.lane->kind);
                w.lane->h = h;
            }
        }
        std::vector<bsf_mega_record> recs;
        std::uint32_t nrec = 0;
        bsf_stage_counts counts{};
        bsf_island isl{};
        std::vector<std::int32_t> mn, mx;
        if (status == BSF_OK) {
            run_unit(S, w, status, err, recs, nrec, counts, isl, mn, mx);
            // a handle whose device context failed stays unusable: retire its lane
            if (status == BSF_E_STATE || status == BSF_E_CUDA) laneDead = true;
        }
        lk.lock();
        Request* r = w.req;
        if (!err.empty()) S->err = err;
        if (r->kind == BSF_REQ_RANGE) {
            for (std::uint32_t k = 0; k < nrec; ++k) {
                bsf_mega_record rec = recs[k];
                rec.world_index += static_cast<std::int32_t>(w.begin);
                r->records.push_back(rec);
            }
            add_counts(r->counts, counts);
            --r->inflight;
            r->done += w.end - w.begin;
            if (status == BSF_OK) S->worldsCompleted += w.end - w.begin;
            if (status != BSF_OK && r->res.status == BSF_OK) {
                r->res.status = status;
                r->aborted = true;
                S->ranges.erase(std::remove(S->ranges.begin(), S->ranges.end(), r), S->ranges.end());
            }
            const bool allOut = r->aborted || r->next >= r->seeds.size();
            if (allOut && r->inflight == 0) {
                std::sort(r->records.begin(), r->records.end(), [](const bsf_mega_record& a, const bsf_mega_record& b) {
                    return a.world_index != b.world_index ? a.world_index < b.world_index
                                                          : a.center_index < b.center_index;
                });
                r->res.records = static_cast<std::uint32_t>(r->records.size());
                r->res.counts = r->counts;
                finish(*S, r);
            }
        } else {
            r->res.status = status;
            r->res.island = isl;
            if (status == BSF_OK && isl.found) {
                const std::uint32_t cells = static_cast<std::uint32_t>((isl.max_x - isl.min_x + 1)) *
                                            static_cast<std::uint32_t>((isl.max_z - isl.min_z + 1));
                mn.resize(cells);
                mx.resize(cells);
                r->minY = std::move(mn);
                r->maxY = std::move(mx);
                r->res.preview_columns = cells;
            }
            finish(*S, r);
        }
        w.lane->busy = false;
        --S->busyLanes;
        if (laneDead) {
            void* h = w.lane->h;
            S->bytesInUse -= w.lane->bytes;
            S->lanes.erase(std::remove_if(S->lanes.begin(), S->lanes.end(),
                                          [&](const std::unique_ptr<Lane>& l) { return l.get() == w.lane; }),
                           S->lanes.end());
            if (h) {
                lk.unlock();
                bsf_close(h);
                lk.lock();
            }
        }
        S->cvWork.notify_all();
        S->cvDone.notify_all();
    }
}

Request* find(Server* S, std::uint64_t ticket) {
    auto it = S->reqs.find(ticket);
    return it == S->reqs.end() ? nullptr : it->second.get();
}

void percentiles(std::vector<double> v, double& p50, double& p99, double& p999) {
    p50 = p99 = p999 = 0.0;
    if (v.empty()) return;
    std::sort(v.begin(), v.end());
    auto rank = [&](double q) {  // nearest-rank percentile
        std::size_t k = static_cast<std::size_t>(q * static_cast<double>(v.size()) + 0.999999999);
        k = std::max<std::size_t>(k, 1);
        return v[std::min(k, v.size()) - 1];
    };
    p50 = rank(0.50);
    p99 = rank(0.99);
    p999 = rank(0.999);
}

}  // namespace

extern "C" {

void bsf_default_server_config(bsf_server_config* c) {
    if (!c) return;
    c->device = 0;
    c->profile = BSF_PROFILE_MEGA;
    c->hbm_budget_bytes = 0;
    c->chunk_worlds = 8192;
    c->max_lanes = 4;
    c->preview_lanes = 2;
    c->max_preview_radius = 16;
}

void* bsf_server_open(const bsf_server_config* cfgIn) {
    Server* S = new (std::nothrow) Server();
    if (!S) return nullptr;
    bsf_server_config cfg;
    bsf_default_server_config(&cfg);
    if (cfgIn) cfg = *cfgIn;
    if (cfg.chunk_worlds < 1 || cfg.chunk_worlds > (1u << 20) || cfg.max_lanes < 1 || cfg.max_lanes > 64 ||
        cfg.preview_lanes < 1 || cfg.preview_lanes > 64 || cfg.max_preview_radius < 1 ||
        cfg.max_preview_radius > 24 || cfg.profile < 0 || cfg.profile > 3) {
        S->err = "bad server config (chunk_worlds 1..1048576, max_lanes 1..64, preview_lanes 1..64, "
                 "max_preview_radius 1..24, profile 0..3)";
        S->stopping = true;
        return S;
    }
    for (int k = 0; k < 2; ++k) bsf_default_config(&S->laneCfg[k]);
    S->laneCfg[BSF_REQ_RANGE].device = cfg.device;
    S->laneCfg[BSF_REQ_RANGE].capacity = cfg.chunk_worlds;
    S->laneCfg[BSF_REQ_RANGE].profile = cfg.profile;
    S->laneCfg[BSF_REQ_RANGE].centers = 8;
    S->laneCfg[BSF_REQ_RANGE].max_exact_radius = 24;
    S->laneCfg[BSF_REQ_PREVIEW].device = cfg.device;
    S->laneCfg[BSF_REQ_PREVIEW].capacity = 1;
    S->laneCfg[BSF_REQ_PREVIEW].profile = cfg.profile;
    S->laneCfg[BSF_REQ_PREVIEW].centers = 1;
    S->laneCfg[BSF_REQ_PREVIEW].max_exact_radius = cfg.max_preview_radius;
    for (int k = 0; k < 2; ++k) bsf_config_footprint(&S->laneCfg[k], &S->laneBytes[k]);
    if (cfg.hbm_budget_bytes == 0) {
        std::size_t freeB = 0, totalB = 0;
        if (cudaSetDevice(cfg.device) != cudaSuccess || cudaMemGetInfo(&freeB, &totalB) != cudaSuccess) {
            S->err = "no usable CUDA device for the server";
            S->stopping = true;
            return S;
        }
        cfg.hbm_budget_bytes = freeB / 2;
    }
    S->cfg = cfg;
    if (cfg.hbm_budget_bytes < S->laneBytes[BSF_REQ_RANGE] + S->laneBytes[BSF_REQ_PREVIEW]) {
        S->err = "hbm_budget_bytes is below one range lane plus one preview lane";
        S->stopping = true;
        return S;
    }
    // One resident lane of each class, then the rest of max_lanes range lanes and
    // preview_lanes preview lanes while they fit the budget, all up front: a lane
    // opened under load (allocations, graph captures) holds up the requests
    // already running for about 100 ms. Lanes evicted later reopen on demand.
    std::vector<int> opening = {BSF_REQ_RANGE, BSF_REQ_PREVIEW};
    for (int t = 1; t < cfg.max_lanes; ++t) opening.push_back(BSF_REQ_RANGE);
    for (int t = 1; t < cfg.preview_lanes; ++t) opening.push_back(BSF_REQ_PREVIEW);
    for (std::size_t i = 0; i < opening.size(); ++i) {
        const int k = opening[i];
        if (i >= 2 && S->bytesInUse + S->laneBytes[k] > cfg.hbm_budget_bytes) continue;
        void* h = bsf_open(&S->laneCfg[k]);
        const char* e = h ? bsf_last_error(h) : "handle allocation failed";
        if (!h || (e && e[0])) {
            S->err = std::string("opening a lane: ") + (e ? e : "");
            if (h) bsf_close(h);
            S->stopping = true;
            return S;
        }
        configure_lane(h, k);
        auto lane = std::make_unique<Lane>();
        lane->kind = k;
        lane->h = h;
        lane->bytes = bsf_handle_footprint(h);
        S->bytesInUse += lane->bytes;
        S->lanes.push_back(std::move(lane));
    }
    S->bytesPeak = S->bytesInUse;
    for (int t = 0; t < cfg.max_lanes; ++t) S->workers.emplace_back(worker_loop, S, BSF_REQ_RANGE);
    for (int t = 0; t < cfg.preview_lanes; ++t) S->workers.emplace_back(worker_loop, S, BSF_REQ_PREVIEW);
    return S;
}

void bsf_server_close(void* sv) {
    Server* S = static_cast<Server*>(sv);
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stopping = true;
    }
    S->cvWork.notify_all();
    for (auto& t : S->workers) t.join();
    for (auto& l : S->lanes)
        if (l->h) bsf_close(l->h);
    delete S;
}

const char* bsf_server_last_error(const void* sv) {
    // Workers rewrite the message under the lock; each caller thread gets its own copy.
    thread_local std::string copy;
    Server* S = const_cast<Server*>(static_cast<const Server*>(sv));
    if (!S) return "null server";
    std::lock_guard<std::mutex> lk(S->mu);
    copy = S->err;
    return copy.c_str();
}

int bsf_server_submit_range(void* sv, const int64_t* seeds, uint32_t count, int32_t radius, int32_t profile,
                            const bsf_match_settings* ms, uint64_t* ticket) {
    Server* S = static_cast<Server*>(sv);
    if (!S || !seeds || count == 0 || !ticket || profile < -1 || profile > 3) return BSF_E_ARG;
    if (radius < 0 || radius > 24) return BSF_E_LIMIT;
    auto r = std::make_unique<Request>();
    r->kind = BSF_REQ_RANGE;
    r->radius = radius;
    r->profile = profile < 0 ? S->cfg.profile : profile;
    if (ms) r->ms = *ms;
    else bsf_default_match_settings(&r->ms);
    r->seeds.assign(seeds, seeds + count);
    r->res.kind = BSF_REQ_RANGE;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->workers.empty()) return BSF_E_STATE;
    r->ticket = S->nextTicket++;
    r->submitted = Clock::now();
    *ticket = r->ticket;
    S->ranges.push_back(r.get());
    S->reqs[r->ticket] = std::move(r);
    ++S->submitted[BSF_REQ_RANGE];
    S->cvWork.notify_all();  // range and preview workers wait on one condition
    return BSF_OK;
}

int bsf_server_submit_preview(void* sv, int64_t seed, int32_t cx, int32_t cz, int32_t radius,
                              const bsf_match_settings* ms, uint64_t* ticket) {
    Server* S = static_cast<Server*>(sv);
    if (!S || !ticket) return BSF_E_ARG;
    if (radius < 0 || radius > S->cfg.max_preview_radius) return BSF_E_LIMIT;
    auto r = std::make_unique<Request>();
    r->kind = BSF_REQ_PREVIEW;
    r->radius = radius;
    if (ms) r->ms = *ms;
    else bsf_default_match_settings(&r->ms);
    r->seed = seed;
    r->cx = cx;
    r->cz = cz;
    r->res.kind = BSF_REQ_PREVIEW;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->workers.empty()) return BSF_E_STATE;
    r->ticket = S->nextTicket++;
    r->submitted = Clock::now();
    *ticket = r->ticket;
    S->previews.push_back(r.get());
    S->reqs[r->ticket] = std::move(r);
    ++S->submitted[BSF_REQ_PREVIEW];
    S->cvWork.notify_all();  // range and preview workers wait on one condition
    return BSF_OK;
}

int bsf_server_poll(void* sv, uint64_t ticket, int32_t waitMs, bsf_server_result* out) {
    Server* S = static_cast<Server*>(sv);
    if (!S || !out) return BSF_E_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    if (!find(S, ticket)) return BSF_E_ARG;
    auto ready = [&] {
        const Request* r = find(S, ticket);
        return !r || r->finished;
    };
    if (waitMs < 0) S->cvDone.wait(lk, ready);
    else if (waitMs > 0) S->cvDone.wait_for(lk, std::chrono::milliseconds(waitMs), ready);
    const Request* r = find(S, ticket);
    if (!r) return BSF_E_ARG;
    if (!r->finished) return BSF_PENDING;
    *out = r->res;
    return BSF_OK;
}

int bsf_server_records(void* sv, uint64_t ticket, bsf_mega_record* out, uint32_t cap, uint32_t* n) {
    Server* S = static_cast<Server*>(sv);
    if (!S || (!out && cap) || !n) return BSF_E_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    const Request* r = find(S, ticket);
    if (!r || !r->finished || r->kind != BSF_REQ_RANGE) return BSF_E_ARG;
    const std::uint32_t k = std::min<std::uint32_t>(cap, static_cast<std::uint32_t>(r->records.size()));
    if (k) std::memcpy(out, r->records.data(), sizeof(bsf_mega_record) * k);
    *n = k;
    return BSF_OK;
}

int bsf_server_preview_columns(void* sv, uint64_t ticket, int32_t* minY, int32_t* maxY, uint32_t cap) {
    Server* S = static_cast<Server*>(sv);
    if (!S || !minY || !maxY) return BSF_E_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    const Request* r = find(S, ticket);
    if (!r || !r->finished || r->kind != BSF_REQ_PREVIEW) return BSF_E_ARG;
    if (cap < r->minY.size()) return BSF_E_LIMIT;
    if (!r->minY.empty()) {
        std::memcpy(minY, r->minY.data(), r->minY.size() * 4);
        std::memcpy(maxY, r->maxY.data(), r->maxY.size() * 4);
    }
    return BSF_OK;
}

int bsf_server_release(void* sv, uint64_t ticket) {
    Server* S = static_cast<Server*>(sv);
    if (!S) return BSF_E_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    const Request* r = find(S, ticket);
    if (!r || !r->finished) return BSF_E_ARG;
    S->reqs.erase(ticket);
    S->cvDone.notify_all();
    return BSF_OK;
}

int bsf_server_get_stats(void* sv, bsf_server_stats* out) {
    Server* S = static_cast<Server*>(sv);
    if (!S || !out) return BSF_E_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    bsf_server_stats st{};
    for (int k = 0; k < 2; ++k) {
        st.submitted[k] = S->submitted[k];
        st.completed[k] = S->completed[k];
        st.failed[k] = S->failed[k];
        percentiles(S->latency[k], st.p50_ms[k], st.p99_ms[k], st.p999_ms[k]);
    }
    st.worlds_completed = S->worldsCompleted;
    st.hbm_bytes_in_use = S->bytesInUse;
    st.hbm_bytes_peak = S->bytesPeak;
    st.hbm_budget = S->cfg.hbm_budget_bytes;
    for (const auto& l : S->lanes) ++st.lanes_open[l->kind];
    st.max_busy_lanes = S->maxBusy;
    st.deferred = S->deferred;
    st.evictions = S->evictions;
    *out = st;
    return BSF_OK;
}

}  // extern "C"
