// Reference GPU arm: the reference worker's own GPU kernels, driven from the host.
//
// TEST AND BENCH INFRASTRUCTURE ONLY (a checker and a baseline): nothing in the
// product links or loads it. tests/ use it to pin the CUDA product path against
// the reference's GPU code, and bench.py times it as the reference GPU bar.
//
// oracle/build_ref.sh compiles the reference's unmodified native/src/
// gpu_p20_benchmark.cpp into a device image (oracle/_ref/ref_worker.cubin) with
// the reference's own nvcc flags (--fmad=false --ftz=false --prec-div=true
// --prec-sqrt=true). The reference's host program cannot run here (its sources
// are C++ for the host architecture of the machine that builds it), so this file
// restates the host side of its `stage0stream` mode (streamStage0Filter,
// native/src/gpu_p20_benchmark.cpp:7310-7613) over the CUDA driver API:
//   - the same device buffers, sized as the reference sizes them (:7342-7366;
//     coarse micro-batch buffers :1131-1151, capacity 1024);
//   - per centre the same launches with the same arguments and launch shapes:
//     p20KernelFromSeeds <<<count, 64>>>, applyP20MinimumGateKernel when the
//     profile's P20 minimum is above 1, stage0UpperCompact192SharedYKernel
//     <<<count, 192>>>, stage0LowerCompactKernel<32> <<<count, 32>>> (:7421-7454);
//   - the host P19 step (:7467-7489), here through the oracle's restatement of
//     buildMonsterFeatures / p19native::score / megaTopologyReject (pinned to the
//     reference's host code by golden vectors);
//   - the coarse micro-batches of runCoarseScoresCachedAt (:1188-1218):
//     generateCoarseSignsDirect23Kernel <<<n, 256>>> and
//     scoreCoarseSignsParallelKernel<64> <<<n, 64>>>;
//   - the record packing of :7504-7554 (the oracle's or_pack_record).
// Kernels are found by name in the loaded image (cuModuleEnumerateFunctions).
#include <cuda.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "bsf_oracle.h"

namespace {

void ck(CUresult r, const char* what) {
    if (r != CUDA_SUCCESS) {
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        throw std::runtime_error(std::string(what) + ": " + (s ? s : "unknown CUDA driver error"));
    }
}

constexpr int kFullPoints = 256;          // stage0gpu::FULL_POINTS
constexpr int kTerrainStates = 66;        // terraincache::STATE_COUNT
constexpr int kClimateStates = 10;        // climatecache::STATE_COUNT
constexpr int kColumns = 61 * 61;         // coarsecore::COLUMNS
constexpr int kCells = kColumns * 17;     // coarsecore::CELLS
constexpr int kCoarseChunk = 1024;        // coarseChunkCapacity (:7368)
const int kCenterX[8] = {0, 15, 0, 15, -15, -15, 0, 15};
const int kCenterZ[8] = {0, 0, 15, 15, 0, 15, -15, -15};

struct RefGpu {
    CUcontext ctx = nullptr;
    CUdevice dev = 0;
    CUmodule mod = nullptr;
    CUfunction fP20 = nullptr, fGate = nullptr, fUpper = nullptr, fLower = nullptr, fCoarse = nullptr,
               fScore = nullptr;
    int capacity = 0;
    std::vector<CUdeviceptr> owned;
    CUdeviceptr seeds = 0, p20 = 0, p20Gate = 0, upper = 0, high = 0, upperMasks = 0, highest = 0;
    CUdeviceptr tPerm = 0, tOff = 0, cPerm = 0, cOff = 0, d5 = 0, d7 = 0;
    // coarse micro-batch buffers (coarsegpu::Buffers)
    CUdeviceptr bSeeds = 0, bIdx = 0, bTemp = 0, bRain = 0, bBlend = 0, bN1 = 0, bN2 = 0, bN3 = 0, bN4 = 0, bN5 = 0,
                bSigns = 0, bLabels = 0, bQueue = 0, bSeen = 0, bMinY = 0, bCompCols = 0, bScores = 0;
    double ms[3] = {0, 0, 0};  // last batch: GPU stage0 wall, host P19, coarse (wall, incl. copies)

    CUdeviceptr alloc(std::size_t bytes) {
        CUdeviceptr p = 0;
        ck(cuMemAlloc(&p, bytes), "cuMemAlloc");
        owned.push_back(p);
        return p;
    }
};

// Finds the one kernel whose mangled name contains `token`.
CUfunction find_kernel(CUmodule mod, const std::vector<CUfunction>& all, const char* token) {
    CUfunction hit = nullptr;
    for (CUfunction f : all) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        if (std::strstr(name, token)) {
            if (hit) throw std::runtime_error(std::string("ambiguous kernel name token ") + token);
            hit = f;
        }
    }
    if (!hit) throw std::runtime_error(std::string("kernel not found in the reference image: ") + token);
    (void)mod;
    return hit;
}

void launch(CUfunction f, unsigned grid, unsigned block, void** args, const char* what) {
    ck(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr), what);
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void copy_err(const std::exception& e, char* err, std::size_t len) {
    if (err && len) {
        std::snprintf(err, len, "%s", e.what());
    }
}

void run_batch(RefGpu* g, const std::int64_t* seedsIn, std::uint32_t count, int centers, int profileId, int research,
               std::uint8_t* out) {
    or_profile prof;
    or_profile_get(profileId, &prof);
    int n = static_cast<int>(count);  // kernel argument (its address is passed)
    const std::size_t rec = research ? 34 : 16;
    ck(cuCtxSetCurrent(g->ctx), "cuCtxSetCurrent");
    ck(cuMemcpyHtoD(g->seeds, seedsIn, static_cast<std::size_t>(n) * 8), "seed upload");
    std::vector<int> p20(n), upper(n), high(n), coarse(n);
    std::vector<std::uint8_t> highest(static_cast<std::size_t>(n) * kFullPoints);
    std::vector<or_region> reg(n);
    std::vector<int> coarseList;
    std::vector<std::int64_t> cSeeds(kCoarseChunk);
    std::vector<int> cIdx(kCoarseChunk), cScores(kCoarseChunk);
    g->ms[0] = g->ms[1] = g->ms[2] = 0;
    for (int c = 0; c < centers; ++c) {
        double t0 = now_ms();
        int offX = kCenterX[c] * 4, offZ = kCenterZ[c] * 4;
        int reload = c != 0 ? 1 : 0;
        ck(cuMemsetD8(g->high, 0, static_cast<std::size_t>(n) * 4), "memset high");
        {
            CUdeviceptr nul = 0;
            void* a[] = {&g->seeds, &n, &g->p20, &nul, &g->tPerm, &g->tOff, &g->cPerm, &g->cOff, &g->upperMasks,
                         &g->d5, &g->d7, &offX, &offZ, &reload, &reload};
            launch(g->fP20, count, 64, a, "p20KernelFromSeeds");
        }
        CUdeviceptr later = g->p20;
        int p20Min = prof.p20MinCount;
        if (p20Min > 1) {
            void* a[] = {&g->p20, &g->p20Gate, &n, &p20Min};
            launch(g->fGate, (count + 255) / 256, 256, a, "applyP20MinimumGateKernel");
            later = g->p20Gate;
        }
        {
            CUdeviceptr nul = 0;
            void* a[] = {&g->seeds, &n, &later, &g->upper, &g->upperMasks, &nul, &g->tPerm, &g->tOff, &g->cPerm,
                         &g->cOff, &g->d5, &g->d7, &offX, &offZ};
            launch(g->fUpper, count, 192, a, "stage0UpperCompact192SharedYKernel");
        }
        {
            CUdeviceptr nul = 0;
            int upperMin = prof.upperMinCount;
            void* a[] = {&g->seeds, &n, &later, &g->upper, &upperMin, &g->upperMasks, &g->high, &g->highest,
                         &nul, &g->tPerm, &g->tOff, &g->d5, &g->d7, &offX, &offZ, &nul};
            launch(g->fLower, count, 32, a, "stage0LowerCompactKernel<32>");
        }
        ck(cuMemcpyDtoH(p20.data(), g->p20, static_cast<std::size_t>(n) * 4), "p20 download");
        ck(cuMemcpyDtoH(upper.data(), g->upper, static_cast<std::size_t>(n) * 4), "upper download");
        ck(cuMemcpyDtoH(high.data(), g->high, static_cast<std::size_t>(n) * 4), "high download");
        ck(cuMemcpyDtoH(highest.data(), g->highest, highest.size()), "highest download");
        double t1 = now_ms();
        g->ms[0] += t1 - t0;

        coarseList.clear();
        for (int i = 0; i < n; ++i) {
            or_region& r = reg[i];
            std::memset(&r, 0, sizeof(r));
            r.p20 = p20[i];
            r.upper = upper[i];
            r.high = high[i];
            r.p19Score = std::numeric_limits<double>::quiet_NaN();
            if (!(p20[i] >= prof.p20MinCount && upper[i] >= prof.upperMinCount && high[i] >= prof.highMinCount))
                continue;
            or_monster_features(highest.data() + static_cast<std::size_t>(i) * kFullPoints, &r.f);
            r.p19Evaluated = 1;
            r.p19Score = or_p19_score(upper[i], &r.f);
            r.p19Extreme = or_p19_extreme(&r.f);
            r.p19Pass = (r.p19Extreme || r.p19Score >= prof.p19MinScore) ? 1 : 0;
            r.megaReject = (r.p19Pass && prof.megaTopologyFilter &&
                            or_mega_topology_reject(r.p19Score, r.p19Extreme, &r.f)) ? 1 : 0;
            if (r.p19Pass && !r.megaReject) coarseList.push_back(i);
        }
        double t2 = now_ms();
        g->ms[1] += t2 - t1;

        for (std::size_t off = 0; off < coarseList.size(); off += kCoarseChunk) {
            int chunk = static_cast<int>(std::min<std::size_t>(kCoarseChunk, coarseList.size() - off));
            for (int j = 0; j < chunk; ++j) {
                cSeeds[j] = seedsIn[coarseList[off + j]];
                cIdx[j] = coarseList[off + j];
            }
            ck(cuMemcpyHtoD(g->bSeeds, cSeeds.data(), static_cast<std::size_t>(chunk) * 8), "coarse seeds");
            ck(cuMemcpyHtoD(g->bIdx, cIdx.data(), static_cast<std::size_t>(chunk) * 4), "coarse indices");
            {
                void* a[] = {&g->bSeeds, &chunk, &g->bTemp, &g->bRain, &g->bBlend, &g->bN1, &g->bN2, &g->bN3,
                             &g->bN4, &g->bN5, &g->bSigns, &offX, &offZ, &g->bIdx, &g->tPerm, &g->tOff, &g->cPerm,
                             &g->cOff};
                launch(g->fCoarse, static_cast<unsigned>(chunk), 256, a, "generateCoarseSignsDirect23Kernel");
            }
            {
                void* a[] = {&g->bSigns, &chunk, &g->bLabels, &g->bQueue, &g->bSeen, &g->bMinY, &g->bCompCols,
                             &g->bScores};
                launch(g->fScore, static_cast<unsigned>(chunk), 64, a, "scoreCoarseSignsParallelKernel<64>");
            }
            ck(cuMemcpyDtoH(cScores.data(), g->bScores, static_cast<std::size_t>(chunk) * 4), "coarse scores");
            for (int j = 0; j < chunk; ++j) {
                or_region& r = reg[coarseList[off + j]];
                r.coarse = cScores[j];
                r.coarseEvaluated = 1;
            }
        }
        g->ms[2] += now_ms() - t2;
        for (int i = 0; i < n; ++i)
            or_pack_record(&reg[i], research, out + (static_cast<std::size_t>(i) * centers + c) * rec);
    }
}

}  // namespace

extern "C" {

// Loads the reference image and allocates the buffers of a stage0stream worker
// of `capacity` worlds on `device` (its primary context). NULL on failure (err).
void* rg_open(const char* cubinPath, int device, int capacity, char* err, std::size_t errLen) {
    RefGpu* g = new RefGpu();
    try {
        if (capacity < 1) throw std::invalid_argument("capacity must be >= 1");
        ck(cuInit(0), "cuInit");
        ck(cuDeviceGet(&g->dev, device), "cuDeviceGet");
        ck(cuDevicePrimaryCtxRetain(&g->ctx, g->dev), "cuDevicePrimaryCtxRetain");
        ck(cuCtxSetCurrent(g->ctx), "cuCtxSetCurrent");
        ck(cuModuleLoad(&g->mod, cubinPath), "cuModuleLoad (reference image)");
        unsigned nf = 0;
        ck(cuModuleGetFunctionCount(&nf, g->mod), "cuModuleGetFunctionCount");
        std::vector<CUfunction> all(nf);
        ck(cuModuleEnumerateFunctions(all.data(), nf, g->mod), "cuModuleEnumerateFunctions");
        g->fP20 = find_kernel(g->mod, all, "6p20gpu18p20KernelFromSeedsE");
        g->fGate = find_kernel(g->mod, all, "25applyP20MinimumGateKernelE");
        g->fUpper = find_kernel(g->mod, all, "4p33y34stage0UpperCompact192SharedYKernelE");
        g->fLower = find_kernel(g->mod, all, "8p30lower24stage0LowerCompactKernelILi32EE");
        g->fCoarse = find_kernel(g->mod, all, "9p35coarse33generateCoarseSignsDirect23KernelE");
        g->fScore = find_kernel(g->mod, all, "8p36score30scoreCoarseSignsParallelKernelILi64EE");
        g->capacity = capacity;
        const std::size_t n = static_cast<std::size_t>(capacity);
        g->seeds = g->alloc(n * 8);
        g->p20 = g->alloc(n * 4);
        g->p20Gate = g->alloc(n * 4);
        g->upper = g->alloc(n * 4);
        g->high = g->alloc(n * 4);
        g->upperMasks = g->alloc(n * kFullPoints);
        g->highest = g->alloc(n * kFullPoints);
        g->tPerm = g->alloc(n * kTerrainStates * 256);
        g->tOff = g->alloc(n * kTerrainStates * 3 * 8);
        g->cPerm = g->alloc(n * kClimateStates * 256);
        g->cOff = g->alloc(n * kClimateStates * 3 * 8);
        g->d5 = g->alloc(n * kFullPoints * 8);
        g->d7 = g->alloc(n * kFullPoints * 8);
        const std::size_t cc = kCoarseChunk, cols = cc * kColumns, cells = cc * kCells;
        g->bSeeds = g->alloc(cc * 8);
        g->bIdx = g->alloc(cc * 4);
        g->bTemp = g->alloc(cols * 8);
        g->bRain = g->alloc(cols * 8);
        g->bBlend = g->alloc(cols * 8);
        g->bN1 = g->alloc(cells * 8);
        g->bN2 = g->alloc(cells * 8);
        g->bN3 = g->alloc(cells * 8);
        g->bN4 = g->alloc(cols * 8);
        g->bN5 = g->alloc(cols * 8);
        g->bSigns = g->alloc(cells);
        g->bLabels = g->alloc(cells * 4);
        g->bQueue = g->alloc(cells * 4);
        g->bSeen = g->alloc(cols * 4);
        g->bMinY = g->alloc(cols * 4);
        g->bCompCols = g->alloc(cols * 4);
        g->bScores = g->alloc(cc * 4);
        return g;
    } catch (const std::exception& e) {
        copy_err(e, err, errLen);
        for (CUdeviceptr p : g->owned) cuMemFree(p);
        if (g->mod) cuModuleUnload(g->mod);
        if (g->ctx) cuDevicePrimaryCtxRelease(g->dev);
        delete g;
        return nullptr;
    }
}

// One stage0stream batch: count worlds x centers records (16 lean / 34 research
// bytes, world-major, centre-minor) into out. 0 on success, -1 on failure (err).
int rg_stage0_batch(void* hv, const std::int64_t* seeds, std::uint32_t count, int centers, int profile,
                    int research, std::uint8_t* out, char* err, std::size_t errLen) {
    RefGpu* g = static_cast<RefGpu*>(hv);
    try {
        if (!g || !seeds || !out || count == 0 || static_cast<int>(count) > g->capacity)
            throw std::invalid_argument("bad handle, buffers or count (1..capacity)");
        if (centers != 1 && centers != 8) throw std::invalid_argument("centers must be 1 or 8");
        if (profile < 0 || profile > 3) throw std::invalid_argument("profile must be 0..3");
        run_batch(g, seeds, count, centers, profile, research, out);
        return 0;
    } catch (const std::exception& e) {
        copy_err(e, err, errLen);
        return -1;
    }
}

// Wall milliseconds of the last batch: [0] Stage0 kernels + downloads,
// [1] host P19, [2] coarse micro-batches (uploads, kernels, downloads).
void rg_last_ms(const void* hv, double* ms3) {
    const RefGpu* g = static_cast<const RefGpu*>(hv);
    for (int i = 0; i < 3; ++i) ms3[i] = g ? g->ms[i] : 0.0;
}

void rg_close(void* hv) {
    RefGpu* g = static_cast<RefGpu*>(hv);
    if (!g) return;
    cuCtxSetCurrent(g->ctx);
    cuCtxSynchronize();
    for (CUdeviceptr p : g->owned) cuMemFree(p);
    if (g->mod) cuModuleUnload(g->mod);
    cuDevicePrimaryCtxRelease(g->dev);
    delete g;
}

}  // extern "C"
