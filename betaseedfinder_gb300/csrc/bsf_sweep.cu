// Stage0 scout sweep: consecutive world seeds through the Stage0 gate, with the
// surviving seeds compacted on the device in seed order.
//
// One sweep batch is five small kernels around the screened Stage0 kernel:
//   k_sweep_seeds    seeds[i] = next + i, from a device-side cursor (so a graph of
//                    the batch replays without host arguments);
//   k_sweep_count    per block of 1024 worlds: survivors and the stage passes;
//   k_sweep_write    each block writes its survivors at (list total + the sum of
//                    the earlier blocks' counts + its ballot prefix), so the list
//                    is in world (= seed) order without a sort;
//   k_sweep_advance  list total += batch survivors; cursor += batch size.
// A world survives when one of its regions passes the profile's P20, Upper and
// high gates: the regions the app hands to P19, i.e. rejectStage 0 or >= 5
// (IslandSearchEngine.java:1368-1372).
#include "bsf_internal.h"

#include <cstdio>
#include <stdexcept>

namespace bsf {
namespace {

constexpr int SWEEP_BLOCK = 1024;

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

__global__ void k_sweep_seeds(std::int64_t* __restrict__ seeds, int n, const unsigned long long* next) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) seeds[i] = static_cast<std::int64_t>(*next + static_cast<unsigned long long>(i));
}

__device__ __forceinline__ bool region_gates(const RegionInfo& r, const Profile& prof, bool& p20, bool& up) {
    p20 = r.p20 >= prof.p20MinCount;
    up = p20 && r.upper >= prof.upperMinCount;
    return up && r.high >= prof.highMinCount;
}

__device__ __forceinline__ bool world_survives(const RegionInfo* regions, int world, int centers, const Profile& prof,
                                               int& p20s, int& ups, int& his) {
    bool any = false;
    for (int c = 0; c < centers; ++c) {
        bool p20, up;
        const bool hi = region_gates(regions[static_cast<std::size_t>(world) * centers + c], prof, p20, up);
        p20s += p20;
        ups += up;
        his += hi;
        any |= hi;
    }
    return any;
}

// stage[0..2]: regions passing P20, P20+Upper, P20+Upper+high; stage[3]: surviving worlds.
__global__ void __launch_bounds__(SWEEP_BLOCK) k_sweep_count(const RegionInfo* __restrict__ regions, int n,
                                                             int centers, Profile prof, int* __restrict__ blockCounts,
                                                             unsigned long long* __restrict__ stage) {
    const int world = blockIdx.x * SWEEP_BLOCK + threadIdx.x;
    int p20s = 0, ups = 0, his = 0;
    const bool surv = world < n && world_survives(regions, world, centers, prof, p20s, ups, his);
    const int blockSurv = __syncthreads_count(surv);
    if (threadIdx.x == 0) blockCounts[blockIdx.x] = blockSurv;
    for (int off = 16; off > 0; off >>= 1) {
        p20s += __shfl_xor_sync(0xffffffffu, p20s, off);
        ups += __shfl_xor_sync(0xffffffffu, ups, off);
        his += __shfl_xor_sync(0xffffffffu, his, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (p20s) atomicAdd(&stage[0], static_cast<unsigned long long>(p20s));
        if (ups) atomicAdd(&stage[1], static_cast<unsigned long long>(ups));
        if (his) atomicAdd(&stage[2], static_cast<unsigned long long>(his));
    }
    if (threadIdx.x == 0 && blockSurv) atomicAdd(&stage[3], static_cast<unsigned long long>(blockSurv));
}

__global__ void __launch_bounds__(SWEEP_BLOCK) k_sweep_write(const RegionInfo* __restrict__ regions,
                                                             const std::int64_t* __restrict__ seeds, int n,
                                                             int centers, Profile prof,
                                                             const int* __restrict__ blockCounts,
                                                             const unsigned long long* total,
                                                             std::int64_t* __restrict__ out,
                                                             unsigned long long outCap) {
    __shared__ int warpCount[SWEEP_BLOCK / 32];
    __shared__ int blockBase;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (warp == 0) {  // the earlier blocks' survivors (a batch has at most a few hundred blocks)
        int s = 0;
        for (int b = lane; b < static_cast<int>(blockIdx.x); b += 32) s += blockCounts[b];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) blockBase = s;
    }
    const int world = blockIdx.x * SWEEP_BLOCK + tid;
    int p20s = 0, ups = 0, his = 0;
    const bool surv = world < n && world_survives(regions, world, centers, prof, p20s, ups, his);
    const unsigned vote = __ballot_sync(0xffffffffu, surv);
    if (lane == 0) warpCount[warp] = __popc(vote);
    __syncthreads();
    if (!surv) return;
    int before = blockBase;
    for (int w = 0; w < warp; ++w) before += warpCount[w];
    before += __popc(vote & ((1u << lane) - 1u));
    const unsigned long long pos = *total + static_cast<unsigned long long>(before);
    if (pos < outCap) out[pos] = seeds[world];
}

__global__ void k_sweep_advance(const int* __restrict__ blockCounts, int blocks, unsigned long long* total,
                                unsigned long long* next, int n) {
    int s = 0;
    for (int b = threadIdx.x; b < blocks; b += 32) s += blockCounts[b];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (threadIdx.x == 0) {
        *total += static_cast<unsigned long long>(s);
        *next += static_cast<unsigned long long>(n);
    }
}

}  // namespace

int sweep_blocks(int n) { return (n + SWEEP_BLOCK - 1) / SWEEP_BLOCK; }

void launch_sweep_seeds(std::int64_t* dSeeds, int n, const SweepState& st, cudaStream_t stream) {
    k_sweep_seeds<<<(n + 255) / 256, 256, 0, stream>>>(dSeeds, n, st.next);
    check(cudaGetLastError(), "k_sweep_seeds");
}

void launch_sweep_compact(const RegionInfo* dRegions, const std::int64_t* dSeeds, int n, int centers,
                          const Profile& prof, const SweepState& st, cudaStream_t stream) {
    const int blocks = sweep_blocks(n);
    k_sweep_count<<<blocks, SWEEP_BLOCK, 0, stream>>>(dRegions, n, centers, prof, st.blockCounts, st.stage);
    check(cudaGetLastError(), "k_sweep_count");
    k_sweep_write<<<blocks, SWEEP_BLOCK, 0, stream>>>(dRegions, dSeeds, n, centers, prof, st.blockCounts, st.total,
                                                     st.out, st.outCap);
    check(cudaGetLastError(), "k_sweep_write");
    k_sweep_advance<<<1, 32, 0, stream>>>(st.blockCounts, blocks, st.total, st.next, n);
    check(cudaGetLastError(), "k_sweep_advance");
}

}  // namespace bsf
