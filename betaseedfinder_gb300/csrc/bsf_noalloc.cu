// Allocation-free chunk-terrain entry point.
//
// Some callers cannot call cudaMalloc: a host that owns every byte of device
// memory and hands the library only pre-allocated buffers (a JVM or game
// runtime with its own pool), a serving loop where an allocation would
// synchronise the device and stall other work in flight, or a process held to
// a device-memory budget that must not grow after start-up. For them
// bsf_chunk_bitmaps_noalloc runs the same kernels as bsf_chunk_bitmaps on
// caller-provided device buffers; its only scratch (the generator-state cache
// between the setup and terrain kernels, plus one counter) lives in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits.
#include "../../include/bsf.h"
#include "bsf_device.cuh"
#include "bsf_internal.h"

#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>

namespace {

constexpr std::uint32_t kMaxWorlds = BSF_NOALLOC_MAX_WORLDS;
constexpr std::size_t kPermBytes = static_cast<std::size_t>(kMaxWorlds) * bsf::WORLD_PERM_BYTES;
constexpr std::size_t kOffsetBytes = static_cast<std::size_t>(kMaxWorlds) * bsf::WORLD_OFFSETS * sizeof(double);
constexpr std::size_t kScratchBytes = kPermBytes + kOffsetBytes + 256;  // + the setup fallback counter

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch[kMaxDevices] = {};

void write_error(char* err, std::size_t errLen, const char* msg) {
    if (err && errLen) {
        std::strncpy(err, msg, errLen - 1);
        err[errLen - 1] = '\0';
    }
}

// Once per device, with that device current: constant tables and the device
// address of the scratch array (the host-side name is only a stand-in).
unsigned char* scratch_for_current_device(char* err, std::size_t errLen) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        write_error(err, errLen, "bsf_chunk_bitmaps_noalloc: no usable current CUDA device");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch[dev]) {
        try {
            bsf::init_lcg_tables();
        } catch (const std::exception& e) {
            write_error(err, errLen, e.what());
            return nullptr;
        }
        void* ptr = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (rc != cudaSuccess || !ptr) {
            char buf[200];
            std::snprintf(buf, sizeof(buf), "bsf_chunk_bitmaps_noalloc: cudaGetSymbolAddress failed: %s",
                          cudaGetErrorString(rc));
            write_error(err, errLen, buf);
            return nullptr;
        }
        g_scratch[dev] = static_cast<unsigned char*>(ptr);
    }
    return g_scratch[dev];
}

}  // namespace

extern "C" int bsf_chunk_bitmaps_noalloc(const int64_t* d_seeds, uint32_t count, int32_t chunk_x, int32_t chunk_z,
                                         uint8_t* d_bitmaps, uint64_t* d_hashes, void* stream, char* err,
                                         size_t err_len) {
    if (!d_seeds || !d_bitmaps || !d_hashes || count == 0) {
        write_error(err, err_len, "bsf_chunk_bitmaps_noalloc: null buffer or zero count");
        return BSF_E_ARG;
    }
    if (count > kMaxWorlds) {
        char buf[160];
        std::snprintf(buf, sizeof(buf), "bsf_chunk_bitmaps_noalloc: count %u exceeds the fixed scratch of %u worlds",
                      count, kMaxWorlds);
        write_error(err, err_len, buf);
        return BSF_E_LIMIT;
    }
    if (chunk_x < -(1 << 20) || chunk_x > (1 << 20) || chunk_z < -(1 << 20) || chunk_z > (1 << 20)) {
        write_error(err, err_len, "bsf_chunk_bitmaps_noalloc: chunk coordinate out of range");
        return BSF_E_ARG;
    }
    unsigned char* base = scratch_for_current_device(err, err_len);
    if (!base) return BSF_E_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bsf::StateCache cache;
    cache.perms = base;
    cache.offsets = reinterpret_cast<double*>(base + kPermBytes);
    cache.capacity = static_cast<int>(kMaxWorlds);
    int* fallbackCounter = reinterpret_cast<int*>(base + kPermBytes + kOffsetBytes);
    try {
        // The array keeps the previous call's contents: the counter must start at zero;
        // the state cache is fully rewritten for the `count` worlds used.
        if (cudaMemsetAsync(fallbackCounter, 0, sizeof(int), s) != cudaSuccess)
            throw std::runtime_error("bsf_chunk_bitmaps_noalloc: counter reset failed");
        bsf::launch_world_init(d_seeds, static_cast<int>(count), cache, fallbackCounter, s);
        bsf::launch_chunk_bitmaps(cache, static_cast<int>(count), chunk_x, chunk_z, d_bitmaps, d_hashes, s);
    } catch (const std::exception& e) {
        write_error(err, err_len, e.what());
        return BSF_E_CUDA;
    }
    write_error(err, err_len, "");
    return BSF_OK;
}
