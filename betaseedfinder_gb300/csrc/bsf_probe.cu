// Screen-bound probe (instrumentation): every FP32 screening primitive of
// bsf_screen.cuh evaluated beside its exact FP64 twin of bsf_device.cuh on real
// generator states at random lattice points, reporting the largest observed
// |FP32 - FP64| as a fraction of the bound the screen relies on. A screened
// sign is only sound while that fraction stays below 1; tests require a margin.
#include "../../include/bsf.h"
#include "bsf_device.cuh"
#include "bsf_internal.h"
#include "bsf_screen.cuh"

#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

namespace bsf {
namespace {

using namespace screen;

constexpr int KINDS = BSF_PROBE_KINDS;

__device__ __forceinline__ std::uint64_t mix64(std::uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Rng {
    std::uint64_t s;
    __device__ std::uint64_t next() {
        s += 0x9E3779B97F4A7C15ULL;
        return mix64(s);
    }
    __device__ int range(int lo, int hi) {  // [lo, hi]
        return lo + static_cast<int>(next() % static_cast<std::uint64_t>(hi - lo + 1));
    }
};

__device__ __forceinline__ void record(float* maxRatio, unsigned long long* counts, int kind, float ratio) {
    // non-negative floats order like their bit patterns
    atomicMax(reinterpret_cast<int*>(&maxRatio[kind]), __float_as_int(ratio));
    atomicAdd(&counts[kind], 1ULL);
}

__device__ __forceinline__ double lattice_scale(int st) {
    if (st < 16) return NOISE_XZ * exp2_neg(st);
    if (st < 32) return NOISE_XZ * exp2_neg(st - 16);
    if (st < 40) return (NOISE_XZ / 80.0) * exp2_neg(st - 32);
    if (st < 50) return 1.121 * exp2_neg(st - 40);
    return 200.0 * exp2_neg(st - 50);
}

// Index guard: a world or state index outside the staged cache records a code
// in err and the sample is skipped (the indices come from bounded draws).
__device__ __forceinline__ bool bad_index(const StateCache& c, int w, int st, int* err) {
    if (w >= 0 && w < c.capacity && st >= 0 && st < ST_COUNT) return false;
    atomicExch(err, 1000000 + w * 100 + st);
    return true;
}

__device__ __forceinline__ Gen gen_of(const StateCache& c, int w, int st) {
    Gen g;
    g.p = c.perms + (static_cast<std::size_t>(w) * ST_COUNT + st) * PERM_BYTES;
    const double* o = c.offsets + (static_cast<std::size_t>(w) * ST_COUNT + st) * 4;
    g.a = o[0];
    g.b = o[1];
    g.c = o[2];
    return g;
}

// Axis entry of lattice coordinate k: the FP64 builder, or the double-float one
// (which falls back to FP64 near an integer, as the kernels do).
__device__ __forceinline__ AxisF axis_entry(int k, int st, double off, bool df) {
    AxisF a;
    if (df) {
        const double sc = lattice_scale(st);
        if (make_axis_df(k, df_of(sc), df_of(off), a)) return a;
    }
    return make_axis(static_cast<double>(k) * lattice_scale(st), off);
}

// Kind 0/1: one 3D octave (17 levels, weight 1) against E_OCT3 (FP64 / double-float axes).
__device__ void probe_octave3(const StateCache& c, int w, Rng& r, bool df, float* mr, unsigned long long* cnt,
                              int* err) {
    const int st = r.range(0, OCT3 - 1);
    if (bad_index(c, w, st, err)) return;
    const int span = df ? 92 : 4096;  // double-float axes serve Stage0's coordinates -88..92
    const int kx = r.range(-span, span), kz = r.range(-span, span);
    const Gen g = gen_of(c, w, st);
    const int k = st < 16 ? st : (st < 32 ? st - 16 : st - 32);
    const double sy = st < 32 ? NOISE_Y * exp2_neg(k) : (NOISE_Y / 160.0) * exp2_neg(k);
    YEntry ya[17];
    build_yaxis(sy, g.b, ya);
    YF yf[17];
    build_yf(ya, yf);
    double v64[17];
    octave3_column<0, 17>(g, static_cast<double>(kx) * lattice_scale(st), static_cast<double>(kz) * lattice_scale(st),
                          ya, 1.0, v64, true);
    float v32[17];
    octave3f<0, 17>(g.p, axis_entry(kx, st, g.a, df), axis_entry(kz, st, g.c, df), yf, 1.0f, v32, true);
    float worst = 0.0f;
    for (int y = 0; y < 17; ++y) worst = fmaxf(worst, static_cast<float>(fabs(static_cast<double>(v32[y]) - v64[y])));
    record(mr, cnt, df ? 1 : 0, worst / E_OCT3);
}

// Kind 2/3: one 2D octave against E_OCT2.
__device__ void probe_octave2(const StateCache& c, int w, Rng& r, bool df, float* mr, unsigned long long* cnt,
                              int* err) {
    const int st = r.range(ST_N4, ST_TEMP - 1);
    if (bad_index(c, w, st, err)) return;
    const int span = df ? 92 : 4096;
    const int kx = r.range(-span, span), kz = r.range(-span, span);
    const Gen g = gen_of(c, w, st);
    const double v64 = octave2(g, static_cast<double>(kx) * lattice_scale(st), static_cast<double>(kz) * lattice_scale(st));
    const float v32 = octave2f(g.p, axis_entry(kx, st, g.a, df), axis_entry(kz, st, g.c, df));
    record(mr, cnt, df ? 3 : 2, static_cast<float>(fabs(static_cast<double>(v32) - v64)) / E_OCT2);
}

// The climate octaves' FP64 scale (WorldChunkManager173.java:95-126 constants).
__device__ __forceinline__ double climate_sx(int i) {
    const int grp = i < 4 ? 0 : (i < 8 ? 1 : 2), o = i < 4 ? i : (i < 8 ? i - 4 : i - 8);
    const double scale[3] = {0.02500000037252903, 0.05000000074505806, 0.25};
    const double octScale[3] = {0.25, 0.3333333333333333, 0.5882352941176471};
    double d7 = 1.0;
    for (int k = 0; k < o; ++k) d7 *= octScale[grp];
    return scale[grp] / 1.5 * d7;
}

// Kind 4/5: one simplex sample against its own returned bound (double-float / FP64 geometry).
__device__ void probe_simplex(const StateCache& c, int w, Rng& r, float* mr, unsigned long long* cnt, int* err) {
    const int i = r.range(0, 9);
    if (bad_index(c, w, ST_TEMP + i, err)) return;
    const int bx = 4 * r.range(-100, 100) + 2, bz = 4 * r.range(-100, 100) + 2;
    const Gen g = gen_of(c, w, ST_TEMP + i);
    const double sx = climate_sx(i);
    const double X = static_cast<double>(bx), Z = static_cast<double>(bz);
    const double v64 = simplex2(g, X * sx, Z * sx);
    const double gab[3] = {g.a, g.b, g.c};
    Fe f;
    if (simplex2f_df(g, climate_split(gab), bx, bz, sx, f))
        record(mr, cnt, 4, static_cast<float>(fabs(static_cast<double>(f.v) - v64)) / fmaxf(f.e, 1e-30f));
    const Fe h = simplex2f(g, X * sx, Z * sx);
    record(mr, cnt, 5, static_cast<float>(fabs(static_cast<double>(h.v) - v64)) / fmaxf(h.e, 1e-30f));
}

// GenTable reads offsets as [idx][3]; the cache stores [idx][4].
__global__ void k_repack_offsets(StateCache c, int worlds, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= worlds * ST_COUNT) return;
    for (int j = 0; j < 3; ++j) out[i * 3 + j] = c.offsets[i * 4 + j];
}

// Kind 6: temperature and rain; kind 7: column shape d5 and d7, against their bounds.
__device__ void probe_climate_shape(const StateCache& c, const double* offs3, int w, Rng& r, float* mr,
                                    unsigned long long* cnt) {
    const int cx = r.range(-100, 100), cz = r.range(-100, 100);
    const int bx = cx * 4 + 2, bz = cz * 4 + 2;
    GenTable t;
    t.perm = c.perms + static_cast<std::size_t>(w) * ST_COUNT * PERM_BYTES;
    t.off = offs3 + static_cast<std::size_t>(w) * ST_COUNT * 3;
    float4 clim[10];
    for (int i = 0; i < 10; ++i) clim[i] = climate_split(t.off + (ST_TEMP + i) * 3);
    double temp64, rain64;
    climate_at(t, bx, bz, temp64, rain64);
    Fe temp, rain;
    climate_f(t, clim, bx, bz, temp, rain);
    record(mr, cnt, 6, fmaxf(static_cast<float>(fabs(static_cast<double>(temp.v) - temp64)) / fmaxf(temp.e, 1e-30f),
                             static_cast<float>(fabs(static_cast<double>(rain.v) - rain64)) / fmaxf(rain.e, 1e-30f)));
    // noise4 / noise5 sums in both forms, then the shape
    double n4 = 0.0, n5 = 0.0;
    float f4 = 0.0f, f5 = 0.0f;
    for (int k = 0; k < 26; ++k) {
        const int st = ST_N4 + k, oct = k < 10 ? k : k - 10;
        const Gen g = gen_of(c, w, st);
        const double s = lattice_scale(st);
        const double v = octave2(g, static_cast<double>(cx) * s, static_cast<double>(cz) * s) *
                         static_cast<double>(1 << oct);
        const float vf = octave2f(g.p, make_axis(static_cast<double>(cx) * s, g.a),
                                  make_axis(static_cast<double>(cz) * s, g.c)) * static_cast<float>(1 << oct);
        if (k < 10) { n4 = n4 + v; f4 = f4 + vf; }
        else { n5 = n5 + v; f5 = f5 + vf; }
    }
    double d5, d7;
    column_shape(temp64, rain64, n4, n5, d5, d7);
    Fe fd5, fd7;
    if (column_shape_f(temp, rain, Fe{f4, E_N4}, Fe{f5, E_N5}, fd5, fd7))
        record(mr, cnt, 7, fmaxf(static_cast<float>(fabs(static_cast<double>(fd5.v) - d5)) / fmaxf(fd5.e, 1e-30f),
                                 static_cast<float>(fabs(static_cast<double>(fd7.v) - d7)) / fmaxf(fd7.e, 1e-30f)));
}

// One kernel per probe kind (kind 0..3 by `kind`, 4 the simplex pair, 6 climate and shape).
__global__ void k_screen_probe(StateCache cache, const double* offs3, int worlds, int samples, std::uint64_t seed,
                               int kind, float* maxRatio, unsigned long long* counts, int* err) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    Rng r{mix64(seed ^ (0x632BE59BD9B4E019ULL * static_cast<std::uint64_t>(tid + 1) + kind))};
    for (int i = 0; i < samples; ++i) {
        const int w = r.range(0, worlds - 1);
        if (bad_index(cache, w, 0, err)) return;
        switch (kind) {
            case 0: probe_octave3(cache, w, r, false, maxRatio, counts, err); break;
            case 1: probe_octave3(cache, w, r, true, maxRatio, counts, err); break;
            case 2: probe_octave2(cache, w, r, false, maxRatio, counts, err); break;
            case 3: probe_octave2(cache, w, r, true, maxRatio, counts, err); break;
            case 4: probe_simplex(cache, w, r, maxRatio, counts, err); break;
            default: probe_climate_shape(cache, offs3, w, r, maxRatio, counts); break;
        }
    }
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        throw std::runtime_error(buf);
    }
}

}  // namespace
}  // namespace bsf

extern "C" int bsf_screen_probe(const int64_t* seeds, uint32_t worlds, uint32_t samples_per_thread, uint64_t rng,
                                double* max_ratio, uint64_t* counts, char* err, size_t err_len) {
    using namespace bsf;
    if (!seeds || worlds == 0 || worlds > 4096 || samples_per_thread == 0 || !max_ratio || !counts) return BSF_E_ARG;
    void* base = nullptr;
    int status = BSF_OK;
    try {
        init_lcg_tables();
        const std::size_t n = worlds;
        auto up = [](std::size_t v) { return (v + 255) & ~static_cast<std::size_t>(255); };
        const std::size_t oSeeds = 0, oOff = up(n * 8), oPerm = oOff + up(n * WORLD_OFFSETS * 8),
                          oOff3 = oPerm + up(n * WORLD_PERM_BYTES), oStat = oOff3 + up(n * ST_COUNT * 3 * 8),
                          bytes = oStat + 1024;
        check(cudaMalloc(&base, bytes), "probe buffers");
        unsigned char* b = static_cast<unsigned char*>(base);
        std::int64_t* dSeeds = reinterpret_cast<std::int64_t*>(b + oSeeds);
        StateCache cache;
        cache.offsets = reinterpret_cast<double*>(b + oOff);
        cache.perms = b + oPerm;
        cache.capacity = static_cast<int>(n);
        double* offs3 = reinterpret_cast<double*>(b + oOff3);
        int* fallbacks = reinterpret_cast<int*>(b + oStat);
        float* dRatio = reinterpret_cast<float*>(b + oStat + 256);
        unsigned long long* dCounts = reinterpret_cast<unsigned long long*>(b + oStat + 512);
        check(cudaMemcpy(dSeeds, seeds, n * 8, cudaMemcpyHostToDevice), "probe seeds");
        check(cudaMemset(b + oStat, 0, 1024), "memset");
        launch_world_init(dSeeds, static_cast<int>(n), cache, fallbacks, nullptr);
        k_repack_offsets<<<static_cast<unsigned>((n * ST_COUNT + 255) / 256), 256>>>(cache, static_cast<int>(n), offs3);
        check(cudaGetLastError(), "k_repack_offsets");
        int* dErr = fallbacks + 8;
        check(cudaDeviceSynchronize(), "probe set-up");
        const int kinds[6] = {0, 1, 2, 3, 4, 6};
        for (int kind : kinds) {
            k_screen_probe<<<152 * 4, 128>>>(cache, offs3, static_cast<int>(n), static_cast<int>(samples_per_thread),
                                             rng, kind, dRatio, dCounts, dErr);
            check(cudaGetLastError(), "k_screen_probe launch");
            const std::string what = "k_screen_probe kind " + std::to_string(kind);
            check(cudaDeviceSynchronize(), what.c_str());
        }
        int hErr = 0;
        check(cudaMemcpy(&hErr, dErr, sizeof(int), cudaMemcpyDeviceToHost), "probe error flag");
        if (hErr) throw std::runtime_error("probe index guard " + std::to_string(hErr));
        float hr[KINDS];
        unsigned long long hc[KINDS];
        check(cudaMemcpy(hr, dRatio, sizeof(hr), cudaMemcpyDeviceToHost), "probe ratios");
        check(cudaMemcpy(hc, dCounts, sizeof(hc), cudaMemcpyDeviceToHost), "probe counts");
        for (int k = 0; k < KINDS; ++k) {
            max_ratio[k] = hr[k];
            counts[k] = hc[k];
        }
    } catch (const std::exception& e) {
        if (err && err_len) std::snprintf(err, err_len, "%s", e.what());
        status = BSF_E_CUDA;
    }
    if (base) cudaFree(base);
    return status;
}
