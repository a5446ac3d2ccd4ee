// bsf_worker: drop-in for the reference worker executable's streaming modes.
//
//   bsf_worker stage0stream [capacity=32768] [general|mega|record60|record80] [research|lean] [centers=1|8]
//   bsf_worker stream [capacity=32768]
//   bsf_worker megastream [capacity=32768] [profile=mega] [radius=7]
//   bsf_worker hunt <sequence_seed> <regions> [profile=mega] [radius=7] [outdir=.] [capacity=32768]
//                   [min_blocks=1000] [audit_mask=0] [top_keep=50]
//                   (headless search writing hunter_candidates.csv and the result boards, bsf_hunt.cpp)
//   bsf_worker boards <top_keep> <outdir>   |   bsf_worker candrows   |   bsf_worker javafmt <value> <precision>
//                   (no GPU: the result boards, candidate-log rows and Java number formatting of
//                   the hunt's writers, from records given on stdin)
//
// stage0stream / stream keep the reference protocol byte for byte
// (gpu_p20_benchmark.cpp:7310-7685; Java side src/GpuStage0Scout.java:143-335,
// src/GpuP20Scout.java:45-93): an 8-byte magic on stdout at start, then per
// request a LE u32 world count (0 or EOF ends the stream) and count LE i64 seeds
// on stdin, answered by a LE u32 count and the records. Errors print
// "ERROR: <message>" on stderr and exit 1; a closed stdout ends cleanly.
// megastream is the new MEGA mode: same request framing, response = LE u32
// record count followed by fixed 104-byte island records (see write_mega_record).
#include "../../include/bsf.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

bool read_exact(void* dst, std::size_t n) {
    return std::fread(dst, 1, n, stdin) == n;
}

bool read_le32(std::uint32_t& v, bool& eof) {
    unsigned char b[4];
    const std::size_t got = std::fread(b, 1, 4, stdin);
    if (got == 0 && std::feof(stdin)) {
        eof = true;
        return false;
    }
    if (got != 4) throw std::runtime_error("truncated stream request header");
    v = static_cast<std::uint32_t>(b[0]) | (static_cast<std::uint32_t>(b[1]) << 8) |
        (static_cast<std::uint32_t>(b[2]) << 16) | (static_cast<std::uint32_t>(b[3]) << 24);
    return true;
}

void put_le32(std::vector<unsigned char>& o, std::uint32_t v) {
    for (int k = 0; k < 4; ++k) o.push_back(static_cast<unsigned char>(v >> (8 * k)));
}

void put_le64(std::vector<unsigned char>& o, std::uint64_t v) {
    for (int k = 0; k < 8; ++k) o.push_back(static_cast<unsigned char>(v >> (8 * k)));
}

bool write_all(const void* p, std::size_t n) {
    if (std::fwrite(p, 1, n, stdout) != n) return false;
    return std::fflush(stdout) == 0;
}

int parse_profile(const std::string& v) {
    if (v == "general") return BSF_PROFILE_GENERAL;
    if (v == "mega") return BSF_PROFILE_MEGA;
    if (v == "record60") return BSF_PROFILE_RECORD60;
    if (v == "record80") return BSF_PROFILE_RECORD80;
    throw std::runtime_error("hunt profile must be general, mega, record60, or record80");
}

// HuntProfileConfig display names and gates (gpu_p20_benchmark.cpp:7262-7290).
const char* profile_name(int p) {
    static const char* names[] = {"GENERAL", "MEGA 30k+", "RECORD 60k+ (empirical)",
                                  "WORLD RECORD COARSE 700 (compact-thick safe)"};
    return names[p];
}

struct Gates {
    int p20, upper, high, coarse;
    double p19;
    bool megaTopology;
};
Gates profile_gates(int p) {
    switch (p) {
        case BSF_PROFILE_MEGA: return Gates{1, 8, 6, 85, 4.02, true};
        case BSF_PROFILE_RECORD60: return Gates{3, 19, 12, 95, 6.70, false};
        case BSF_PROFILE_RECORD80: return Gates{3, 19, 20, 700, 6.70, false};
        default: return Gates{1, 5, 5, 85, 4.02, false};
    }
}

// The stage pass counters of the stage0stream close summary, counted from the
// response records as the reference counts them (gpu_p20_benchmark.cpp:7556-7571).
struct StreamCounters {
    unsigned long long p20 = 0, stage1 = 0, stage05 = 0, p19Evaluated = 0, p19Passed = 0, p19Rejected = 0,
                       megaRejected = 0, coarseEvaluated = 0, coarsePassed = 0;

    void add(const unsigned char* r, const Gates& g) {
        const int a = r[0], b = r[1], c = r[2];
        const int d = r[4] | (r[5] << 8);
        if (a >= g.p20) ++p20;
        if (a >= g.p20 && b >= g.upper) ++stage1;
        if (a >= g.p20 && b >= g.upper && c >= g.high) {
            ++stage05;
            ++p19Evaluated;
            if (r[3] != 0) {
                ++p19Passed;
                if (r[7] != 0) {
                    ++megaRejected;
                } else {
                    ++coarseEvaluated;
                    if (d >= g.coarse) ++coarsePassed;
                }
            } else {
                ++p19Rejected;
            }
        }
    }
};

// printDevice (gpu_p20_benchmark.cpp:979-992): the device lines of the startup banner.
void print_device(int device) {
    char info[512];
    if (bsf_device_summary(device, info, sizeof(info)) == BSF_OK) std::fputs(info, stderr);
}

struct Handle {
    void* h = nullptr;
    explicit Handle(const bsf_config& c) {
        h = bsf_open(&c);
        if (!h) throw std::runtime_error("out of memory opening the GPU worker");
        if (bsf_last_error(h)[0] != '\0') throw std::runtime_error(bsf_last_error(h));
    }
    ~Handle() { bsf_close(h); }
};

std::vector<std::int64_t> read_seeds(std::uint32_t count) {
    std::vector<std::int64_t> seeds(count);
    std::vector<unsigned char> raw(static_cast<std::size_t>(count) * 8);
    if (!read_exact(raw.data(), raw.size())) throw std::runtime_error("truncated stream seed batch");
    for (std::uint32_t i = 0; i < count; ++i) {
        std::uint64_t v = 0;
        for (int k = 0; k < 8; ++k) v |= static_cast<std::uint64_t>(raw[i * 8 + k]) << (8 * k);
        seeds[i] = static_cast<std::int64_t>(v);
    }
    return seeds;
}

int stage0stream(std::uint32_t capacity, int profile, bool research, int centers) {
    if (capacity < 1) throw std::runtime_error("Stage0 stream capacity must be >= 1");
    if (centers != 1 && centers != 8) throw std::runtime_error("Stage0 stream center count must be 1 or 8");
    bsf_config cfg;
    bsf_default_config(&cfg);
    cfg.capacity = capacity;
    cfg.profile = profile;
    cfg.research = research ? 1 : 0;
    cfg.centers = centers;
    cfg.max_exact_radius = 1;
    Handle h(cfg);
    const Gates g = profile_gates(profile);
    // startup banner (gpu_p20_benchmark.cpp:7328-7343), logged verbatim by the app
    print_device(cfg.device);
    std::fprintf(stderr, "Stage0+P19+coarse stream capacity: %u worlds / %llu regions\n", capacity,
                 static_cast<unsigned long long>(capacity) * centers);
    std::fprintf(stderr, "Production multi-center: %d exact radius-7 regions/world | 15-chunk spacing | "
                 "region budget semantics\n", centers);
    std::fprintf(stderr, "Profile: %s | P20>=%d | Upper>=%d | High>=%d | P19>=%g/extreme | Coarse>=%d | %s\n",
                 profile_name(profile), g.p20, g.upper, g.high, g.p19, g.coarse,
                 g.megaTopology ? "Mega topology reject ON" : "topology reject OFF");
    if (profile == BSF_PROFILE_RECORD60 || profile == BSF_PROFILE_RECORD80)
        std::fprintf(stderr, "WARNING: record profile is empirically validated, not mathematically lossless.\n");
    std::fprintf(stderr, "Response telemetry: %s\n",
                 research ? "RESEARCH 34 bytes/region" : "LEAN 16 bytes/region + exact P19 double");
    std::fprintf(stderr, "Stage0+P19+coarse pipeline: exact P20 -> full upper survivors -> lower reentry -> "
                 "exact Stage0.75 gate -> optional Mega topology reject -> exact radius-7 coarse score "
                 "(GB300: FP32-screened kernels with exact FP64 fallback, device-side queues)\n");
    const std::size_t rec = research ? 34 : 16;
    const char magic[8] = {'S', 'T', '0', 'R', '3', '8', '1', '6'};
    if (!write_all(magic, 8)) return 0;
    std::vector<unsigned char> out;
    unsigned long long worlds = 0;
    StreamCounters sc;
    for (;;) {
        std::uint32_t count = 0;
        bool eof = false;
        if (!read_le32(count, eof) || count == 0) break;
        if (count > capacity) throw std::runtime_error("Stage0 stream batch exceeds configured world capacity");
        const std::vector<std::int64_t> seeds = read_seeds(count);
        out.assign(4 + static_cast<std::size_t>(count) * centers * rec, 0);
        out[0] = static_cast<unsigned char>(count);
        out[1] = static_cast<unsigned char>(count >> 8);
        out[2] = static_cast<unsigned char>(count >> 16);
        out[3] = static_cast<unsigned char>(count >> 24);
        const int st = bsf_stage0_filter(h.h, seeds.data(), count, out.data() + 4, out.size() - 4);
        if (st != BSF_OK) throw std::runtime_error(bsf_last_error(h.h));
        for (std::size_t i = 0; i < static_cast<std::size_t>(count) * centers; ++i) sc.add(out.data() + 4 + i * rec, g);
        if (!write_all(out.data(), out.size())) {
            std::fprintf(stderr, "Stage0+P19+coarse stream parent closed response pipe; exiting cleanly\n");
            break;
        }
        worlds += count;
    }
    // close summary (gpu_p20_benchmark.cpp:7601-7611)
    std::fprintf(stderr,
                 "Stage0+P19+coarse stream closed | worlds=%llu | regions=%llu | P20Passed=%llu | Stage1Passed=%llu"
                 " | Stage0.5Passed=%llu | Stage0.75Evaluated=%llu | Stage0.75Passed=%llu | Stage0.75Rejected=%llu"
                 " | MegaTopologyRejected=%llu | CoarseEvaluated=%llu | CoarsePassedTarget=%llu\n",
                 worlds, worlds * static_cast<unsigned long long>(centers), sc.p20, sc.stage1, sc.stage05,
                 sc.p19Evaluated, sc.p19Passed, sc.p19Rejected, sc.megaRejected, sc.coarseEvaluated, sc.coarsePassed);
    return 0;
}

int p20stream(std::uint32_t capacity) {
    if (capacity < 1) throw std::runtime_error("stream capacity must be >= 1");
    bsf_config cfg;
    bsf_default_config(&cfg);
    cfg.capacity = capacity;
    cfg.centers = 1;
    cfg.profile = BSF_PROFILE_GENERAL;
    cfg.max_exact_radius = 1;
    Handle h(cfg);
    std::fprintf(stderr, "P20 stream capacity: %u seeds\n", capacity);
    const char magic[8] = {'P', '2', '0', 'S', 'T', 'R', '0', '1'};
    if (!write_all(magic, 8)) return 0;
    std::vector<unsigned char> out;
    unsigned long long seedsTotal = 0, passed = 0;
    for (;;) {
        std::uint32_t count = 0;
        bool eof = false;
        if (!read_le32(count, eof) || count == 0) break;
        if (count > capacity) throw std::runtime_error("stream batch exceeds configured capacity");
        const std::vector<std::int64_t> seeds = read_seeds(count);
        out.assign(4 + count, 0);
        for (int k = 0; k < 4; ++k) out[k] = static_cast<unsigned char>(count >> (8 * k));
        if (bsf_p20_filter(h.h, seeds.data(), count, out.data() + 4, count) != BSF_OK)
            throw std::runtime_error(bsf_last_error(h.h));
        for (std::uint32_t i = 0; i < count; ++i) passed += out[4 + i] > 0;
        if (!write_all(out.data(), out.size())) throw std::runtime_error("failed writing stream response");
        seedsTotal += count;
    }
    std::fprintf(stderr, "P20 stream closed | seeds=%llu | passed=%llu\n", seedsTotal, passed);
    return 0;
}

// 104-byte MEGA record: seed i64, world u32, centre u32, centre chunk x/z i32,
// p20/upper/high/coarse i32, P19 score f64 bits, island found/blocks/columns,
// minX/maxX/minZ/maxZ/minY/maxY, centerX/centerZ, touchesSide, radiusUsed i32, one zero i32.
void write_mega_record(std::vector<unsigned char>& o, const bsf_mega_record& r) {
    put_le64(o, static_cast<std::uint64_t>(r.seed));
    put_le32(o, static_cast<std::uint32_t>(r.world_index));
    put_le32(o, static_cast<std::uint32_t>(r.center_index));
    put_le32(o, static_cast<std::uint32_t>(r.center_chunk_x));
    put_le32(o, static_cast<std::uint32_t>(r.center_chunk_z));
    put_le32(o, static_cast<std::uint32_t>(r.p20));
    put_le32(o, static_cast<std::uint32_t>(r.upper));
    put_le32(o, static_cast<std::uint32_t>(r.high));
    put_le32(o, static_cast<std::uint32_t>(r.coarse));
    std::uint64_t bits;
    std::memcpy(&bits, &r.p19_score, 8);
    put_le64(o, bits);
    const bsf_island& i = r.island;
    const std::int32_t f[14] = {i.found, i.blocks, i.columns, i.min_x, i.max_x, i.min_z, i.max_z,
                                i.min_y, i.max_y, i.center_x, i.center_z, i.touches_side, i.radius_used, 0};
    for (std::int32_t v : f) put_le32(o, static_cast<std::uint32_t>(v));
}

int megastream(std::uint32_t capacity, int profile, int radius) {
    bsf_config cfg;
    bsf_default_config(&cfg);
    cfg.capacity = capacity;
    cfg.profile = profile;
    cfg.centers = 8;
    Handle h(cfg);
    std::fprintf(stderr, "MEGA stream capacity: %u worlds | profile %s | exact radius %d\n", capacity,
                 profile_name(profile), radius);
    const char magic[8] = {'M', 'E', 'G', 'A', 'S', 'T', '0', '1'};
    if (!write_all(magic, 8)) return 0;
    std::vector<bsf_mega_record> recs(65536);
    for (;;) {
        std::uint32_t count = 0;
        bool eof = false;
        if (!read_le32(count, eof) || count == 0) break;
        if (count > capacity) throw std::runtime_error("MEGA stream batch exceeds configured world capacity");
        const std::vector<std::int64_t> seeds = read_seeds(count);
        std::uint32_t n = 0;
        bsf_stage_counts counts;
        if (bsf_mega_search(h.h, seeds.data(), count, radius, nullptr, recs.data(),
                            static_cast<std::uint32_t>(recs.size()), &n, &counts) != BSF_OK)
            throw std::runtime_error(bsf_last_error(h.h));
        std::vector<unsigned char> out;
        put_le32(out, n);
        for (std::uint32_t k = 0; k < n; ++k) write_mega_record(out, recs[k]);
        if (!write_all(out.data(), out.size())) break;
    }
    return 0;
}

}  // namespace

namespace bsfhunt {
int hunt_main(int argc, char** argv);
int javafmt_main(int argc, char** argv);
int boards_main(int argc, char** argv);
int candrows_main(int argc, char** argv);
}  // namespace bsfhunt

int main(int argc, char** argv) {
    try {
        if (argc < 2) {
            std::fprintf(stderr,
                         "Usage:\n"
                         "  bsf_worker stage0stream [capacity=32768] [general|mega|record60|record80] [research|lean] "
                         "[centers=1|8]\n"
                         "  bsf_worker stream [capacity=32768]\n"
                         "  bsf_worker megastream [capacity=32768] [profile=mega] [radius=7]\n"
                         "  bsf_worker hunt <sequence_seed> <regions> [profile=mega] [radius=7] [outdir=.] "
                         "[capacity=32768] [min_blocks=1000] [audit_mask=0] [top_keep=50]\n"
                         "  bsf_worker boards <top_keep> <outdir>   (records on stdin)\n"
                         "  bsf_worker candrows   (records on stdin; candidate-log rows on stdout)\n"
                         "  bsf_worker javafmt <value> <precision>\n");
            return 1;
        }
        const std::string mode = argv[1];
        if (mode == "hunt") return bsfhunt::hunt_main(argc, argv);
        if (mode == "javafmt") return bsfhunt::javafmt_main(argc, argv);
        if (mode == "boards") return bsfhunt::boards_main(argc, argv);
        if (mode == "candrows") return bsfhunt::candrows_main(argc, argv);
        const std::uint32_t cap = argc > 2 ? static_cast<std::uint32_t>(std::strtoul(argv[2], nullptr, 10)) : 32768u;
        if (mode == "stream") return p20stream(cap);
        if (mode == "stage0stream") {
            const int profile = argc > 3 ? parse_profile(argv[3]) : BSF_PROFILE_GENERAL;
            bool research = true;
            if (argc > 4) {
                const std::string t = argv[4];
                if (t == "research") research = true;
                else if (t == "lean") research = false;
                else throw std::runtime_error("stage0stream telemetry must be research or lean");
            }
            const int centers = argc > 5 ? std::atoi(argv[5]) : 1;
            return stage0stream(cap, profile, research, centers);
        }
        if (mode == "megastream") {
            const int profile = argc > 3 ? parse_profile(argv[3]) : BSF_PROFILE_MEGA;
            const int radius = argc > 4 ? std::atoi(argv[4]) : 7;
            return megastream(cap, profile, radius);
        }
        throw std::runtime_error("unknown mode: " + mode);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "ERROR: %s\n", e.what());
        return 1;
    }
}
