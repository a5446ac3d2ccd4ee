// Headless MEGA hunt for bsf_worker: the reference app's GPU search loop
// (IslandSearchEngine.java:1314-1443, batches of worlds from deterministic
// seeds, one attempt per region) and its candidate log, hunter_candidates.csv
// (initializeCandidateCsv / appendCandidateCsv, IslandSearchEngine.java:4826-4960),
// written from the C ABI's MEGA records, plus the run manifest (manifest.txt, the
// reference's key=value format) and the stage counters (run_manifest.json). With an audit mask
// it also re-scans a sample of rejected regions exactly and logs them like the
// reference's record_reject_audits.csv (processLeanRejectAudit,
// IslandSearchEngine.java:2126-2188; sampling :1403-1476, 2512-2529).
//
// It keeps the reference's top-result boards and writes their files
// (bsf_boards.h).
//
//   bsf_worker hunt <sequence_seed> <regions> [profile=mega] [radius=7] [outdir=.]
//                   [capacity=32768] [min_blocks=1000] [audit_mask=0] [top_keep=50]
//   bsf_worker javafmt <value> <precision>      (formatting check: Java's %.<p>f)
//   bsf_worker boards <top_keep> <outdir>       (board files from records on stdin, one per
//        line: seed blocks columns centerX centerZ minX maxX minZ maxZ minY maxY radius touches)
#include "../../include/bsf.h"
#include "bsf_boards.h"

#include <charconv>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace bsfhunt {

// deterministicSeedForAttempt (IslandSearchEngine.java:2551-2556), SplitMix64.
std::int64_t seed_for_attempt(std::int64_t sequenceSeed, std::int64_t attempt) {
    std::uint64_t z = static_cast<std::uint64_t>(sequenceSeed) +
                      static_cast<std::uint64_t>(attempt) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return static_cast<std::int64_t>(z ^ (z >> 31));
}

// Java's String.format(Locale.US, "%.<prec>f", v): the shortest decimal digits
// that identify v, rounded half-up at <prec> fractional places.
std::string java_fixed(double v, int prec) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "Infinity" : "-Infinity";
    char buf[64];
    const auto res = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::scientific);
    std::string sci(buf, res.ptr);
    bool neg = false;
    if (!sci.empty() && sci[0] == '-') {
        neg = true;
        sci.erase(0, 1);
    }
    const std::size_t ePos = sci.find('e');
    std::string digits;
    for (std::size_t i = 0; i < ePos; ++i)
        if (sci[i] != '.') digits.push_back(sci[i]);
    const int exp10 = std::atoi(sci.c_str() + ePos + 1);  // value = d.ddd x 10^exp10
    // integer part digits = exp10 + 1; place the digits on a fixed grid
    int intLen = exp10 + 1;
    std::string intPart, frac;
    if (intLen <= 0) {
        intPart = "0";
        frac = std::string(static_cast<std::size_t>(-intLen), '0') + digits;
    } else if (static_cast<std::size_t>(intLen) >= digits.size()) {
        intPart = digits + std::string(static_cast<std::size_t>(intLen) - digits.size(), '0');
    } else {
        intPart = digits.substr(0, static_cast<std::size_t>(intLen));
        frac = digits.substr(static_cast<std::size_t>(intLen));
    }
    bool roundUp = false;
    if (frac.size() > static_cast<std::size_t>(prec)) {
        roundUp = frac[static_cast<std::size_t>(prec)] >= '5';
        frac.resize(static_cast<std::size_t>(prec));
    }
    frac.resize(static_cast<std::size_t>(prec), '0');
    if (roundUp) {
        std::string all = intPart + frac;
        int i = static_cast<int>(all.size()) - 1;
        for (; i >= 0; --i) {
            if (all[static_cast<std::size_t>(i)] == '9') {
                all[static_cast<std::size_t>(i)] = '0';
            } else {
                ++all[static_cast<std::size_t>(i)];
                break;
            }
        }
        if (i < 0) all.insert(all.begin(), '1');
        intPart = all.substr(0, all.size() - static_cast<std::size_t>(prec));
        frac = all.substr(all.size() - static_cast<std::size_t>(prec));
    }
    std::string out = neg ? "-" : "";
    out += intPart;
    if (prec > 0) out += "." + frac;
    return out;
}

const char* jbool(bool b) { return b ? "true" : "false"; }

const char* kHeader =
    "attempt,seed,stage0,stage0Y88,coarse,p20,upper,high,p19Pass,p19Score,p19Extreme,searchCenterChunkX,"
    "searchCenterChunkZ,matched,status,rawBlocks,verifiedBlocks,rawRadius,verifiedRadius,rawTouchesSide,"
    "verifiedTouchesSide,columns,width,depth,footprintArea,fillPercent,avgThickness,minY,maxY,centerX,centerZ,"
    "minX,maxX,minZ,maxZ,hotScanned,hotRadius,hotBlocks,hotTouchesSide,finalSource\n";

// One candidate line (appendCandidateCsv): raw = the scan at the search radius
// after border verification, verified = the chosen island, hot = the hot scan.
std::string candidate_line(std::int64_t attempt, const bsf_mega_record& r, bool duplicate) {
    const bsf_island& raw = r.raw_island;
    const bsf_island& fin = r.island;
    const bsf_island& hot = r.hot_island;
    const bool haveRaw = raw.found != 0, haveFinal = fin.found != 0, haveHot = hot.found != 0;
    const bool finalIsHot = haveFinal && r.final_source == 2;
    const bool matched = haveFinal && !duplicate;
    // the final island is the raw scan's or the hot scan's: never a border-verified replacement
    const char* finalSource = duplicate ? "duplicate_merged" : (finalIsHot ? "hot_scan" : (haveFinal ? "raw" : "none"));
    const char* status;
    if (duplicate) status = "duplicate_region_merged";
    else if (haveFinal && finalIsHot && fin.touches_side) status = "matched_hot_scan_still_touches_side";
    else if (haveFinal && finalIsHot) status = "matched_hot_scan";
    else if (haveFinal && fin.touches_side) status = "matched_still_touches_side";
    else if (haveFinal) status = "matched";
    else if (haveRaw) status = "border_rejected_or_invalid";
    else if (r.hot_scanned) status = "hot_scan_no_match";
    else status = "no_match";
    // finalComponent = verified if any, else raw
    const bsf_island& comp = haveFinal ? fin : raw;
    const bool haveComp = haveFinal || haveRaw;
    const int columns = haveComp ? comp.columns : 0;
    const int width = haveComp ? comp.max_x - comp.min_x + 1 : 0;
    const int depth = haveComp ? comp.max_z - comp.min_z + 1 : 0;
    const int area = width * depth;
    const double fill = haveComp ? 100.0 * comp.columns / static_cast<double>(area > 1 ? area : 1) : 0.0;
    const double thick = haveComp ? comp.blocks / static_cast<double>(comp.columns > 1 ? comp.columns : 1) : 0.0;
    char buf[1024];
    std::snprintf(buf, sizeof(buf),
                  "%lld,%lld,%d,%d,%d,%d,%d,%d,%s,%s,%s,%d,%d,%s,%s,%d,%d,%d,%d,%s,%s,%d,%d,%d,%d,%s,%s,%d,%d,%d,%d,%d,"
                  "%d,%d,%d,%s,%d,%d,%s,%s\n",
                  static_cast<long long>(attempt), static_cast<long long>(r.seed), r.high, r.high, r.coarse, r.p20,
                  r.upper, r.high, jbool(r.p19_pass != 0), java_fixed(r.p19_score, 6).c_str(),
                  jbool(r.p19_extreme != 0), r.center_chunk_x, r.center_chunk_z, jbool(matched), status,
                  haveRaw ? raw.blocks : 0, haveFinal ? fin.blocks : 0, haveRaw ? raw.radius_used : 0,
                  haveFinal ? fin.radius_used : 0, jbool(haveRaw && raw.touches_side),
                  jbool(haveFinal && fin.touches_side), columns, width, depth, area, java_fixed(fill, 4).c_str(),
                  java_fixed(thick, 4).c_str(), haveComp ? comp.min_y : 0, haveComp ? comp.max_y : 0,
                  haveComp ? comp.center_x : 0, haveComp ? comp.center_z : 0, haveComp ? comp.min_x : 0,
                  haveComp ? comp.max_x : 0, haveComp ? comp.min_z : 0, haveComp ? comp.max_z : 0,
                  jbool(r.hot_scanned != 0), haveHot ? hot.radius_used : 0, haveHot ? hot.blocks : 0,
                  jbool(haveHot && hot.touches_side), finalSource);
    return buf;
}

const char* kAuditHeader =
    "attempt,seed,searchCenterChunkX,searchCenterChunkZ,rejectStage,rejectReason,p20,upper,high,p19Pass,p19Score,"
    "p19Extreme,coarse,exactScanMs,exactMatched,exactBlocks,exactColumns,exactWidth,exactDepth,exactMinY,exactMaxY,"
    "exactRadiusUsed,exactTouchesSideBorder\n";

// The worker profile's gates (HuntProfileConfig, gpu_p20_benchmark.cpp:7262-7290).
struct Gates {
    int p20, upper, high, coarse;
};
Gates gates_of(int profile) {
    switch (profile) {
        case BSF_PROFILE_MEGA: return Gates{1, 8, 6, 85};
        case BSF_PROFILE_RECORD60: return Gates{3, 19, 12, 95};
        case BSF_PROFILE_RECORD80: return Gates{3, 19, 20, 700};
        default: return Gates{1, 5, 5, 85};
    }
}

const char* reject_name(int stage) {  // rejectStageName (IslandSearchEngine.java:2190-2201)
    switch (stage) {
        case 1: return "p20";
        case 2: return "upper";
        case 3: return "reentry";
        case 4: return "high";
        case 5: return "p19";
        case 6: return "coarse";
        case 7: return "mega_topology";
        default: return "unknown";
    }
}

int parse_profile_name(const std::string& v) {
    if (v == "general") return BSF_PROFILE_GENERAL;
    if (v == "mega") return BSF_PROFILE_MEGA;
    if (v == "record60") return BSF_PROFILE_RECORD60;
    if (v == "record80") return BSF_PROFILE_RECORD80;
    throw std::invalid_argument("unknown profile " + v);
}

// Java's Double.toString for the settings written to the manifest: the shortest
// digits that identify the value, with at least one fractional digit (4.02, 6.7, 2.0).
std::string java_double(double v) {
    char buf[64];
    const auto res = std::to_chars(buf, buf + sizeof(buf), v);
    std::string t(buf, res.ptr);
    if (t.find_first_of(".eE") == std::string::npos) t += ".0";
    return t;
}

// The settings and outcome of one headless hunt, as manifest.txt records them.
struct ManifestInfo {
    std::string status, outdir, label;
    long long startMs = 0, endMs = 0;
    std::int64_t checked = 0, matches = 0, topUpdates = 0, regionBudget = 0, sequenceSeed = 0;
    int profile = BSF_PROFILE_MEGA, radius = 7, topKeep = 50;
    std::uint32_t capacity = 32768;
    std::int64_t auditMask = 0;
    bsf_match_settings ms{};
};

// writeManifest (IslandSearchEngine.java:4309-4449): "BetaSeedFinder run manifest"
// then key=value lines in the reference's order and groups, so the app's run
// history (RunRepository.refresh/parseManifest, RunRepository.java:25-40, 163-171;
// RunRecord.java:29-41) lists headless hunts beside its own runs. Keys that only
// describe the app's CPU path or GUI are written with the values a headless GPU
// hunt has (no previews, no feature log, deterministic seeds).
void write_manifest(const ManifestInfo& m) {
    static const char* kProfileName[4] = {"GENERAL", "MEGA 30k+", "RECORD 60k+", "WORLD RECORD 80k+"};
    const Gates g = gates_of(m.profile);
    const double p19Min = (m.profile == BSF_PROFILE_RECORD60 || m.profile == BSF_PROFILE_RECORD80) ? 6.70 : 4.02;
    const bool mega = m.profile == BSF_PROFILE_MEGA;
    const bool rec60 = m.profile == BSF_PROFILE_RECORD60, rec80 = m.profile == BSF_PROFILE_RECORD80;
    auto jb = [](bool b) { return b ? "true" : "false"; };
    std::string s = "BetaSeedFinder run manifest\n";
    auto kv = [&](const char* k, const std::string& v) { s += std::string(k) + "=" + v + "\n"; };
    auto ki = [&](const char* k, long long v) { kv(k, std::to_string(v)); };
    kv("build", "GB300-sm103a-bsf_worker-hunt");
    kv("status", m.status);
    kv("runFolder", m.outdir);
    kv("runLabel", m.label);
    ki("startEpochMs", m.startMs);
    ki("endEpochMs", m.endMs);
    if (m.endMs > m.startMs) {
        char b[64];
        std::snprintf(b, sizeof(b), "%.3f", (m.endMs - m.startMs) / 1000.0);
        kv("elapsedSeconds", b);
    }
    ki("checked", m.checked);
    ki("matches", m.matches);
    ki("topUpdates", m.topUpdates);
    kv("checkedUnit", "radius7Regions");
    ki("regionBudget", m.regionBudget);
    ki("gpuCoverageCentersPerWorld", 8);
    ki("gpuCoverageCenterSpacingChunks", 15);
    kv("gpuProtocol", "ST0R3816");
    ki("gpuTerrainPerlinCacheStates", 66);
    ki("gpuClimatePerlinCacheStates", 10);
    kv("gpuCachedCoarseInitialization", "true");
    s += "\n";
    ki("chunkRadius", m.radius);
    ki("seedsToCheck", m.regionBudget);
    ki("threads", 1);
    kv("gpuStage0Enabled", "true");
    ki("gpuStage0BatchSize", m.capacity);
    kv("gpuStage0Compatible", "true");
    kv("gpuStage0Executable", "bsf_worker");
    kv("gpuP20Enabled", "false");
    ki("minBlocks", m.ms.min_blocks);
    ki("minColumns", m.ms.min_columns);
    ki("minYForMatch", m.ms.min_y_for_match);
    ki("minWidth", m.ms.min_width);
    ki("minDepth", m.ms.min_depth);
    kv("minAvgThickness", java_double(m.ms.min_avg_thickness));
    ki("topResultsToKeep", m.topKeep);
    kv("savePreviews", "false");
    kv("featureLoggingEnabled", "false");
    kv("filterShadowResearchEnabled", "false");
    kv("nativeResponseMode", "lean");
    kv("overnightResearchForcedAuditsEnabled", jb(m.auditMask > 0));
    s += "\n";
    kv("hunterMode", "true");
    ki("huntProfile", m.profile);
    kv("huntProfileName", kProfileName[m.profile]);
    kv("megaMode", jb(mega));
    kv("recordHuntMode", jb(rec60));
    kv("extremeRecordHuntMode", jb(rec80));
    ki("effectiveP20MinPositiveColumns", g.p20);
    kv("effectiveP19MinScore", java_double(p19Min));
    kv("filterResearchEnabled", "false");
    ki("megaUpperMinPositiveColumns", g.upper);
    ki("megaHighMinReentryColumns", g.high);
    kv("megaExtremeTopologyBypassPreserved", "true");
    ki("hunterCoarseMinCells", g.coarse);
    kv("stage075MonsterGateThreshold", java_double(p19Min));
    kv("stage075MonsterGateTrees", "16");
    kv("recordRejectAuditPath", m.auditMask > 0 ? m.outdir + "/record_reject_audits.csv" : "");
    kv("leanTelemetryP19Score", "exactDouble");
    kv("borderVerifyRadii", "10,13,16,20,24");
    ki("borderVerifyMaxRadius", 24);
    ki("dangerousRejectExactScanMinCoarse", g.coarse);
    kv("hotSeedScanEnabled", "true");
    ki("hotSeedCoarseThreshold", 120);
    ki("hotSeedScanRadius", 16);
    s += "\n";
    kv("performanceProfilerEnabled", "false");
    kv("deterministicSeedMode", "true");
    ki("deterministicSeedSequenceSeed", m.sequenceSeed);
    const std::string path = m.outdir + "/manifest.txt";
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fwrite(s.data(), 1, s.size(), f);
    std::fclose(f);
}

long long epoch_ms() {
    return std::chrono::duration_cast<std::chrono::milliseconds>(
               std::chrono::system_clock::now().time_since_epoch()).count();
}

int hunt_main(int argc, char** argv) {
    if (argc < 4) throw std::invalid_argument("hunt needs <sequence_seed> <regions>");
    const std::int64_t sequenceSeed = std::strtoll(argv[2], nullptr, 10);
    const std::int64_t regionsToCheck = std::strtoll(argv[3], nullptr, 10);
    const std::string profileName = argc > 4 ? argv[4] : "mega";
    const int profile = parse_profile_name(profileName);
    const int radius = argc > 5 ? std::atoi(argv[5]) : 7;
    const std::string outdir = argc > 6 ? argv[6] : ".";
    const std::uint32_t capacity = argc > 7 ? static_cast<std::uint32_t>(std::strtoul(argv[7], nullptr, 10)) : 32768u;
    const int minBlocks = argc > 8 ? std::atoi(argv[8]) : 1000;
    // audits: rejected regions with (seed & mask) == 0, P20 rejects with (attempt & p20Mask) == 0
    // (the record profiles use the same mask; the others 32767, IslandSearchEngine.java:2520-2525)
    const std::int64_t auditMask = argc > 9 ? std::strtoll(argv[9], nullptr, 10) : 0;
    const std::int64_t p20AuditMask =
        (profile == BSF_PROFILE_RECORD60 || profile == BSF_PROFILE_RECORD80) ? auditMask : 32767;
    const int topKeep = argc > 10 ? std::atoi(argv[10]) : 50;  // SearchSettings.topResultsToKeep
    const Gates gate = gates_of(profile);
    if (regionsToCheck <= 0 || capacity == 0 || radius < 0 || radius > 24 || topKeep < 1)
        throw std::invalid_argument("hunt: regions, capacity and top_keep must be positive and radius 0..24");
    Boards boards(topKeep);
    boards.write(outdir);  // "No results yet." boards and the CSV header, as at the reference's run start
    ManifestInfo mi;
    {
        char* abs = realpath(outdir.c_str(), nullptr);
        mi.outdir = abs ? abs : outdir;
        std::free(abs);
        const std::size_t cut = mi.outdir.find_last_of('/');
        mi.label = cut == std::string::npos ? mi.outdir : mi.outdir.substr(cut + 1);
    }
    mi.status = "RUNNING";
    mi.startMs = epoch_ms();
    mi.regionBudget = regionsToCheck;
    mi.sequenceSeed = sequenceSeed;
    mi.profile = profile;
    mi.radius = radius;
    mi.topKeep = topKeep;
    mi.capacity = capacity;
    mi.auditMask = auditMask;
    bsf_default_match_settings(&mi.ms);
    mi.ms.min_blocks = minBlocks;
    write_manifest(mi);  // the reference writes a RUNNING manifest at run start (:761)

    bsf_config cfg;
    bsf_default_config(&cfg);
    cfg.capacity = capacity;
    cfg.profile = profile;
    cfg.centers = 8;
    cfg.max_exact_radius = 24;
    void* h = bsf_open(&cfg);
    if (!h) throw std::runtime_error("bsf_open failed");
    if (bsf_last_error(h)[0]) {
        const std::string e = bsf_last_error(h);
        bsf_close(h);
        throw std::runtime_error("bsf_open: " + e);
    }
    bsf_match_settings ms;
    bsf_default_match_settings(&ms);
    ms.min_blocks = minBlocks;

    const std::string csvPath = outdir + "/hunter_candidates.csv";
    std::FILE* csv = std::fopen(csvPath.c_str(), "wb");
    if (!csv) {
        bsf_close(h);
        throw std::runtime_error("cannot write " + csvPath);
    }
    std::fputs(kHeader, csv);
    std::FILE* audits = nullptr;
    if (auditMask > 0) {
        audits = std::fopen((outdir + "/record_reject_audits.csv").c_str(), "wb");
        if (!audits) {
            std::fclose(csv);
            bsf_close(h);
            throw std::runtime_error("cannot write record_reject_audits.csv");
        }
        std::fputs(kAuditHeader, audits);
    }
    std::vector<std::uint8_t> regionRecs(audits ? capacity * static_cast<std::size_t>(8) * 34 : 0);
    std::int64_t audited = 0, auditHits = 0;

    const int centers = 8;
    std::vector<std::int64_t> seeds(capacity);
    std::vector<bsf_mega_record> recs(capacity * static_cast<std::size_t>(centers));
    std::set<std::tuple<std::int64_t, int, int, int, int, int, int, int, int>> seen;  // registerUniqueMatch keys
    std::int64_t issuedRegions = 0, issuedWorlds = 0, candidates = 0, matches = 0, duplicates = 0, bestBlocks = 0;
    std::int64_t topUpdates = 0;
    bsf_stage_counts total{};
    const auto t0 = std::chrono::steady_clock::now();
    while (issuedRegions < regionsToCheck) {
        const std::int64_t remaining = regionsToCheck - issuedRegions;
        const int regionsThisBatch = static_cast<int>(std::min<std::int64_t>(
            static_cast<std::int64_t>(capacity) * centers, remaining));
        const int count = (regionsThisBatch + centers - 1) / centers;
        for (int i = 0; i < count; ++i) seeds[i] = seed_for_attempt(sequenceSeed, issuedWorlds + i + 1);
        std::uint32_t n = 0;
        bsf_stage_counts c{};
        const int rc = bsf_mega_search(h, seeds.data(), static_cast<std::uint32_t>(count), radius, &ms, recs.data(),
                                       static_cast<std::uint32_t>(recs.size()), &n, &c);
        if (rc != BSF_OK) {
            const std::string e = bsf_last_error(h);
            std::fclose(csv);
            bsf_close(h);
            throw std::runtime_error("bsf_mega_search: " + e);
        }
        for (std::size_t f = 0; f < sizeof(bsf_stage_counts) / sizeof(uint64_t); ++f)
            reinterpret_cast<uint64_t*>(&total)[f] += reinterpret_cast<const uint64_t*>(&c)[f];
        for (std::uint32_t k = 0; k < n; ++k) {
            const bsf_mega_record& r = recs[k];
            const int regionOffset = r.world_index * centers + r.center_index;
            if (regionOffset >= regionsThisBatch) continue;  // centres past the requested region count
            bool duplicate = false;
            if (r.island.found) {
                const auto key = std::make_tuple(r.seed, r.island.min_x, r.island.max_x, r.island.min_z,
                                                 r.island.max_z, r.island.min_y, r.island.max_y, r.island.blocks,
                                                 r.island.columns);
                duplicate = !seen.insert(key).second;
                if (duplicate) ++duplicates;
                else {
                    ++matches;
                    if (r.island.blocks > bestBlocks) bestBlocks = r.island.blocks;
                    const bsf_island& i = r.island;
                    topUpdates += boards.add(make_board_record(r.seed, i.blocks, i.columns, i.center_x, i.center_z, i.min_x, i.max_x,
                                                 i.min_z, i.max_z, i.min_y, i.max_y, i.radius_used,
                                                 i.touches_side != 0, outdir));
                }
            }
            const std::int64_t attempt = issuedRegions + regionOffset + 1;
            std::fputs(candidate_line(attempt, r, duplicate).c_str(), csv);
            ++candidates;
        }
        if (audits) {
            if (bsf_last_region_records(h, regionRecs.data(), regionRecs.size()) != BSF_OK) {
                const std::string e = bsf_last_error(h);
                std::fclose(csv);
                std::fclose(audits);
                bsf_close(h);
                throw std::runtime_error("bsf_last_region_records: " + e);
            }
            for (int ro = 0; ro < regionsThisBatch; ++ro) {
                const std::uint8_t* q = regionRecs.data() + static_cast<std::size_t>(ro) * 34;
                const int p20 = q[0], upper = q[1], high = q[2];
                const bool p19Pass = q[3] != 0, extreme = q[6] != 0, mega = q[7] != 0;
                const int coarse = q[4] | (q[5] << 8);
                double p19Score;
                std::memcpy(&p19Score, q + 8, 8);
                int stage;  // rejectStage (IslandSearchEngine.java:1368-1376), with the worker's gates
                if (p20 < gate.p20) stage = 1;
                else if (upper < gate.upper) stage = 2;
                else if (high < gate.high) stage = 4;
                else if (!p19Pass) stage = 5;
                else if (mega) stage = 7;
                else if (coarse < gate.coarse) stage = 6;
                else stage = 0;
                const std::int64_t attempt = issuedRegions + ro + 1;
                const std::int64_t seed = seeds[ro / centers];
                const bool sampled = stage == 1 ? (attempt & p20AuditMask) == 0
                                                : (stage != 0 && stage != 7 && (seed & auditMask) == 0);
                if (!sampled) continue;
                // GpuStage0Scout centres (src/GpuStage0Scout.java:19-21)
                static const int kCx[8] = {0, 15, 0, 15, -15, -15, 0, 15};
                static const int kCz[8] = {0, 0, 15, 15, 0, 15, -15, -15};
                const int cx = kCx[ro % centers], cz = kCz[ro % centers];
                bsf_island isl{};
                const auto a0 = std::chrono::steady_clock::now();
                if (bsf_exact_scan(h, seed, cx, cz, radius, &ms, &isl) != BSF_OK) {
                    const std::string e = bsf_last_error(h);
                    std::fclose(csv);
                    std::fclose(audits);
                    bsf_close(h);
                    throw std::runtime_error("bsf_exact_scan: " + e);
                }
                const double ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a0).count();
                char line[512];
                std::snprintf(line, sizeof(line), "%lld,%lld,%d,%d,%d,%s,%d,%d,%d,%s,%s,%s,%d,%s,%s,%d,%d,%d,%d,%d,%d,%d,%s\n",
                              static_cast<long long>(attempt), static_cast<long long>(seed), cx, cz, stage,
                              reject_name(stage), p20, upper, high, jbool(p19Pass), java_fixed(p19Score, 6).c_str(),
                              jbool(extreme), coarse, java_fixed(ms_, 3).c_str(), jbool(isl.found != 0),
                              isl.found ? isl.blocks : 0, isl.found ? isl.columns : 0,
                              isl.found ? isl.max_x - isl.min_x + 1 : 0, isl.found ? isl.max_z - isl.min_z + 1 : 0,
                              isl.found ? isl.min_y : -1, isl.found ? isl.max_y : -1,
                              isl.found ? isl.radius_used : radius, jbool(isl.found && isl.touches_side));
                std::fputs(line, audits);
                ++audited;
                if (isl.found) ++auditHits;
            }
        }
        issuedWorlds += count;
        issuedRegions += regionsThisBatch;
    }
    std::fclose(csv);
    if (audits) std::fclose(audits);
    boards.write(outdir);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    bsf_close(h);
    mi.status = "FINISHED";
    mi.endMs = epoch_ms();
    mi.checked = issuedRegions;
    mi.matches = matches;
    mi.topUpdates = topUpdates;
    write_manifest(mi);

    // the worker's own counters beside the reference manifest (stage counts have no manifest keys)
    const std::string manifestPath = outdir + "/run_manifest.json";
    std::FILE* m = std::fopen(manifestPath.c_str(), "wb");
    if (!m) throw std::runtime_error("cannot write " + manifestPath);
    std::fprintf(m,
                 "{\n  \"mode\": \"gpu_hunt\",\n  \"deterministicSeedSequenceSeed\": %lld,\n  \"seedsToCheck\": %lld,\n"
                 "  \"worldsChecked\": %lld,\n  \"profile\": \"%s\",\n  \"chunkRadius\": %d,\n  \"minBlocks\": %d,\n"
                 "  \"candidates\": %lld,\n  \"matches\": %lld,\n  \"duplicateRegionHits\": %lld,\n"
                 "  \"bestBlocks\": %lld,\n  \"p20Passed\": %llu,\n  \"upperPassed\": %llu,\n  \"highPassed\": %llu,\n"
                 "  \"p19Passed\": %llu,\n  \"megaRejected\": %llu,\n  \"coarseEvaluated\": %llu,\n"
                 "  \"coarsePassed\": %llu,\n  \"rejectAudits\": %lld,\n  \"rejectAuditMatches\": %lld,\n"
                 "  \"elapsedSeconds\": %.3f\n}\n",
                 static_cast<long long>(sequenceSeed), static_cast<long long>(regionsToCheck),
                 static_cast<long long>(issuedWorlds), profileName.c_str(), radius, minBlocks,
                 static_cast<long long>(candidates), static_cast<long long>(matches),
                 static_cast<long long>(duplicates), static_cast<long long>(bestBlocks),
                 static_cast<unsigned long long>(total.p20_passed), static_cast<unsigned long long>(total.upper_passed),
                 static_cast<unsigned long long>(total.high_passed), static_cast<unsigned long long>(total.p19_passed),
                 static_cast<unsigned long long>(total.mega_rejected),
                 static_cast<unsigned long long>(total.coarse_evaluated),
                 static_cast<unsigned long long>(total.coarse_passed), static_cast<long long>(audited),
                 static_cast<long long>(auditHits), secs);
    std::fclose(m);
    std::fprintf(stderr, "HUNT DONE | regions=%lld worlds=%lld candidates=%lld matches=%lld duplicates=%lld | %.2f s\n",
                 static_cast<long long>(regionsToCheck), static_cast<long long>(issuedWorlds),
                 static_cast<long long>(candidates), static_cast<long long>(matches),
                 static_cast<long long>(duplicates), secs);
    return 0;
}

int boards_main(int argc, char** argv) {
    if (argc < 4) throw std::invalid_argument("boards needs <top_keep> <outdir>");
    const int keep = std::atoi(argv[2]);
    if (keep < 1) throw std::invalid_argument("boards: top_keep must be positive");
    const std::string outdir = argv[3];
    Boards boards(keep);
    long long seed;
    int v[12];
    while (std::scanf("%lld %d %d %d %d %d %d %d %d %d %d %d %d", &seed, &v[0], &v[1], &v[2], &v[3], &v[4], &v[5],
                      &v[6], &v[7], &v[8], &v[9], &v[10], &v[11]) == 13)
        boards.add(make_board_record(seed, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10],
                                     v[11] != 0, outdir));
    boards.write(outdir);
    return 0;
}

// Candidate-log rows from records given on stdin, one per line: attempt seed p20
// upper high coarse p19_pass p19_score p19_extreme center_chunk_x center_chunk_z
// duplicate hot_scanned final_source, then the chosen, raw and hot islands as
// found blocks columns min_x max_x min_z max_z min_y max_y center_x center_z
// touches_side radius_used. Writes the header, then one row per record.
int candrows_main(int, char**) {
    std::fputs(kHeader, stdout);
    long long attempt, seed;
    for (;;) {
        bsf_mega_record r{};
        int duplicate = 0;
        if (std::scanf("%lld %lld %d %d %d %d %d %lf %d %d %d %d %d %d", &attempt, &seed, &r.p20, &r.upper, &r.high,
                       &r.coarse, &r.p19_pass, &r.p19_score, &r.p19_extreme, &r.center_chunk_x, &r.center_chunk_z,
                       &duplicate, &r.hot_scanned, &r.final_source) != 14)
            break;
        r.seed = seed;
        for (bsf_island* i : {&r.island, &r.raw_island, &r.hot_island})
            if (std::scanf("%d %d %d %d %d %d %d %d %d %d %d %d %d", &i->found, &i->blocks, &i->columns, &i->min_x,
                           &i->max_x, &i->min_z, &i->max_z, &i->min_y, &i->max_y, &i->center_x, &i->center_z,
                           &i->touches_side, &i->radius_used) != 13)
                throw std::invalid_argument("candrows: truncated record");
        std::fputs(candidate_line(attempt, r, duplicate != 0).c_str(), stdout);
    }
    return 0;
}

int javafmt_main(int argc, char** argv) {
    if (argc < 4) throw std::invalid_argument("javafmt needs <value> <precision>");
    std::printf("%s\n", java_fixed(std::strtod(argv[2], nullptr), std::atoi(argv[3])).c_str());
    return 0;
}

}  // namespace bsfhunt
