// Harness around the reference's own host C++ (test infrastructure only).
//
// Compiled by oracle/build_ref.sh with the reference headers included in place
// from the reference checkout (native/src/p20_exact_math.hpp,
// coarse_exact_core.hpp, p19_monster_gate.hpp); nothing from the reference is
// copied into this repository. The exported functions let the tests pin the C
// oracle against the reference's arithmetic on many random inputs. Only this
// container builds it (the reference sources are not present elsewhere).
#include "p20_exact_math.hpp"
#include "coarse_exact_core.hpp"
#include "p19_monster_gate.hpp"

#include <cstdint>
#include <cstring>

namespace {

// Terrain-stream generator index -> (Random seed multiplier, constructors to
// skip before it) following BetaTerrain173.java:84-91 and
// WorldChunkManager173.java:24-31, composed from the reference's p20 helpers.
void build_state(std::int64_t seed, int index, p20::PerlinState& st) {
    p20::JavaRandom rng;
    int skip;
    if (index < 66) {
        rng.setSeed(seed);
        skip = index < 40 ? index : index + 8;
    } else if (index < 70) {
        rng.setSeed(static_cast<std::int64_t>(static_cast<std::uint64_t>(seed) * 9871ULL));
        skip = index - 66;
    } else if (index < 74) {
        rng.setSeed(static_cast<std::int64_t>(static_cast<std::uint64_t>(seed) * 39811ULL));
        skip = index - 70;
    } else {
        rng.setSeed(static_cast<std::int64_t>(static_cast<std::uint64_t>(seed) * 543321ULL));
        skip = index - 74;
    }
    p20::PerlinState scratch;
    for (int i = 0; i < skip; ++i) p20::initPerlin(rng, scratch);
    p20::initPerlin(rng, st);
}

void to_state(const std::uint8_t* perm, const double* abc, p20::PerlinState& st) {
    for (int i = 0; i < 256; ++i) { st.perm[i] = perm[i]; st.perm[i + 256] = perm[i]; }
    st.a = abc[0]; st.b = abc[1]; st.c = abc[2];
}

}  // namespace

extern "C" {

int ref_world_state(std::int64_t seed, int index, std::uint8_t* perm256, double* abc3) {
    p20::PerlinState st;
    build_state(seed, index, st);
    for (int i = 0; i < 256; ++i) perm256[i] = static_cast<std::uint8_t>(st.perm[i]);
    abc3[0] = st.a; abc3[1] = st.b; abc3[2] = st.c;
    return 0;
}

double ref_perlin3(const std::uint8_t* perm, const double* abc, double x, double y, double z) {
    p20::PerlinState st; to_state(perm, abc, st);
    return p20::perlin3(st, x, y, z);
}

double ref_perlin2(const std::uint8_t* perm, const double* abc, double x, double z) {
    p20::PerlinState st; to_state(perm, abc, st);
    return p20::perlin2(st, x, z);
}

double ref_simplex2(const std::uint8_t* perm, const double* abc, double x, double z) {
    p20::PerlinState st; to_state(perm, abc, st);
    return p20::simplex2(st, x, z);
}

void ref_perlin3_full17(const std::uint8_t* perm, const double* abc, double xCoord, double yScale,
                        double zCoord, double* out17) {
    p20::PerlinState st; to_state(perm, abc, st);
    coarsecore::perlin3Full17(st, xCoord, yScale, zCoord, out17);
}

void ref_perlin3_upper6(const std::uint8_t* perm, const double* abc, double xCoord, double yScale,
                        double zCoord, double* out6) {
    p20::PerlinState st; to_state(perm, abc, st);
    p20::perlin3Upper6(st, xCoord, yScale, zCoord, out6);
}

int ref_coarse_score(std::int64_t seed, std::uint8_t* signsOut) {
    static thread_local coarsecore::HostScratch* scratch = nullptr;
    if (!scratch) scratch = new coarsecore::HostScratch();
    const int score = coarsecore::generateAndScoreHost(seed, *scratch);
    if (signsOut) std::memcpy(signsOut, scratch->signs.data(), coarsecore::CELLS);
    return score;
}

// The reference's coarse noise sums (generateAndScoreHost, coarse_exact_core.hpp:218-386)
// around centre (0,0): column c = x*61+z at coarse (-28+x, -28+z); n1..n3 [3721][17], n4/n5 [3721].
void ref_coarse_noise(std::int64_t seed, double* n1, double* n2, double* n3, double* n4, double* n5) {
    static thread_local coarsecore::HostScratch* scratch = nullptr;
    if (!scratch) scratch = new coarsecore::HostScratch();
    coarsecore::generateAndScoreHost(seed, *scratch);
    std::memcpy(n1, scratch->noise1.data(), sizeof(double) * coarsecore::CELLS);
    std::memcpy(n2, scratch->noise2.data(), sizeof(double) * coarsecore::CELLS);
    std::memcpy(n3, scratch->noise3.data(), sizeof(double) * coarsecore::CELLS);
    std::memcpy(n4, scratch->noise4.data(), sizeof(double) * coarsecore::COLUMNS);
    std::memcpy(n5, scratch->noise5.data(), sizeof(double) * coarsecore::COLUMNS);
}

// features[12] = fullY88, fullY96, fullY104, fullY112, y88Largest, y88Width,
// y88Depth, y88Touches, y96Largest, y96Width, y96Depth, y96Touches
static p19native::MonsterFeatures to_features(const int* f) {
    p19native::MonsterFeatures p;
    p.stage0FullY88 = f[0]; p.stage0FullY96 = f[1]; p.stage0FullY104 = f[2]; p.stage0FullY112 = f[3];
    p.stage0Y88LargestCluster = f[4]; p.stage0Y88Width = f[5]; p.stage0Y88Depth = f[6];
    p.stage0Y88TouchesBorder = f[7] != 0;
    p.stage0Y96LargestCluster = f[8]; p.stage0Y96Width = f[9]; p.stage0Y96Depth = f[10];
    p.stage0Y96TouchesBorder = f[11] != 0;
    return p;
}

double ref_p19_score(int scout, const int* features12) {
    return p19native::score(scout, to_features(features12));
}

int ref_p19_extreme(const int* features12) {
    return p19native::hasExtremeTopologySignal(to_features(features12)) ? 1 : 0;
}

std::uint64_t ref_splitmix(std::uint64_t sequenceSeed, std::uint64_t attempt) {
    return p20::splitMixDeterministicSeed(sequenceSeed, attempt);
}

}  // extern "C"
