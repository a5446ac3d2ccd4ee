// Top-result boards of a hunt: the reference app's leaderboard and its two
// sideboards (IslandSearchEngine.java:4987-5226, 5340-5367), written as
// top_largest_results.txt (and its legacy mirror top_floating_results.txt),
// top_filled_footprint_results.txt, top_raw_footprint_results.txt and
// top_island_sideboards.csv.
//
// Each board is a java.util.PriorityQueue ordered by its "better" comparator
// (the head is the board's worst record): a record enters while the board holds
// fewer than `keep`, otherwise it replaces the head only when strictly better.
// Files list the board in the queue's array order stably sorted best first, so
// ties keep the heap's order; the heap below makes the same sift moves as
// PriorityQueue's offer / poll, so tied records come out in the same order.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace bsfhunt {

std::string java_fixed(double v, int prec);  // String.format(Locale.US, "%.<prec>f", v)

struct BoardRecord {  // ResultRecord (IslandSearchEngine.java:6592-6650)
    std::int64_t seed = 0;
    int blocks = 0, columns = 0, centerX = 0, centerZ = 0;
    int minWorldX = 0, maxWorldX = 0, minWorldZ = 0, maxWorldZ = 0, minY = 0, maxY = 0;
    int width = 0, depth = 0, footprintArea = 0;
    double fillPercent = 0.0, avgThickness = 0.0;
    int chunkRadiusUsed = 0;
    bool touchesSideBorder = false;
    std::string previewPath;
};

inline BoardRecord make_board_record(std::int64_t seed, int blocks, int columns, int centerX, int centerZ, int minX,
                                     int maxX, int minZ, int maxZ, int minY, int maxY, int radius, bool touches,
                                     const std::string& outdir) {
    BoardRecord r;
    r.seed = seed;
    r.blocks = blocks;
    r.columns = columns;
    r.centerX = centerX;
    r.centerZ = centerZ;
    r.minWorldX = minX;
    r.maxWorldX = maxX;
    r.minWorldZ = minZ;
    r.maxWorldZ = maxZ;
    r.minY = minY;
    r.maxY = maxY;
    r.width = maxX - minX + 1;
    r.depth = maxZ - minZ + 1;
    r.footprintArea = r.width * r.depth;
    r.fillPercent = 100.0 * columns / static_cast<double>(std::max(1, r.footprintArea));
    r.avgThickness = blocks / static_cast<double>(std::max(1, columns));
    r.chunkRadiusUsed = radius;
    r.touchesSideBorder = touches;
    // previewPathFor (:5363-5367): the run directory resolved with the file name
    r.previewPath = outdir + "/floating_seed_" + std::to_string(seed) + "_x" + std::to_string(centerX) + "_z" +
                    std::to_string(centerZ) + ".png";
    return r;
}

inline int cmp_int(int a, int b) { return a < b ? -1 : (a > b ? 1 : 0); }
inline int cmp_double(double a, double b) { return a < b ? -1 : (a > b ? 1 : 0); }  // no NaNs here

// compareLargestBetter / compareFilledFootprintBetter / compareRawFootprintBetter (:5020-5049)
inline int better_largest(const BoardRecord& a, const BoardRecord& b) {
    if (int c = cmp_int(a.blocks, b.blocks)) return c;
    if (int c = cmp_int(a.columns, b.columns)) return c;
    if (int c = cmp_int(a.footprintArea, b.footprintArea)) return c;
    return cmp_double(a.avgThickness, b.avgThickness);
}
inline int better_filled(const BoardRecord& a, const BoardRecord& b) {
    if (int c = cmp_int(a.columns, b.columns)) return c;
    if (int c = cmp_int(a.footprintArea, b.footprintArea)) return c;
    if (int c = cmp_int(a.blocks, b.blocks)) return c;
    return cmp_double(a.fillPercent, b.fillPercent);
}
inline int better_raw(const BoardRecord& a, const BoardRecord& b) {
    if (int c = cmp_int(a.footprintArea, b.footprintArea)) return c;
    if (int c = cmp_int(a.columns, b.columns)) return c;
    if (int c = cmp_int(a.blocks, b.blocks)) return c;
    return cmp_double(a.fillPercent, b.fillPercent);
}

class Board {
public:
    using Better = int (*)(const BoardRecord&, const BoardRecord&);
    Board(Better better, int keep) : better_(better), keep_(keep) {}

    // addToBoard (:5067-5085)
    bool add(const BoardRecord& r) {
        if (static_cast<int>(heap_.size()) < keep_) {
            offer(r);
            return true;
        }
        if (better_(r, heap_.front()) > 0) {
            poll();
            offer(r);
            return true;
        }
        return false;
    }

    // getSortedBoardLocked (:5058-5065): array order, stably sorted best first
    std::vector<BoardRecord> sorted() const {
        std::vector<BoardRecord> v = heap_;
        std::stable_sort(v.begin(), v.end(),
                         [this](const BoardRecord& a, const BoardRecord& b) { return better_(b, a) < 0; });
        return v;
    }
    bool empty() const { return heap_.empty(); }

private:
    // A binary min-heap under better_ (head = worst), with the JDK queue's
    // moves: offer sifts the new record up from the end while it is strictly
    // worse than its parent; poll moves the last record to the root and sifts it
    // down, taking the right child only when it is strictly worse than the left.
    void offer(const BoardRecord& r) {
        heap_.push_back(r);
        std::size_t k = heap_.size() - 1;
        const BoardRecord x = heap_[k];
        while (k > 0) {
            const std::size_t parent = (k - 1) >> 1;
            if (better_(x, heap_[parent]) >= 0) break;
            heap_[k] = heap_[parent];
            k = parent;
        }
        heap_[k] = x;
    }
    void poll() {
        const BoardRecord x = heap_.back();
        heap_.pop_back();
        if (heap_.empty()) return;
        const std::size_t n = heap_.size(), half = n >> 1;
        std::size_t k = 0;
        while (k < half) {
            std::size_t child = 2 * k + 1;
            const std::size_t right = child + 1;
            if (right < n && better_(heap_[child], heap_[right]) > 0) child = right;
            if (better_(x, heap_[child]) <= 0) break;
            heap_[k] = heap_[child];
            k = child;
        }
        heap_[k] = x;
    }

    Better better_;
    int keep_;
    std::vector<BoardRecord> heap_;
};

// buildBoardText + appendResultDetails (:5179-5217)
inline std::string board_text(const char* title, const char* sortDescription, const std::vector<BoardRecord>& sorted,
                              int keep) {
    std::string s = std::string(title) + "\n" + sortDescription + "\nKeeping top " + std::to_string(keep) + "\n\n";
    for (std::size_t i = 0; i < sorted.size(); ++i) {
        const BoardRecord& r = sorted[i];
        s += "#" + std::to_string(i + 1) + "\n";
        s += "seed=" + std::to_string(r.seed) + "\n";
        s += "blocks=" + std::to_string(r.blocks) + "\n";
        s += "chunkRadiusUsed=" + std::to_string(r.chunkRadiusUsed) + "\n";
        s += std::string("touchesSideBorder=") + (r.touchesSideBorder ? "true" : "false") + "\n";
        s += "columns=" + std::to_string(r.columns) + "\n";
        s += "filledFootprintColumns=" + std::to_string(r.columns) + "\n";
        s += "footprint=" + std::to_string(r.width) + "x" + std::to_string(r.depth) + "\n";
        s += "footprintArea=" + std::to_string(r.footprintArea) + "\n";
        s += "fillPercent=" + java_fixed(r.fillPercent, 2) + "\n";
        s += "avgThickness=" + java_fixed(r.avgThickness, 2) + "\n";
        s += "centerX=" + std::to_string(r.centerX) + "\n";
        s += "centerZ=" + std::to_string(r.centerZ) + "\n";
        s += "boundsX=" + std::to_string(r.minWorldX) + " to " + std::to_string(r.maxWorldX) + "\n";
        s += "boundsZ=" + std::to_string(r.minWorldZ) + " to " + std::to_string(r.maxWorldZ) + "\n";
        s += "yRange=" + std::to_string(r.minY) + " to " + std::to_string(r.maxY) + "\n";
        s += "preview=" + r.previewPath + "\n";
        s += "\n";
    }
    return s;
}

constexpr const char* kSideboardsHeader =
    "board,rank,seed,blocks,columns,width,depth,footprintArea,fillPercent,avgThickness,minY,maxY,centerX,centerZ,"
    "chunkRadiusUsed,touchesSideBorder\n";

// saveSideboardsCsvLocked + appendBoardCsv (:5219-5226, 5340-5361)
inline std::string sideboards_csv(const std::vector<BoardRecord>& largest, const std::vector<BoardRecord>& filled,
                                  const std::vector<BoardRecord>& raw) {
    std::string s = kSideboardsHeader;
    auto rows = [&s](const char* board, const std::vector<BoardRecord>& v) {
        for (std::size_t i = 0; i < v.size(); ++i) {
            const BoardRecord& r = v[i];
            s += std::string(board) + "," + std::to_string(i + 1) + "," + std::to_string(r.seed) + "," +
                 std::to_string(r.blocks) + "," + std::to_string(r.columns) + "," + std::to_string(r.width) + "," +
                 std::to_string(r.depth) + "," + std::to_string(r.footprintArea) + "," +
                 java_fixed(r.fillPercent, 4) + "," + java_fixed(r.avgThickness, 4) + "," + std::to_string(r.minY) +
                 "," + std::to_string(r.maxY) + "," + std::to_string(r.centerX) + "," + std::to_string(r.centerZ) +
                 "," + std::to_string(r.chunkRadiusUsed) + "," + (r.touchesSideBorder ? "true" : "false") + "\n";
        }
    };
    rows("largest", largest);
    rows("filled_footprint", filled);
    rows("raw_footprint", raw);
    return s;
}

// The three boards of a run and their files (initialised as the reference does
// at run start, :4262-4291, and rewritten with every board's final state).
struct Boards {
    explicit Boards(int keep)
        : keep(keep), largest(better_largest, keep), filled(better_filled, keep), raw(better_raw, keep) {}

    // recordTopResult + recordSideboardResults (:4987-5017, 5087-5117); true when
    // the largest board took the record (the reference counts these as topUpdates)
    bool add(const BoardRecord& r) {
        const bool top = largest.add(r);
        filled.add(r);
        raw.add(r);
        return top;
    }

    static void write_file(const std::string& path, const std::string& text) {
        std::FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) throw std::runtime_error("cannot write " + path);
        std::fwrite(text.data(), 1, text.size(), f);
        std::fclose(f);
    }

    void write(const std::string& outdir) const {
        const std::string largestText =
            largest.empty() ? std::string("Top largest floating islands\nNo results yet.\n")
                            : board_text("Top largest floating islands",
                                         "Sorted by blocks, then occupied columns, then footprint area, then thickness",
                                         largest.sorted(), keep);
        write_file(outdir + "/top_largest_results.txt", largestText);
        write_file(outdir + "/top_floating_results.txt", largestText);
        write_file(outdir + "/top_filled_footprint_results.txt",
                   filled.empty() ? std::string("Top filled-footprint floating islands\nNo results yet.\n")
                                  : board_text("Top filled-footprint floating islands",
                                               "Sorted by occupied X/Z columns. This is raw footprint area with fill "
                                               "ratio accounted for.",
                                               filled.sorted(), keep));
        write_file(outdir + "/top_raw_footprint_results.txt",
                   raw.empty() ? std::string("Top raw-footprint floating islands\nNo results yet.\n")
                               : board_text("Top raw-footprint floating islands",
                                            "Sorted by bounding-box footprint area. Fill percentage is shown so sparse "
                                            "boxes are obvious.",
                                            raw.sorted(), keep));
        write_file(outdir + "/top_island_sideboards.csv", sideboards_csv(largest.sorted(), filled.sorted(), raw.sorted()));
    }

    int keep;
    Board largest, filled, raw;
};

}  // namespace bsfhunt
