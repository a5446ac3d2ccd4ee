"""Hunt result boards (bsf_worker boards / hunt): the leaderboard and the two
sideboards of IslandSearchEngine.java:4987-5226 and 5340-5367, checked on CPU
against a separate restatement of the same rules: java.util.PriorityQueue
offer/poll moves (head = worst record), a stable best-first sort of the queue's
array, and the board file formats."""
import os
import subprocess
from decimal import ROUND_HALF_UP, Decimal

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf
from betaseedfinder_gb300 import build as bsf_build


@pytest.fixture(scope="module")
def worker():
    bsf_build.build()
    return bsf.WORKER_PATH


def jfmt(v, prec):  # String.format(Locale.US, "%.<prec>f"): shortest digits, half-up
    return str(Decimal(repr(v)).quantize(Decimal(1).scaleb(-prec), rounding=ROUND_HALF_UP))


def record(seed, blocks, columns, cx, cz, minx, maxx, minz, maxz, miny, maxy, radius, touches, outdir):
    w, d = maxx - minx + 1, maxz - minz + 1
    area = w * d
    return dict(seed=seed, blocks=blocks, columns=columns, cx=cx, cz=cz, minx=minx, maxx=maxx, minz=minz, maxz=maxz,
                miny=miny, maxy=maxy, w=w, d=d, area=area, fill=100.0 * columns / max(1, area),
                thick=blocks / max(1, columns), radius=radius, touches=touches,
                preview="%s/floating_seed_%d_x%d_z%d.png" % (outdir, seed, cx, cz))


def cmp(a, b):
    return (a > b) - (a < b)


def largest(a, b):
    return cmp((a["blocks"], a["columns"], a["area"], a["thick"]), (b["blocks"], b["columns"], b["area"], b["thick"]))


def filled(a, b):
    return cmp((a["columns"], a["area"], a["blocks"], a["fill"]), (b["columns"], b["area"], b["blocks"], b["fill"]))


def raw(a, b):
    return cmp((a["area"], a["columns"], a["blocks"], a["fill"]), (b["area"], b["columns"], b["blocks"], b["fill"]))


class JavaQueue:
    """PriorityQueue with a comparator: binary heap, sift-up on offer, last-to-root
    sift-down on poll (the right child only when strictly smaller)."""

    def __init__(self, c):
        self.c, self.q = c, []

    def offer(self, x):
        q, k = self.q, len(self.q)
        q.append(x)
        while k > 0:
            p = (k - 1) >> 1
            if self.c(x, q[p]) >= 0:
                break
            q[k] = q[p]
            k = p
        q[k] = x

    def poll(self):
        q = self.q
        x = q.pop()
        if not q:
            return
        n, k = len(q), 0
        while k < n >> 1:
            ch = 2 * k + 1
            if ch + 1 < n and self.c(q[ch], q[ch + 1]) > 0:
                ch += 1
            if self.c(x, q[ch]) <= 0:
                break
            q[k] = q[ch]
            k = ch
        q[k] = x

    def add(self, r, keep):
        if len(self.q) < keep:
            self.offer(r)
        elif self.c(r, self.q[0]) > 0:
            self.poll()
            self.offer(r)

    def sorted(self):
        import functools
        return sorted(self.q, key=functools.cmp_to_key(lambda a, b: self.c(b, a)))  # stable


def text(title, desc, rows, keep):
    if not rows:
        return "%s\nNo results yet.\n" % title
    s = "%s\n%s\nKeeping top %d\n\n" % (title, desc, keep)
    for i, r in enumerate(rows):
        s += ("#%d\nseed=%d\nblocks=%d\nchunkRadiusUsed=%d\ntouchesSideBorder=%s\ncolumns=%d\n"
              "filledFootprintColumns=%d\nfootprint=%dx%d\nfootprintArea=%d\nfillPercent=%s\navgThickness=%s\n"
              "centerX=%d\ncenterZ=%d\nboundsX=%d to %d\nboundsZ=%d to %d\nyRange=%d to %d\npreview=%s\n\n") % (
            i + 1, r["seed"], r["blocks"], r["radius"], "true" if r["touches"] else "false", r["columns"],
            r["columns"], r["w"], r["d"], r["area"], jfmt(r["fill"], 2), jfmt(r["thick"], 2), r["cx"], r["cz"],
            r["minx"], r["maxx"], r["minz"], r["maxz"], r["miny"], r["maxy"], r["preview"])
    return s


def csv_text(boards):
    s = ("board,rank,seed,blocks,columns,width,depth,footprintArea,fillPercent,avgThickness,minY,maxY,centerX,"
         "centerZ,chunkRadiusUsed,touchesSideBorder\n")
    for name, rows in boards:
        for i, r in enumerate(rows):
            s += "%s,%d,%d,%d,%d,%d,%d,%d,%s,%s,%d,%d,%d,%d,%d,%s\n" % (
                name, i + 1, r["seed"], r["blocks"], r["columns"], r["w"], r["d"], r["area"], jfmt(r["fill"], 4),
                jfmt(r["thick"], 4), r["miny"], r["maxy"], r["cx"], r["cz"], r["radius"],
                "true" if r["touches"] else "false")
    return s


@pytest.mark.parametrize("keep,n", [(7, 300), (50, 20), (1, 40)])
def test_boards_follow_the_reference_queue_and_formats(worker, tmp_path, keep, n):
    rng = np.random.default_rng(keep * 1000 + n)
    outdir = str(tmp_path)
    lines, recs = [], []
    for i in range(n):
        # small ranges, so that many records tie on every key
        minx, minz = int(rng.integers(-500, 500)), int(rng.integers(-500, 500))
        w, d = int(rng.integers(10, 14)), int(rng.integers(10, 14))
        cols = int(rng.integers(100, 104))
        blocks = int(rng.integers(1000, 1004))
        v = (int(rng.integers(-2 ** 40, 2 ** 40)), blocks, cols, minx + w // 2, minz + d // 2, minx, minx + w - 1, minz,
             minz + d - 1, int(rng.integers(60, 80)), int(rng.integers(80, 100)), int(rng.integers(7, 25)),
             int(rng.integers(0, 2)))
        lines.append(" ".join(str(x) for x in v))
        recs.append(record(*v, outdir))
    out = subprocess.run([worker, "boards", str(keep), outdir], input="\n".join(lines) + "\n", capture_output=True,
                         text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    qs = [JavaQueue(largest), JavaQueue(filled), JavaQueue(raw)]
    for r in recs:
        for q in qs:
            q.add(r, keep)
    L, F, R = (q.sorted() for q in qs)
    read = lambda name: open(os.path.join(outdir, name)).read()
    big = text("Top largest floating islands",
               "Sorted by blocks, then occupied columns, then footprint area, then thickness", L, keep)
    assert read("top_largest_results.txt") == big and read("top_floating_results.txt") == big
    assert read("top_filled_footprint_results.txt") == text(
        "Top filled-footprint floating islands",
        "Sorted by occupied X/Z columns. This is raw footprint area with fill ratio accounted for.", F, keep)
    assert read("top_raw_footprint_results.txt") == text(
        "Top raw-footprint floating islands",
        "Sorted by bounding-box footprint area. Fill percentage is shown so sparse boxes are obvious.", R, keep)
    assert read("top_island_sideboards.csv") == csv_text([("largest", L), ("filled_footprint", F),
                                                          ("raw_footprint", R)])


def test_empty_boards_say_no_results(worker, tmp_path):
    out = subprocess.run([worker, "boards", "50", str(tmp_path)], input="", capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert open(tmp_path / "top_largest_results.txt").read() == "Top largest floating islands\nNo results yet.\n"
    assert open(tmp_path / "top_island_sideboards.csv").read().count("\n") == 1
