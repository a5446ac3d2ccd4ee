#!/usr/bin/env python3
"""Generate tests/golden/stage0_reference.json: Stage0 region values for centre
(0,0) computed from the reference's own coarse sign grids.

The reference's Stage0 scout samples the 16x16 lattice at coarse coordinates
-28 + 4i (radius 7, step 4; BetaTerrain173.java:1542-1546) with climate at
block 4c+2 (:2538-2540), and evaluates the same full 17-level density there as
the coarse grid (coarse_exact_core.hpp:74-81, from -28, climate 4c+2). So Stage0
sample (i, k) is point (4i, 4k) of coarsecore::generateAndScoreHost's 61x61x17
sign grid. From those reference signs this script derives:
- p20: the 8x8 P20 axis columns {0,2,5,7,8,10,13,15} with a positive level in
  11..16 (BetaTerrain173.java:1801-1809, mask bits 11..16 at :1574);
- upper: all 256 columns with a positive level in 11..16;
- the highest re-entry level of each upper-positive column
  (highestSparseReentryYIndex, BetaTerrain173.java:2490-2504) and high, the
  columns whose highest re-entry is >= 11;
- the P19 features (buildMonsterFeatures / fillMonsterShapeStats,
  gpu_p20_benchmark.cpp:1022-1114);
- the P19 score and extreme flag from the reference's p19native code on those
  features, with upper as the scout count (gpu_p20_benchmark.cpp:7477-7480).

Runs where the reference checkout exists (oracle/_ref is built from it).
"""
import ctypes
import json
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "stage0_reference.json")
P20_AXIS = (0, 2, 5, 7, 8, 10, 13, 15)


def highest_reentry(levels):
    """Highest level that is positive after an earlier positive run and a gap (-1: none)."""
    saw_pos = saw_gap = False
    highest = -1
    for y, pos in enumerate(levels):
        if pos:
            if saw_pos and saw_gap:
                highest = y
            saw_pos = True
        elif saw_pos:
            saw_gap = True
    return highest


def shape_stats(grid):
    """Largest 4-connected cluster; bounding box and border contact of all set cells."""
    cells = {(x, z) for x in range(16) for z in range(16) if grid[x][z]}
    if not cells:
        return [0, 0, 0, 0]
    largest, seen = 0, set()
    for start in cells:
        if start in seen:
            continue
        seen.add(start)
        stack, size = [start], 0
        while stack:
            x, z = stack.pop()
            size += 1
            for n in ((x - 1, z), (x + 1, z), (x, z - 1), (x, z + 1)):
                if n in cells and n not in seen:
                    seen.add(n)
                    stack.append(n)
        largest = max(largest, size)
    xs = [c[0] for c in cells]
    zs = [c[1] for c in cells]
    touches = any(x in (0, 15) or z in (0, 15) for x, z in cells)
    return [largest, max(xs) - min(xs) + 1, max(zs) - min(zs) + 1, int(touches)]


def stage0_from_signs(R, seed):
    signs = np.zeros(61 * 61 * 17, np.uint8)
    R.ref_coarse_score(seed, signs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    grid = signs.reshape(61, 61, 17)
    cols = [[grid[4 * i, 4 * k] for k in range(16)] for i in range(16)]
    upper_pos = [[bool(cols[i][k][11:].any()) for k in range(16)] for i in range(16)]
    p20 = sum(upper_pos[i][k] for i in P20_AXIS for k in P20_AXIS)
    upper = sum(upper_pos[i][k] for i in range(16) for k in range(16))
    highest = [[highest_reentry(cols[i][k]) if upper_pos[i][k] else -1 for k in range(16)] for i in range(16)]
    flat = [h for row in highest for h in row]
    high = sum(h >= 11 for h in flat)
    full = [sum(h >= t for h in flat) for t in (11, 12, 13, 14)]
    y88 = [[highest[i][k] >= 11 for k in range(16)] for i in range(16)]
    y96 = [[highest[i][k] >= 12 for k in range(16)] for i in range(16)]
    features = full + shape_stats(y88) + shape_stats(y96)
    f = np.asarray(features, np.int32)
    score = R.ref_p19_score(upper, f.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    extreme = R.ref_p19_extreme(f.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return {"seed": int(seed), "p20": p20, "upper": upper, "high": high, "features": features,
            "p19_score_bits": format(int(np.float64(score).view(np.uint64)), "016x"), "p19_extreme": int(extreme != 0)}


def main():
    if po.build_ref() is None:
        raise SystemExit("reference checkout not available; cannot regenerate")
    R = po.ref()
    seq = 20261203
    as_i64 = lambda u: int(np.uint64(u).view(np.int64))
    regions = [stage0_from_signs(R, as_i64(R.ref_splitmix(seq, a))) for a in range(1, 25)]
    # more worlds whose centre-(0,0) region reaches the P19 gate (high >= 5), found by scanning
    a, gated = 25, 0
    while gated < 12:
        r = stage0_from_signs(R, as_i64(R.ref_splitmix(seq, a)))
        a += 1
        if r["p20"] >= 1 and r["upper"] >= 5 and r["high"] >= 5:
            regions.append(r)
            gated += 1
    # centre-(0,0) regions with high coarse scores (tests/golden/high_coarse_regions.json)
    for seed in (31415940913, 31415927080, 31415946975):
        regions.append(stage0_from_signs(R, seed))
    out = {"generator": "tests/golden/make_stage0_golden.py",
           "source": "reference coarsecore::generateAndScoreHost signs and p19native score, centre (0,0)",
           "features_order": "fullY88 fullY96 fullY104 fullY112 y88Largest y88Width y88Depth y88Touches "
                             "y96Largest y96Width y96Depth y96Touches",
           "regions": regions}
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", OUT, len(regions), "regions;", sum(r["high"] >= 5 for r in regions), "reach P19")


if __name__ == "__main__":
    main()
