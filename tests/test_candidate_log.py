"""Candidate-log rows (hunter_candidates.csv) on CPU, for every status branch:
the worker's row writer (bsf_worker candrows, the code the hunt uses) against a
separate restatement of the reference's selection and row rules.

processGpuRegionAttempt (IslandSearchEngine.java:1878-1971) takes the normal
match (the scan at the search radius, already border-verified), runs the hot
scan when coarse >= 120, keeps the hot result only when compareComponents
(:4079-4094) says it is strictly better, and logs (normal, match, hotScanRan,
hot, duplicateMerged). appendCandidateCsv (:4836-4960) derives matched, status
and finalSource from those, comparing results by identity, and prints the row
with Java's %d/%s/%.nf formatting (%n = "\\n" on this platform)."""
import subprocess

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf
from betaseedfinder_gb300 import build as bsf_build

from test_boards import jfmt


@pytest.fixture(scope="module")
def worker():
    bsf_build.build()
    return bsf.WORKER_PATH


class Comp:
    """A MatchResult's component with the fields the row reads."""

    def __init__(self, rng, radius):
        self.blocks = int(rng.integers(1000, 1006))
        self.columns = int(rng.integers(100, 104))
        self.minX = int(rng.integers(-300, 300))
        self.maxX = self.minX + int(rng.integers(9, 13))
        self.minZ = int(rng.integers(-300, 300))
        self.maxZ = self.minZ + int(rng.integers(9, 13))
        self.minY = int(rng.integers(68, 80))
        self.maxY = self.minY + int(rng.integers(0, 30))
        self.centerX = (self.minX + self.maxX) // 2
        self.centerZ = (self.minZ + self.maxZ) // 2
        self.touches = bool(rng.integers(0, 2))
        self.radius = radius

    def ints(self):
        return [1, self.blocks, self.columns, self.minX, self.maxX, self.minZ, self.maxZ, self.minY, self.maxY,
                self.centerX, self.centerZ, int(self.touches), self.radius]


NONE = [0] * 13


def compare(a, b):  # compareComponents
    key = lambda c: (c.blocks, c.columns, (c.maxX - c.minX + 1) * (c.maxZ - c.minZ + 1))
    return (key(a) > key(b)) - (key(a) < key(b))


def java_row(attempt, seed, w, normal, match, hot_ran, hot, dup):
    """appendCandidateCsv, restated; `is` stands for Java's reference equality."""
    raw = normal
    final = match if match is not None else raw
    matched = match is not None and not dup
    final_is_hot = hot is not None and match is hot
    final_is_border = match is not None and normal is not None and match is not normal and not final_is_hot
    if dup:
        source = "duplicate_merged"
    elif final_is_hot:
        source = "hot_scan"
    elif final_is_border:
        source = "border_verify"
    elif match is not None:
        source = "raw"
    else:
        source = "none"
    if dup:
        status = "duplicate_region_merged"
    elif match is not None and final_is_hot and match.touches:
        status = "matched_hot_scan_still_touches_side"
    elif match is not None and final_is_hot:
        status = "matched_hot_scan"
    elif match is not None and match.touches:
        status = "matched_still_touches_side"
    elif match is not None:
        status = "matched"
    elif normal is not None:
        status = "border_rejected_or_invalid"
    elif hot_ran:
        status = "hot_scan_no_match"
    else:
        status = "no_match"
    b = lambda v: "true" if v else "false"
    f = final
    width = 0 if f is None else f.maxX - f.minX + 1
    depth = 0 if f is None else f.maxZ - f.minZ + 1
    area = width * depth
    fill = 0.0 if f is None else 100.0 * f.columns / max(1, area)
    thick = 0.0 if f is None else f.blocks / max(1, f.columns)
    g = lambda name: 0 if f is None else getattr(f, name)
    cells = [attempt, seed, w["high"], w["high"], w["coarse"], w["p20"], w["upper"], w["high"], b(w["p19Pass"]),
             jfmt(w["p19Score"], 6), b(w["p19Extreme"]), w["cx"], w["cz"], b(matched), status,
             0 if raw is None else raw.blocks, 0 if match is None else match.blocks,
             0 if normal is None else normal.radius, 0 if match is None else match.radius,
             b(raw is not None and raw.touches), b(match is not None and match.touches), g("columns"), width, depth,
             area, jfmt(fill, 4), jfmt(thick, 4), g("minY"), g("maxY"), g("centerX"), g("centerZ"), g("minX"),
             g("maxX"), g("minZ"), g("maxZ"), b(hot_ran), 0 if hot is None else hot.radius,
             0 if hot is None else hot.blocks, b(hot is not None and hot.touches), source]
    return ",".join(str(c) for c in cells)


def test_candidate_rows_follow_the_reference_rules(worker):
    rng = np.random.default_rng(4860)
    lines, want, statuses = [], [], set()
    for attempt in range(1, 601):
        seed = int(rng.integers(-2 ** 63, 2 ** 63 - 1))
        w = dict(p20=int(rng.integers(1, 64)), upper=int(rng.integers(1, 192)), high=int(rng.integers(1, 60)),
                 coarse=int(rng.integers(85, 200)), p19Pass=bool(rng.integers(0, 2)),
                 p19Score=float(rng.choice([4.02, 6.7, 5.0000005, 4.1234565, rng.uniform(4, 9)])),
                 p19Extreme=bool(rng.integers(0, 2)), cx=int(rng.integers(-15, 16)), cz=int(rng.integers(-15, 16)))
        normal = Comp(rng, int(rng.choice([7, 10, 13, 16, 20, 24]))) if rng.random() < 0.6 else None
        hot_ran = w["coarse"] >= 120
        hot = None
        if hot_ran and rng.random() < 0.7:
            hot = Comp(rng, int(rng.choice([16, 20, 24])))
            if normal is not None and rng.random() < 0.25:  # equal stats: the normal match stays
                hot.blocks, hot.columns = normal.blocks, normal.columns
                hot.minX, hot.maxX, hot.minZ, hot.maxZ = normal.minX, normal.maxX, normal.minZ, normal.maxZ
        match = normal
        if hot is not None and (match is None or compare(hot, match) > 0):
            match = hot
        dup = match is not None and rng.random() < 0.15
        source = 0 if match is None else (2 if match is hot else 1)
        rec = [attempt, seed, w["p20"], w["upper"], w["high"], w["coarse"], int(w["p19Pass"]), repr(w["p19Score"]),
               int(w["p19Extreme"]), w["cx"], w["cz"], int(dup), int(hot_ran), source]
        for c in (match, normal, hot):
            rec += NONE if c is None else c.ints()
        lines.append(" ".join(str(x) for x in rec))
        want.append(java_row(attempt, seed, w, normal, match, hot_ran, hot, dup))
        statuses.add(want[-1].split(",")[14])
    out = subprocess.run([worker, "candrows"], input="\n".join(lines) + "\n", capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 0, out.stderr
    got = out.stdout.splitlines()
    assert got[0].split(",")[0] == "attempt" and len(got[0].split(",")) == 40
    assert got[1:] == want
    # every status this path can produce; border_rejected_or_invalid needs a normal
    # match without a final one, which processGpuRegionAttempt never logs
    assert statuses == {"duplicate_region_merged", "matched_hot_scan_still_touches_side", "matched_hot_scan",
                        "matched_still_touches_side", "matched", "hot_scan_no_match", "no_match"}
