"""GPU parity beyond the small cases: the chunk-bitmap workload at its stated
size, previews across radii 0..16, and regions whose side-border verification
widens the exact scan. Each against the CPU oracle, through the C ABI."""
import json
import os

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
RELAXED = dict(min_blocks=1, min_columns=1, min_y_for_match=0, min_width=1, min_depth=1, min_avg_thickness=0.0)
RELAXED_PO = dict(minBlocks=1, minColumns=1, minYForMatch=0, minWidth=1, minDepth=1, minAvgThickness=0.0)


def test_chunk_bitmaps_4096_consecutive_seeds():
    """4,096 consecutive world seeds from a seeded random 48-bit start, chunk (0,0):
    every 4 KiB stone bitmap and its hash equal the oracle's."""
    start = int(np.random.default_rng(4096).integers(0, 2 ** 48 - 4096))
    seeds = np.arange(start, start + 4096, dtype=np.int64)
    with bsf.Worker(capacity=4096, profile=bsf.PROFILE_GENERAL, centers=1, max_exact_radius=1) as w:
        bm, h = w.chunk_bitmaps(seeds, 0, 0)
    obm, oh = po.chunk_bitmaps(seeds, 0, 0)
    bad = np.flatnonzero((bm != obm).any(axis=1))
    assert bad.size == 0, bad[:10]
    assert np.array_equal(h, oh)
    # nearly every seed has terrain of its own (a few chunks are plain layers of
    # stone at the same height in several worlds, so their bitmaps coincide)
    assert len(set(h.tolist())) > 4000


PREVIEW_CASES = [(int(s), r) for s, r in zip(np.random.default_rng(77).integers(0, 2 ** 48, size=24),
                                             [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16,
                                              0, 2, 5, 8, 11, 14, 16])]


@pytest.fixture(scope="module")
def preview_worker():
    with bsf.Worker(capacity=16, profile=bsf.PROFILE_MEGA, centers=8, max_exact_radius=24) as w:
        yield w


@pytest.mark.parametrize("seed,radius", PREVIEW_CASES)
def test_preview_columns_match_oracle(preview_worker, seed, radius):
    """buildIsland3DData: the chosen component (relaxed match settings, so small
    components count) and its per-column lowest and highest stone."""
    isl, mn, mx = preview_worker.preview(seed, 0, 0, radius, bsf.default_match_settings(**RELAXED))
    o, omn, omx = po.preview(seed, 0, 0, radius, po.match_settings(**RELAXED_PO))
    assert isl.key() == o.key()
    if o.found:
        assert np.array_equal(mn, omn) and np.array_equal(mx, omx)


def _border_regions(n=10):
    """n fixture regions spread over the final radii the verification reached."""
    p = os.path.join(HERE, "golden", "border_regions.json")
    if not os.path.exists(p):
        return []
    regs = sorted(json.load(open(p))["regions"], key=lambda c: (c["final_radius"], c["seed"]))
    if len(regs) <= n:
        return regs
    return [regs[round(i * (len(regs) - 1) / (n - 1))] for i in range(n)]


BORDER = _border_regions()


@pytest.mark.skipif(not BORDER, reason="tests/golden/border_regions.json not generated")
@pytest.mark.parametrize("case", BORDER, ids=lambda c: "%d_%d_%d_r%d" % (c["seed"], c["center_chunk_x"],
                                                                      c["center_chunk_z"], c["final_radius"]))
def test_border_verification_matches_oracle(preview_worker, case):
    """processGpuRegionAttempt for regions whose island reaches the scan's side:
    verifySideBorderMatch widens the scan (radii 10, 13, 16, 20, 24), and the hot
    scan runs at 16 when coarse >= 120. The chosen island equals the oracle's."""
    g = preview_worker.resolve_region(case["seed"], case["center_chunk_x"], case["center_chunk_z"], 7,
                                      case["coarse"])
    o = po.resolve_region(case["seed"], case["center_chunk_x"], case["center_chunk_z"], 7, case["coarse"])
    assert g.key() == o.key()
    assert g.radius_used == case["final_radius"]
