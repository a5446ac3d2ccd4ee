"""GPU: the screened exact scan (FP32 lattice and fill, the FP64 operations at
the cells the screen leaves open) against the all-FP64 scan, island for island.

Both run through the C ABI on one handle: screening on (the queued forms'
default) and off (bsf_set_screening(0), the FP64 kernels of the plain form).
The oracle pins the FP64 scan elsewhere (test_gpu_parity*.py); here every
field of every island and every preview column must agree: over many worlds,
centres and radii 0..24, with default and relaxed match settings, over the
island regions a MEGA search finds, and over the regions that force the
border ladder.
"""
import json
import os

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
RELAXED = dict(min_blocks=1, min_columns=1, min_y_for_match=0, min_width=1, min_depth=1, min_avg_thickness=0.0)
FIELDS = [f for f, _ in bsf.Island._fields_]


def fields(isl):
    return tuple(getattr(isl, f) for f in FIELDS)


@pytest.fixture(scope="module")
def worker():
    from betaseedfinder_gb300 import build
    build.build()
    w = bsf.Worker(capacity=32768, profile=bsf.PROFILE_MEGA, centers=8, max_exact_radius=24)
    yield w
    w.close()


def both(worker, fn):
    worker.set_screening(True)
    a = fn()
    worker.set_screening(False)
    try:
        b = fn()
    finally:
        worker.set_screening(True)
    return a, b


def scan_cases(n, salt):
    rng = np.random.default_rng(salt)
    offsets = [(0, 0), (15, 0), (0, 15), (15, 15), (-15, 0), (-15, 15), (0, -15), (15, -15)]
    out = []
    for _ in range(n):
        seed = int(rng.integers(-2 ** 63, 2 ** 63 - 1))
        cx, cz = offsets[int(rng.integers(0, 8))]
        radius = int(rng.choice([0, 1, 2, 3, 5, 7, 7, 7, 10, 13, 16]))
        out.append((seed, cx, cz, radius))
    return out


@pytest.mark.parametrize("relaxed", [False, True])
def test_screened_exact_scans_equal_fp64(worker, relaxed):
    settings = bsf.default_match_settings(**RELAXED) if relaxed else None
    for seed, cx, cz, r in scan_cases(48, 7 + relaxed):
        a, b = both(worker, lambda: worker.exact_scan(seed, cx, cz, r, settings))
        assert fields(a) == fields(b), (seed, cx, cz, r)


def test_screened_scans_of_island_regions_equal_fp64(worker):
    # regions that hold islands: the coarse survivors of a MEGA search over
    # 32,768 consecutive seeds, scanned again at several radii
    rng = np.random.default_rng(5)
    start = int(rng.integers(0, 2 ** 48 - 32768))
    _, recs = worker.mega_search(np.arange(start, start + 32768, dtype=np.int64))
    regions = [(r.seed, r.center_chunk_x, r.center_chunk_z) for r in recs if r.island.found]
    assert len(regions) >= 5
    for seed, cx, cz in regions:
        for r in (3, 7, 10, 16):
            a, b = both(worker, lambda: worker.exact_scan(seed, cx, cz, r))
            assert fields(a) == fields(b), (seed, cx, cz, r)
        a, b = both(worker, lambda: worker.exact_scan(seed, cx, cz, 7, bsf.default_match_settings(**RELAXED)))
        assert fields(a) == fields(b), (seed, cx, cz)


def test_mega_search_records_equal_fp64(worker):
    # the whole pipeline's island records, screened exact stage against FP64
    rng = np.random.default_rng(11)
    start = int(rng.integers(0, 2 ** 48 - 16384))
    seeds = np.arange(start, start + 16384, dtype=np.int64)
    (ca, ra), (cb, rb) = both(worker, lambda: worker.mega_search(seeds))
    assert ca.as_dict()["islands"] == cb.as_dict()["islands"]
    assert [bytes(x) for x in ra] == [bytes(x) for x in rb]


def test_screened_large_radii_equal_fp64(worker):
    for seed, cx, cz in [(103355891253904, 15, 0), (-4172144997902289642, 0, 0), (2 ** 48 - 1, -15, 15)]:
        for r in (20, 24):
            a, b = both(worker, lambda: worker.exact_scan(seed, cx, cz, r, bsf.default_match_settings(**RELAXED)))
            assert fields(a) == fields(b), (seed, r)


def test_screened_border_ladder_regions_equal_fp64(worker):
    with open(os.path.join(HERE, "golden", "border_regions.json")) as f:
        regions = json.load(f)["regions"]
    for c in regions:
        a, b = both(worker, lambda: worker.resolve_region(c["seed"], c["center_chunk_x"], c["center_chunk_z"], 7,
                                                          c["coarse"]))
        assert fields(a) == fields(b), c


def test_screened_previews_equal_fp64(worker):
    for seed, cx, cz, r in scan_cases(12, 99):
        a, b = both(worker, lambda: worker.preview(seed, cx, cz, r, bsf.default_match_settings(**RELAXED)))
        assert fields(a[0]) == fields(b[0]), (seed, r)
        if a[0].found:
            assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), (seed, r)
