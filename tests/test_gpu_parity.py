"""GPU parity: every output of the sm_103a path against the CPU oracle, bit for bit.

All calls go through the C ABI (libbsf.so via ctypes). Inputs are seeded.
"""
import numpy as np
import pytest

import betaseedfinder_gb300 as bsf
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

EDGE_SEEDS = [0, 1, -1, 2 ** 63 - 1, -2 ** 63, 123456789, -4172144997902289642, 2 ** 48 - 1, 2 ** 48]


def consecutive_seeds(n, salt):
    rng = np.random.default_rng(abs(salt))
    start = int(rng.integers(0, 2 ** 48 - n))
    return np.arange(start, start + n, dtype=np.int64)


@pytest.fixture(scope="module")
def worker():
    from betaseedfinder_gb300 import build
    build.build()
    w = bsf.Worker(capacity=4096, profile=bsf.PROFILE_MEGA, centers=8, max_exact_radius=24)
    yield w
    w.close()


def test_chunk_bitmaps_chunk00_match_oracle(worker):
    seeds = np.concatenate([consecutive_seeds(256, 1), np.array(EDGE_SEEDS, np.int64)])
    bm, h = worker.chunk_bitmaps(seeds, 0, 0)
    obm, oh = po.chunk_bitmaps(seeds, 0, 0)
    assert np.array_equal(bm, obm)
    assert np.array_equal(h, oh)
    assert bm.any(axis=1).all()  # every chunk has stone


@pytest.mark.parametrize("cx,cz", [(-3, 7), (100, -250), (-1, -1)])
def test_chunk_bitmaps_other_chunks_match_oracle(worker, cx, cz):
    seeds = consecutive_seeds(48, cx * 1000 + cz)
    bm, h = worker.chunk_bitmaps(seeds, cx, cz)
    obm, oh = po.chunk_bitmaps(seeds, cx, cz)
    assert np.array_equal(bm, obm) and np.array_equal(h, oh)


def test_p20_filter_matches_oracle(worker):
    seeds = np.concatenate([consecutive_seeds(300, 2), np.array(EDGE_SEEDS, np.int64)])
    got = worker.p20_filter(seeds)
    rec = po.stage0_batch(seeds, centers=1, profile=0, research=False).reshape(-1, 16)
    assert np.array_equal(got, rec[:, 0])


def test_stage0_records_mega_lean_match_oracle(worker):
    seeds = np.concatenate([consecutive_seeds(160, 3), np.array(EDGE_SEEDS, np.int64)])
    got = worker.stage0_filter(seeds)
    ref = po.stage0_batch(seeds, centers=8, profile=1, research=False)
    assert np.array_equal(got, ref), np.flatnonzero(got.reshape(-1, 16).any(1) != ref.reshape(-1, 16).any(1))[:10]


@pytest.mark.parametrize("profile", ["general", "record60"])
def test_stage0_records_research_match_oracle(profile):
    seeds = consecutive_seeds(96, 4 + len(profile))
    with bsf.Worker(capacity=256, profile=profile, research=True, centers=8, max_exact_radius=1) as w:
        got = w.stage0_filter(seeds)
    ref = po.stage0_batch(seeds, centers=8, profile=bsf.PROFILES[profile], research=True)
    assert np.array_equal(got.reshape(-1, 34), ref.reshape(-1, 34))


def test_stage0_single_centre_matches_oracle():
    """Centre (0,0), general profile, research records. The batch includes the
    worlds of tests/golden/stage0_reference.json, whose oracle records equal the
    values the reference's own sign grids imply (test_oracle_golden.py)."""
    import json
    import os
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "stage0_reference.json")))
    pinned = np.array([r["seed"] for r in fx["regions"]], dtype=np.int64)
    seeds = np.concatenate([consecutive_seeds(128, 5), pinned])
    with bsf.Worker(capacity=256, profile="general", research=True, centers=1, max_exact_radius=1) as w:
        got = w.stage0_filter(seeds)
    ref = po.stage0_batch(seeds, centers=1, profile=0, research=True)
    assert np.array_equal(got, ref)


RELAXED = dict(min_blocks=1, min_columns=1, min_y_for_match=0, min_width=1, min_depth=1, min_avg_thickness=0.0)


@pytest.mark.parametrize("seed,cx,cz,radius", [(123456789, 0, 0, 3), (-4172144997902289642, 15, -15, 2),
                                               (987654321, -15, 0, 4), (42, 0, 15, 1)])
def test_exact_scan_relaxed_matches_oracle(worker, seed, cx, cz, radius):
    g = worker.exact_scan(seed, cx, cz, radius, bsf.default_match_settings(**RELAXED))
    o = po.exact_scan(seed, cx, cz, radius, po.match_settings(minBlocks=1, minColumns=1, minYForMatch=0, minWidth=1,
                                                                minDepth=1, minAvgThickness=0.0))
    assert g.key() == o.key()
    assert (g.sum_x, g.sum_z) == (o.sumX, o.sumZ)


@pytest.mark.parametrize("seed", [2024, 77777])
def test_exact_scan_default_settings_r7_matches_oracle(worker, seed):
    g = worker.exact_scan(seed, 0, 0, 7)
    o = po.exact_scan(seed, 0, 0, 7)
    assert g.key() == o.key()


def test_preview_matches_oracle(worker):
    seed = 31337
    s = bsf.default_match_settings(**RELAXED)
    isl, mn, mx = worker.preview(seed, 0, 0, 3, s)
    o, omn, omx = po.preview(seed, 0, 0, 3, po.match_settings(minBlocks=1, minColumns=1, minYForMatch=0, minWidth=1,
                                                               minDepth=1, minAvgThickness=0.0))
    assert isl.key() == o.key()
    if o.found:
        assert np.array_equal(mn, omn) and np.array_equal(mx, omx)


def test_resolve_region_with_hot_scan_matches_oracle(worker):
    seed = 555
    g = worker.resolve_region(seed, 0, 0, 7, 130)
    o = po.resolve_region(seed, 0, 0, 7, 130)
    assert g.key() == o.key()


def test_rng_rejection_seeds_match_oracle(worker):
    """Worlds whose generator setup hits nextInt's rejection loop take the GPU's
    serial rebuild of the affected stream; their bitmaps and Stage0 records must
    still equal the oracle's (whose states are pinned to the reference's)."""
    import json
    import os
    rej = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "rng_rejection_seeds.json")))
    seeds = np.array(rej["seeds"], dtype=np.int64)
    bm, h = worker.chunk_bitmaps(seeds, 0, 0)
    obm, oh = po.chunk_bitmaps(seeds, 0, 0)
    assert np.array_equal(bm, obm) and np.array_equal(h, oh)
    with bsf.Worker(capacity=64, profile="mega", research=True, centers=8, max_exact_radius=24) as w:
        assert np.array_equal(w.stage0_filter(seeds), po.stage0_batch(seeds, centers=8, profile=1, research=True))
        counts, _ = w.mega_search(seeds)
    assert counts.rng_fallbacks >= len(seeds)   # every one of them took the fallback path


def test_mega_pipeline_counts_and_coarse_scores_match_oracle(worker):
    """The whole queued MEGA pipeline against the oracle's restatement: the stage
    counts of every gate (P20, Upper, High, P19, Mega, coarse evaluated / passed,
    islands), every coarse survivor's island, and the coarse score of coarse-
    evaluated regions, which the 34-byte region records carry."""
    seeds = consecutive_seeds(1024, 12)
    counts, recs = worker.mega_search(seeds)
    rr = worker.last_region_records(len(seeds)).reshape(-1, 34).astype(np.int64)
    oc, oisl, oreg = po.mega_pipeline(seeds, profile=1, radius=7)
    got = counts.as_dict()
    for ours, theirs in (("p20_passed", "p20Passed"), ("upper_passed", "upperPassed"),
                         ("high_passed", "highPassed"), ("p19_passed", "p19Passed"),
                         ("mega_rejected", "megaRejected"), ("coarse_evaluated", "coarseEvaluated"),
                         ("coarse_passed", "coarsePassed"), ("islands", "islands")):
        assert got[ours] == getattr(oc, theirs), ours
    ours = sorted((r.world_index * 8 + r.center_index, r.island.key()) for r in recs)
    assert ours == sorted((int(g), i.key()) for g, i in zip(oreg, oisl))
    # coarse-evaluated regions: P19 passed and not Mega-rejected
    evaluated = np.flatnonzero((rr[:, 3] != 0) & (rr[:, 7] == 0))
    assert len(evaluated) == got["coarse_evaluated"] and len(evaluated) > 0
    coarse = rr[:, 4] | (rr[:, 5] << 8)
    for g in evaluated[:24]:
        w, c = divmod(int(g), 8)
        assert coarse[g] == min(po.coarse_score(int(seeds[w]), bsf.CENTER_CHUNK_X[c], bsf.CENTER_CHUNK_Z[c]),
                                65535), (w, c)


@pytest.mark.parametrize("profile", ["general", "record60"])
def test_pipeline_counts_match_oracle_for_other_profiles(profile):
    """The queued pipeline under the general and record60 gates (P20/Upper/High/
    coarse thresholds of the worker's hunt profiles) against the oracle's pipeline
    with the same profile: every stage count and every coarse survivor's island."""
    seeds = consecutive_seeds(768, 40 + len(profile))
    with bsf.Worker(capacity=1024, profile=profile, centers=8, max_exact_radius=24) as w:
        counts, recs = w.mega_search(seeds)
        rr = w.last_region_records(len(seeds)).reshape(-1, 34).astype(np.int64)
    oc, oisl, oreg = po.mega_pipeline(seeds, profile=bsf.PROFILES[profile], radius=7)
    got = counts.as_dict()
    for ours, theirs in (("p20_passed", "p20Passed"), ("upper_passed", "upperPassed"),
                         ("high_passed", "highPassed"), ("p19_passed", "p19Passed"),
                         ("mega_rejected", "megaRejected"), ("coarse_evaluated", "coarseEvaluated"),
                         ("coarse_passed", "coarsePassed"), ("islands", "islands")):
        assert got[ours] == getattr(oc, theirs), (profile, ours)
    assert got["p20_passed"] > 0 and got["coarse_evaluated"] > 0
    ours = sorted((r.world_index * 8 + r.center_index, r.island.key()) for r in recs)
    assert ours == sorted((int(g), i.key()) for g, i in zip(oreg, oisl))
    coarse = rr[:, 4] | (rr[:, 5] << 8)
    for g in np.flatnonzero((rr[:, 3] != 0) & (rr[:, 7] == 0))[:8]:
        w_, c = divmod(int(g), 8)
        assert coarse[g] == po.coarse_score(int(seeds[w_]), bsf.CENTER_CHUNK_X[c], bsf.CENTER_CHUNK_Z[c])
