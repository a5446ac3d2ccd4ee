"""The screened FP32 kernels (default queued form) against the FP64 kernels
(plain form) on large batches: every stage0stream record must be identical.
This exercises the error bounds of bsf_screen.cuh on hundreds of thousands of
lattice columns; the FP64 kernels are themselves pinned to the oracle."""
import numpy as np
import pytest

import betaseedfinder_gb300 as bsf

pytestmark = pytest.mark.gpu


def consecutive(n, salt):
    start = int(np.random.default_rng(salt).integers(0, 2 ** 48 - n))
    return np.arange(start, start + n, dtype=np.int64)


@pytest.mark.parametrize("profile,n", [("mega", 8192), ("general", 4096), ("record80", 2048)])
def test_screened_stage0_records_equal_fp64(profile, n):
    seeds = consecutive(n, 100 + n)
    with bsf.Worker(capacity=n, profile=profile, research=True, centers=8, max_exact_radius=1) as w:
        fast = w.stage0_filter(seeds)
        w.set_mode(bsf.MODE_PLAIN)
        exact = w.stage0_filter(seeds)
    r_fast, r_exact = fast.reshape(-1, 34), exact.reshape(-1, 34)
    bad = np.flatnonzero((r_fast != r_exact).any(axis=1))
    assert bad.size == 0, "regions differ: %s" % bad[:20]
    # the batch must actually reach the late stages for this to mean something
    assert (r_exact[:, 3] > 0).sum() > 0


def test_screened_p20_equal_fp64():
    seeds = consecutive(16384, 7)
    with bsf.Worker(capacity=16384, profile="general", centers=1, max_exact_radius=1) as w:
        fast = w.p20_filter(seeds)
        w.set_mode(bsf.MODE_PLAIN)
        exact = w.p20_filter(seeds)
    assert np.array_equal(fast, exact)


def test_mega_search_forms_agree():
    seeds = consecutive(8192, 11)
    with bsf.Worker(capacity=8192, profile="mega", centers=8, max_exact_radius=24) as w:
        c1, r1 = w.mega_search(seeds)
        w.set_mode(bsf.MODE_PLAIN)
        c2, r2 = w.mega_search(seeds)
    d1, d2 = c1.as_dict(), c2.as_dict()
    d1.pop("rng_fallbacks"), d2.pop("rng_fallbacks")
    assert d1 == d2
    assert [(r.world_index, r.center_index, r.coarse, r.island.key()) for r in r1] == \
           [(r.world_index, r.center_index, r.coarse, r.island.key()) for r in r2]
