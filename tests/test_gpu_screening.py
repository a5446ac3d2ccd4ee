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
    """Queued (screened kernels, device queues, graphs), plain on the screened
    kernels, and plain on the FP64 kernels: the same stage counts, region records
    and islands."""
    seeds = consecutive(8192, 11)
    with bsf.Worker(capacity=8192, profile="mega", centers=8, max_exact_radius=24) as w:
        c1, r1 = w.mega_search(seeds)
        g1 = w.last_region_records(8192)
        w.set_mode(bsf.MODE_PLAIN_SCREENED)
        c3, r3 = w.mega_search(seeds)
        g3 = w.last_region_records(8192)
        w.set_mode(bsf.MODE_PLAIN)
        c2, r2 = w.mega_search(seeds)
    d1, d2, d3 = c1.as_dict(), c2.as_dict(), c3.as_dict()
    for k in ("rng_fallbacks", "screened_tasks", "fallback_tasks"):  # instrumentation, not results
        d1.pop(k), d2.pop(k), d3.pop(k)
    assert d1 == d2 == d3
    assert np.array_equal(g1, g3)
    assert c3.screened_tasks == c1.screened_tasks  # the same screened kernels ran
    assert [(r.world_index, r.center_index, r.coarse, r.island.key()) for r in r3] == \
           [(r.world_index, r.center_index, r.coarse, r.island.key()) for r in r1]
    # the screening must decide the vast majority of columns without FP64
    assert c1.screened_tasks > 0 and c1.fallback_tasks < 0.01 * c1.screened_tasks
    assert [(r.world_index, r.center_index, r.coarse, r.island.key()) for r in r1] == \
           [(r.world_index, r.center_index, r.coarse, r.island.key()) for r in r2]


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_every_launch_variant_gives_identical_records(variant):
    """Every Stage0 and coarse launch shape, on both grid shapes, against the FP64
    form."""
    seeds = consecutive(2049, 300 + variant)  # odd: the last pass holds one world
    with bsf.Worker(capacity=2049, profile="general", research=True, centers=8, max_exact_radius=1) as w:
        w.set_mode(bsf.MODE_PLAIN)
        exact = w.stage0_filter(seeds)
        w.set_mode(bsf.MODE_QUEUED)
        w.set_launch_variants(variant, variant)
        for persistent in (True, False):
            w.set_persistent(persistent)
            fast = w.stage0_filter(seeds)
            assert np.array_equal(fast, exact), (variant, persistent)
        w.set_launch_variants(0, 0)


def test_autotune_reports_and_keeps_results_exact():
    seeds = consecutive(2048, 404)
    with bsf.Worker(capacity=2048, profile="mega", research=True, centers=8, max_exact_radius=1) as w:
        report = w.autotune(1024)
        assert "stage0:" in report and "coarse:" in report and "->" in report
        fast = w.stage0_filter(seeds)
        w.set_mode(bsf.MODE_PLAIN)
        exact = w.stage0_filter(seeds)
    assert np.array_equal(fast, exact)


def test_batch_graph_replays_match_first_capture():
    """The queued mega batch runs as a cached CUDA graph keyed by batch size and
    seed source: replays, other sizes and device-resident seeds agree with the
    plain (uncaptured) form."""
    torch = pytest.importorskip("torch")
    seeds = consecutive(4096, 515)
    with bsf.Worker(capacity=4096, profile="mega", centers=8, max_exact_radius=24) as w:
        runs = []
        for n in (4096, 1000, 4096, 1000):
            before = w.kernel_launches
            c, r = w.mega_search(seeds[:n])
            runs.append((c.as_dict(), [(x.world_index, x.center_index, x.coarse, x.island.key()) for x in r]))
            # one graph replay = six kernels, plus the exact stage's own launches
            assert w.kernel_launches - before >= 6
        dev = torch.from_numpy(seeds).cuda()
        torch.cuda.synchronize()
        cd, rd = w.mega_search_device(dev.data_ptr(), len(seeds))
        w.set_mode(bsf.MODE_PLAIN)
        cp, rp = w.mega_search(seeds)
    assert runs[0] == runs[2] and runs[1] == runs[3]
    strip = lambda d: {k: v for k, v in d.items() if k not in ("rng_fallbacks", "screened_tasks", "fallback_tasks")}
    assert strip(runs[0][0]) == strip(cp.as_dict()) == strip(cd.as_dict())
    key = lambda rs: [(x.world_index, x.center_index, x.coarse, x.island.key()) for x in rs]
    assert runs[0][1] == key(rp) == key(rd)


def test_per_world_grids_give_identical_results():
    """bsf_set_persistent(0) (one CTA per world / half-region, used by served
    range lanes) changes only the launch shape."""
    seeds = consecutive(4096, 616)
    with bsf.Worker(capacity=4096, profile="mega", research=True, centers=8, max_exact_radius=24) as w:
        a = w.stage0_filter(seeds)
        ca, ra = w.mega_search(seeds)
        w.set_persistent(False)
        b = w.stage0_filter(seeds)
        cb, rb = w.mega_search(seeds)
    assert np.array_equal(a, b)
    assert ca.as_dict() == cb.as_dict()
    assert [(x.world_index, x.center_index, x.coarse, x.island.key()) for x in ra] == \
           [(x.world_index, x.center_index, x.coarse, x.island.key()) for x in rb]


def test_exact_fallback_paths_alone_match_fp64():
    """Screening off: every column task goes down the fallback path (the warp
    resolves each undecided column inline with the warp-cooperative FP64
    column) and must give the FP64 kernels' records and MEGA results."""
    seeds = consecutive(1024, 888)
    with bsf.Worker(capacity=1024, profile="mega", research=True, centers=8, max_exact_radius=24) as w:
        w.set_mode(bsf.MODE_PLAIN)
        exact = w.stage0_filter(seeds)
        cp, rp = w.mega_search(seeds)
        w.set_mode(bsf.MODE_QUEUED)
        w.set_screening(False)
        forced = w.stage0_filter(seeds)
        cf, rf = w.mega_search(seeds)
        w.set_screening(True)
    assert np.array_equal(forced, exact)
    strip = lambda c: {k: v for k, v in c.as_dict().items() if k not in ("rng_fallbacks", "screened_tasks", "fallback_tasks")}
    assert strip(cf) == strip(cp)
    assert cf.fallback_tasks == cf.screened_tasks > 0
    assert [(x.world_index, x.center_index, x.coarse, x.island.key()) for x in rf] == \
           [(x.world_index, x.center_index, x.coarse, x.island.key()) for x in rp]


def test_device_seed_records_carry_their_seeds_in_every_form():
    """bsf_mega_search_device in the three forms: each record's seed is the seed at
    its world index (gathered on the device with the region's outcome), and the
    records equal those of bsf_mega_search on the same seeds from host memory."""
    torch = pytest.importorskip("torch")
    seeds = consecutive(8192, 12)
    d = torch.from_numpy(seeds).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    with bsf.Worker(capacity=8192, profile="mega", centers=8, max_exact_radius=24) as w:
        _, host = w.mega_search(seeds)
        want = [(r.seed, r.world_index, r.center_index, r.coarse, r.island.key()) for r in host]
        assert want, "the batch reaches the exact stage"
        for mode in (bsf.MODE_QUEUED, bsf.MODE_PLAIN_SCREENED, bsf.MODE_PLAIN):
            w.set_mode(mode)
            _, recs = w.mega_search_device(d.data_ptr(), len(seeds), stream=stream)
            got = [(r.seed, r.world_index, r.center_index, r.coarse, r.island.key()) for r in recs]
            assert got == want, mode
            assert all(r.seed == seeds[r.world_index] for r in recs)


def test_pipelined_range_equals_batch_calls():
    """bsf_mega_search_range(_device): 3.25 batches pipelined over the handle and its
    twin give the records (world index counted from the range start) and summed
    stage counts of one bsf_mega_search call per batch."""
    torch = pytest.importorskip("torch")
    cap = 4096
    seeds = consecutive(cap * 3 + cap // 4, 21)
    with bsf.Worker(capacity=cap, profile="mega", centers=8, max_exact_radius=24) as w:
        want, wc = [], None
        for off in range(0, len(seeds), cap):
            c, r = w.mega_search(seeds[off:off + cap])
            want += [(x.seed, x.world_index + off, x.center_index, x.coarse, x.island.key()) for x in r]
            d = c.as_dict()
            wc = d if wc is None else {k: wc[k] + d[k] for k in d}
        single = w.footprint
        c1, r1 = w.mega_search_range(seeds)
        assert w.footprint == 2 * single  # the twin holds the same buffers
        d = torch.from_numpy(seeds).cuda()
        c2, r2 = w.mega_search_range_device(d.data_ptr(), len(seeds), stream=torch.cuda.current_stream().cuda_stream)
    assert want, "the range reaches the exact stage"
    for c, r in ((c1, r1), (c2, r2)):
        assert [(x.seed, x.world_index, x.center_index, x.coarse, x.island.key()) for x in r] == want
        got = c.as_dict()
        for k in ("rng_fallbacks", "screened_tasks", "fallback_tasks"):
            got.pop(k), wc.pop(k, None)
        assert got == {k: v for k, v in wc.items() if k in got}
    assert all(x.seed == seeds[x.world_index] for x in r1)
