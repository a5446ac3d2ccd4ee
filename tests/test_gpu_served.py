"""Served mode (bsf_server_*): every result is the same whether a request runs
alone or mixed with others on the device, and equal to the direct handle calls;
admission keeps the lanes' device memory inside the HBM budget."""
import numpy as np
import pytest

import betaseedfinder_gb300 as bsf

pytestmark = pytest.mark.gpu

INSTRUMENTATION = ("rng_fallbacks", "screened_tasks", "fallback_tasks")


def consecutive(n, salt):
    start = int(np.random.default_rng(salt).integers(0, 2 ** 48 - n))
    return np.arange(start, start + n, dtype=np.int64)


def rec_key(records):
    return [(r.seed, r.world_index, r.center_index, r.p20, r.upper, r.high, r.coarse, r.p19_score, r.island.key())
            for r in records]


def counts_key(c):
    d = c.as_dict()
    for k in INSTRUMENTATION:
        d.pop(k)
    return d


@pytest.fixture(scope="module")
def workload():
    ranges = [consecutive(12288, 901), consecutive(6000, 902)]
    direct, targets = [], []
    with bsf.Worker(capacity=12288, profile="mega", centers=8, max_exact_radius=24) as w:
        for seeds in ranges:
            c, r = w.mega_search(seeds)
            direct.append((counts_key(c), rec_key(r)))
            targets += [(x.seed, x.center_chunk_x, x.center_chunk_z) for x in r]
    # previews: regions that reached the exact stage (islands or near misses), plus plain centres
    targets = targets[:4] + [(int(ranges[0][7]), 0, 0), (int(ranges[1][3]), 15, -15)]
    previews = []
    with bsf.Worker(capacity=1, profile="mega", centers=1, max_exact_radius=16) as w:
        for seed, cx, cz in targets:
            for radius in (7, 12):
                isl, mn, mx = w.preview(seed, cx, cz, radius)
                previews.append(((seed, cx, cz, radius), isl.key(),
                                 None if mn is None else (mn.tolist(), mx.tolist())))
    return ranges, direct, previews


def served_results(server, ranges, previews, interleave):
    tickets = []
    if interleave:  # everything in flight at once, previews arriving between range requests
        half = len(previews) // 2
        tickets.append(("r", 0, server.submit_range(ranges[0])))
        for i, (args, _, _) in enumerate(previews[:half]):
            tickets.append(("p", i, server.submit_preview(*args)))
        tickets.append(("r", 1, server.submit_range(ranges[1])))
        for i, (args, _, _) in enumerate(previews[half:], start=half):
            tickets.append(("p", i, server.submit_preview(*args)))
        pending = tickets
    else:  # one request at a time
        pending = []
        for i, seeds in enumerate(ranges):
            t = server.submit_range(seeds)
            server.wait(t, 120)
            pending.append(("r", i, t))
        for i, (args, _, _) in enumerate(previews):
            t = server.submit_preview(*args)
            server.wait(t, 120)
            pending.append(("p", i, t))
    out_r, out_p = {}, {}
    for kind, i, t in pending:
        res = server.wait(t, 120)
        assert res.status == 0, server.last_error()
        if kind == "r":
            out_r[i] = (counts_key(res.counts), rec_key(server.records(t)))
        else:
            cols = None
            if res.island.found:
                mn, mx = server.preview_columns(t, res.preview_columns)
                cols = (mn.tolist(), mx.tolist())
            out_p[i] = (res.island.key(), cols)
        server.release(t)
    return [out_r[i] for i in range(len(ranges))], [out_p[i] for i in range(len(previews))]


def test_served_results_same_alone_and_in_the_mix(workload):
    ranges, direct, previews = workload
    with bsf.Server(profile="mega", chunk_worlds=4096, max_lanes=1) as s:
        alone_r, alone_p = served_results(s, ranges, previews, interleave=False)
    with bsf.Server(profile="mega", chunk_worlds=4096, max_lanes=4) as s:
        # every configured lane is open before the first request (the budget allows them all)
        assert list(s.stats().lanes_open) == [4, 2] and s.stats().evictions == 0
        mix_r, mix_p = served_results(s, ranges, previews, interleave=True)
        st = s.stats()
    assert alone_r == mix_r == direct
    expected_p = [(isl, cols) for _, isl, cols in previews]
    assert alone_p == mix_p == expected_p
    # the mix really overlapped work on the device and counted every request
    assert st.max_busy_lanes >= 2
    assert list(st.completed) == [2, len(previews)] and list(st.failed) == [0, 0]
    assert st.worlds_completed == sum(len(r) for r in ranges)
    assert 0 < st.p50_ms[1] <= st.p99_ms[1] <= st.p999_ms[1]
    assert st.hbm_bytes_peak <= st.hbm_budget


def test_handle_footprint_matches_config_footprint():
    for kw in (dict(capacity=4096, centers=8, max_exact_radius=24), dict(capacity=1, centers=1, max_exact_radius=16)):
        with bsf.Worker(profile="mega", **kw) as w:
            assert w.footprint == bsf.config_footprint(profile="mega", **kw)


def test_admission_waits_for_memory_and_stays_in_budget(workload):
    ranges, direct, previews = workload
    chunk = 4096
    range_bytes = bsf.config_footprint(capacity=chunk, centers=8, max_exact_radius=24)
    preview_bytes = bsf.config_footprint(capacity=1, centers=1, max_exact_radius=16)
    budget = range_bytes + preview_bytes + preview_bytes // 2  # room for one lane of each class only
    with bsf.Server(profile="mega", chunk_worlds=chunk, max_lanes=3, hbm_budget_bytes=budget) as s:
        ta = s.submit_range(ranges[0])
        tb = s.submit_range(ranges[1])
        tps = [s.submit_preview(*args) for args, _, _ in previews[:4]]
        ra, rb = s.wait(ta, 120), s.wait(tb, 120)
        got_p = [s.wait(t, 120).island.key() for t in tps]
        st = s.stats()
        assert (counts_key(ra.counts), rec_key(s.records(ta))) == direct[0]
        assert (counts_key(rb.counts), rec_key(s.records(tb))) == direct[1]
    assert got_p == [isl for _, isl, _ in previews[:4]]
    assert st.hbm_budget == budget and st.hbm_bytes_peak <= budget
    assert st.deferred >= 1  # the second range request had to wait for the one range lane
    assert st.lanes_open[0] <= 1 and st.hbm_bytes_in_use <= budget


def test_idle_lanes_of_the_other_class_are_evicted_for_room(workload):
    ranges, direct, previews = workload
    chunk = 4096
    range_bytes = bsf.config_footprint(capacity=chunk, centers=8, max_exact_radius=24)
    preview_bytes = bsf.config_footprint(capacity=1, centers=1, max_exact_radius=16)
    budget = range_bytes + preview_bytes
    with bsf.Server(profile="mega", chunk_worlds=chunk, max_lanes=3, hbm_budget_bytes=budget) as s:
        # three previews at once: the second and third need preview lanes, which fit
        # only after the idle range lane is closed
        tps = [s.submit_preview(*args) for args, _, _ in previews[:3]]
        got_p = [s.wait(t, 120).island.key() for t in tps]
        # a range request then needs its range lane back
        ta = s.submit_range(ranges[1])
        ra = s.wait(ta, 120)
        st = s.stats()
        assert (counts_key(ra.counts), rec_key(s.records(ta))) == direct[1]
    assert got_p == [isl for _, isl, _ in previews[:3]]
    assert st.hbm_bytes_peak <= budget
    assert st.evictions >= 1


def test_skewed_range_jobs_with_per_request_profiles_and_radii():
    """Range jobs of log-uniform lengths, each with its own hunt profile, exact
    radius and island-volume threshold, all in flight at once: every result equals
    the direct handle call for that job alone."""
    rng = np.random.default_rng(4242)
    jobs = []
    for j in range(10):
        n = int(np.exp(rng.uniform(np.log(64), np.log(6000))))
        start = int(rng.integers(0, 2 ** 48 - n))
        profile = int(rng.integers(0, 4))
        radius = int(rng.integers(3, 10))
        ms = bsf.default_match_settings(min_blocks=int(rng.choice([200, 1000, 3000])), min_columns=20)
        jobs.append((np.arange(start, start + n, dtype=np.int64), profile, radius, ms))
    with bsf.Server(profile="mega", chunk_worlds=2048, max_lanes=4) as s:
        tickets = [s.submit_range(seeds, radius=radius, settings=ms, profile=profile)
                   for seeds, profile, radius, ms in jobs]
        served = []
        for t in tickets:
            r = s.wait(t, 300)
            assert r.status == 0, s.last_error()
            served.append((counts_key(r.counts), rec_key(s.records(t))))
            s.release(t)
    with bsf.Worker(capacity=6000, profile="mega", centers=8, max_exact_radius=24) as w:
        for (seeds, profile, radius, ms), got in zip(jobs, served):
            w.set_profile(profile)
            c, r = w.mega_search(seeds, radius=radius, settings=ms)
            assert got == (counts_key(c), rec_key(r))
