"""The drop-in boundary: bsf_worker's stage0stream pipe protocol, as the Java
scout drives it (GpuStage0Scout.java:143-335; gpu_p20_benchmark.cpp:7310-7502).
Batches of 1, 3 and the full capacity go in as LE u32 count + LE i64 seeds; the
answer is the 8-byte magic, then per batch LE u32 count + 34-byte research
records, each equal to the oracle's. A zero count ends the stream; a batch over
the capacity and a truncated batch end it with the reference's errors."""
import struct
import subprocess

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

CAPACITY = 64


def batch(seeds):
    return struct.pack("<I", len(seeds)) + b"".join(struct.pack("<q", int(s)) for s in seeds)


def test_stage0stream_batches_match_the_oracle():
    rng = np.random.default_rng(5)
    batches = [rng.integers(-2 ** 63, 2 ** 63 - 1, size=n, dtype=np.int64) for n in (1, 3, CAPACITY)]
    stdin = b"".join(batch(b) for b in batches) + struct.pack("<I", 0)
    r = subprocess.run([bsf.WORKER_PATH, "stage0stream", str(CAPACITY), "mega", "research", "8"], input=stdin,
                       capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()
    out = r.stdout
    assert out[:8] == b"ST0R3816"
    pos = 8
    for seeds in batches:
        (count,) = struct.unpack_from("<I", out, pos)
        assert count == len(seeds)
        pos += 4
        got = np.frombuffer(out, np.uint8, count * 8 * 34, pos)
        pos += count * 8 * 34
        want = po.stage0_batch(seeds, centers=8, profile=1, research=True)
        assert np.array_equal(got, want.reshape(-1))
    assert pos == len(out)
    # the close summary carries the reference's stage counters (gpu_p20_benchmark.cpp:7601-7611),
    # here recounted from the oracle's records with the MEGA gates (P20 1, Upper 8, High 6, coarse 85)
    recs = np.concatenate([po.stage0_batch(b, centers=8, profile=1, research=True).reshape(-1, 34) for b in batches])
    a, b_, c = recs[:, 0].astype(int), recs[:, 1].astype(int), recs[:, 2].astype(int)
    d = recs[:, 4].astype(int) | (recs[:, 5].astype(int) << 8)
    s05 = (a >= 1) & (b_ >= 8) & (c >= 6)
    p19 = s05 & (recs[:, 3] != 0)
    mega = p19 & (recs[:, 7] != 0)
    want = {"worlds": sum(len(x) for x in batches), "regions": 8 * sum(len(x) for x in batches),
            "P20Passed": int((a >= 1).sum()), "Stage1Passed": int(((a >= 1) & (b_ >= 8)).sum()),
            "Stage0.5Passed": int(s05.sum()), "Stage0.75Evaluated": int(s05.sum()),
            "Stage0.75Passed": int(p19.sum()), "Stage0.75Rejected": int((s05 & ~p19).sum()),
            "MegaTopologyRejected": int(mega.sum()), "CoarseEvaluated": int((p19 & ~mega).sum()),
            "CoarsePassedTarget": int((p19 & ~mega & (d >= 85)).sum())}
    line = [ln for ln in r.stderr.decode().splitlines() if ln.startswith("Stage0+P19+coarse stream closed")]
    assert len(line) == 1, r.stderr.decode()
    got = dict(f.strip().split("=") for f in line[0].split("|")[1:])
    assert {k: int(v) for k, v in got.items()} == want
    assert "Profile: MEGA 30k+ | P20>=1 | Upper>=8 | High>=6 | P19>=4.02/extreme | Coarse>=85" in r.stderr.decode()


def test_stage0stream_rejects_oversized_and_truncated_batches():
    seeds = np.arange(CAPACITY + 1, dtype=np.int64)
    r = subprocess.run([bsf.WORKER_PATH, "stage0stream", str(CAPACITY), "mega", "lean", "8"], input=batch(seeds),
                       capture_output=True, timeout=300)
    assert r.returncode == 1
    assert "Stage0 stream batch exceeds configured world capacity" in r.stderr.decode()
    truncated = struct.pack("<I", 5) + b"".join(struct.pack("<q", s) for s in (1, 2))
    r = subprocess.run([bsf.WORKER_PATH, "stage0stream", str(CAPACITY), "mega", "lean", "8"], input=truncated,
                       capture_output=True, timeout=300)
    assert r.returncode == 1 and "truncated" in r.stderr.decode()


def test_megastream_records_match_the_api():
    """megastream: magic, then per batch LE u32 record count + 104-byte records
    (seed, world, centre, centre chunk x/z, p20, upper, high, coarse, P19 score
    bits, 14 island ints), equal to the C ABI's MEGA records for the same seeds.
    The seeds are the fixture's high-coarse regions, so records exist."""
    import json
    import os
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "high_coarse_regions.json")))
    seeds = np.array(sorted({r["seed"] for r in fx["regions"][:8]}), dtype=np.int64)
    r = subprocess.run([bsf.WORKER_PATH, "megastream", "64", "mega", "7"], input=batch(seeds) + struct.pack("<I", 0),
                       capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()
    out = r.stdout
    assert out[:8] == b"MEGAST01"
    (n,) = struct.unpack_from("<I", out, 8)
    assert len(out) == 12 + n * 104 and n > 0
    with bsf.Worker(capacity=64, profile="mega", centers=8, max_exact_radius=24) as w:
        _, recs = w.mega_search(seeds, radius=7)
    assert n == len(recs)
    for k, rec in enumerate(recs):
        f = struct.unpack_from("<q8iQ14i", out, 12 + k * 104)
        assert f[0] == rec.seed
        assert f[1:9] == (rec.world_index, rec.center_index, rec.center_chunk_x, rec.center_chunk_z, rec.p20,
                          rec.upper, rec.high, rec.coarse)
        assert f[9] == struct.unpack("<Q", struct.pack("<d", rec.p19_score))[0]
        i = rec.island
        assert f[10:23] == (i.found, i.blocks, i.columns, i.min_x, i.max_x, i.min_z, i.max_z, i.min_y, i.max_y,
                            i.center_x, i.center_z, i.touches_side, i.radius_used)


def test_p20_stream_bytes_match_the_oracle():
    """stream (the P20-only fallback path, gpu_p20_benchmark.cpp:7614-7685): magic,
    then per batch LE u32 count + one clamped P20 count byte per seed."""
    rng = np.random.default_rng(9)
    batches = [rng.integers(-2 ** 63, 2 ** 63 - 1, size=n, dtype=np.int64) for n in (2, CAPACITY)]
    stdin = b"".join(batch(b) for b in batches) + struct.pack("<I", 0)
    r = subprocess.run([bsf.WORKER_PATH, "stream", str(CAPACITY)], input=stdin, capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()
    out = r.stdout
    assert out[:8] == b"P20STR01"
    pos = 8
    for seeds in batches:
        (count,) = struct.unpack_from("<I", out, pos)
        assert count == len(seeds)
        got = np.frombuffer(out, np.uint8, count, pos + 4)
        pos += 4 + count
        want = po.stage0_batch(seeds, centers=1, profile=0, research=False).reshape(-1, 16)[:, 0]
        assert np.array_equal(got, want)
    assert pos == len(out)
