"""Stage0 scout sweep (bsf_stage0_sweep): consecutive seeds through the Stage0
gate, survivors compacted on the device in seed order.

The survivors must be exactly the worlds whose regions pass the profile's P20,
Upper and high gates in the oracle's stage0stream records (small sweeps), and in
the product's own stage0stream records, which are pinned to the reference
worker's GPU kernels (sweeps over several batches and survivor-list flushes).
"""
import numpy as np
import pytest

import betaseedfinder_gb300 as bsf
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

GATES = {bsf.PROFILE_GENERAL: (1, 5, 5), bsf.PROFILE_MEGA: (1, 8, 6), bsf.PROFILE_RECORD60: (3, 19, 12),
         bsf.PROFILE_RECORD80: (3, 19, 20)}


def wrap64(v):
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >= 1 << 63 else v


def survivors_from_records(seeds, records, centers, profile):
    """Worlds with a region through the P20, Upper and high gates (lean or research records)."""
    rec = records.reshape(len(seeds), centers, -1)
    p20m, upm, him = GATES[profile]
    ok = (rec[:, :, 0] >= p20m) & (rec[:, :, 1] >= upm) & (rec[:, :, 2] >= him)
    return seeds[ok.any(axis=1)], int(ok.sum())


@pytest.mark.parametrize("profile,centers", [(bsf.PROFILE_MEGA, 1), (bsf.PROFILE_GENERAL, 1),
                                             (bsf.PROFILE_RECORD60, 8)])
def test_sweep_matches_oracle(profile, centers):
    rng = np.random.default_rng(1000 + profile * 10 + centers)
    count = 3000 if centers == 1 else 600
    start = int(rng.integers(0, 2 ** 48 - count))
    with bsf.Worker(capacity=1024, profile=profile, centers=centers, max_exact_radius=2) as w:
        got, total, counts = w.stage0_sweep(start, count)
    seeds = np.arange(start, start + count, dtype=np.int64)
    want, regions_high = survivors_from_records(seeds, po.stage0_batch(seeds, centers=centers, profile=profile),
                                                centers, profile)
    assert total == len(want) == counts["survivors"]
    assert np.array_equal(got, want)
    assert counts["worlds"] == count and counts["regions"] == count * centers
    assert counts["high_passed"] == regions_high
    assert counts["p20_passed"] >= counts["upper_passed"] >= counts["high_passed"] >= total


def test_sweep_many_batches_matches_stage0_records():
    """Several batches per survivor-list flush, several flushes and a partial last batch."""
    cap_worlds = 1024
    count = cap_worlds * 8 * 2 + 777
    start = int(np.random.default_rng(7).integers(0, 2 ** 48 - count))
    seeds = np.arange(start, start + count, dtype=np.int64)
    with bsf.Worker(capacity=cap_worlds, profile=bsf.PROFILE_MEGA, centers=1, max_exact_radius=2) as w:
        got, total, counts = w.stage0_sweep(start, count)
        recs = np.concatenate([w.stage0_filter(seeds[i:i + cap_worlds]) for i in range(0, count, cap_worlds)])
        # a cap below the total returns the first survivors and the full count
        part, total2, _ = w.stage0_sweep(start, count, cap=5)
    want, regions_high = survivors_from_records(seeds, recs, 1, bsf.PROFILE_MEGA)
    assert np.array_equal(got, want) and total == len(want)
    assert counts["high_passed"] == regions_high
    r = recs.reshape(count, 16)
    assert counts["p20_passed"] == int((r[:, 0] >= 1).sum())
    assert counts["upper_passed"] == int(((r[:, 0] >= 1) & (r[:, 1] >= 8)).sum())
    assert total2 == total and np.array_equal(part, want[:5])
    assert np.all(np.diff(got) > 0)


def test_sweep_wraps_at_int64_boundary():
    start = 2 ** 63 - 150
    count = 300
    seeds = np.array([wrap64(start + i) for i in range(count)], dtype=np.int64)
    with bsf.Worker(capacity=256, profile=bsf.PROFILE_GENERAL, centers=1, max_exact_radius=2) as w:
        got, total, _ = w.stage0_sweep(start, count)
    want, _ = survivors_from_records(seeds, po.stage0_batch(seeds, centers=1, profile=bsf.PROFILE_GENERAL), 1,
                                     bsf.PROFILE_GENERAL)
    assert np.array_equal(got, want)


def test_sweep_rejects_bad_arguments():
    with bsf.Worker(capacity=64, profile=bsf.PROFILE_MEGA, centers=1, max_exact_radius=2) as w:
        with pytest.raises(bsf.BsfError):
            w.stage0_sweep(0, 0)
