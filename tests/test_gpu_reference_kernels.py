"""Pin against the reference's own GPU code.

The reference worker's kernels (P20, Upper, Lower, coarse signs and the
parallel coarse scorer), compiled unmodified from the reference source into
oracle/_ref/ref_worker.cubin, run on the GPU in the order of the reference's
stage0stream mode (oracle/ref_gpu.cpp). Their records must equal both the
oracle's (so the oracle is pinned to the reference's GPU code on thousands of
worlds) and the CUDA product path's, byte for byte, lean and research, under
every hunt profile.
"""
import os

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

EDGE_SEEDS = [0, 1, -1, 2 ** 63 - 1, -2 ** 63, 123456789, -4172144997902289642, 2 ** 48 - 1, 2 ** 48]
HERE = os.path.dirname(os.path.abspath(__file__))


def consecutive_seeds(n, salt):
    rng = np.random.default_rng(abs(salt))
    start = int(rng.integers(0, 2 ** 48 - n))
    return np.arange(start, start + n, dtype=np.int64)


def rejection_seeds():
    import json
    with open(os.path.join(HERE, "golden", "rng_rejection_seeds.json")) as f:
        return np.array([int(s) for s in json.load(f)["seeds"]], np.int64)


@pytest.fixture(scope="module")
def ref_gpu():
    if not os.path.exists(po.REF_CUBIN):
        pytest.skip("reference GPU image oracle/_ref/ref_worker.cubin was not built (no reference checkout)")
    g = po.RefGpu(capacity=32768)
    yield g
    g.close()


def diff_rows(a, b, rec):
    a, b = a.reshape(-1, rec), b.reshape(-1, rec)
    return np.flatnonzero((a != b).any(axis=1))


@pytest.mark.parametrize("profile,research", [(bsf.PROFILE_MEGA, True), (bsf.PROFILE_GENERAL, False),
                                              (bsf.PROFILE_RECORD60, True)])
def test_reference_gpu_equals_oracle_and_product(ref_gpu, profile, research):
    seeds = np.concatenate([consecutive_seeds(2048, 40 + profile), np.array(EDGE_SEEDS, np.int64),
                            rejection_seeds()])
    rec = 34 if research else 16
    got_ref = ref_gpu.stage0_batch(seeds, centers=8, profile=profile, research=research)
    want = po.stage0_batch(seeds, centers=8, profile=profile, research=research)
    bad = diff_rows(got_ref, want, rec)
    assert bad.size == 0, ("reference GPU vs oracle", bad[:10])
    with bsf.Worker(capacity=len(seeds), profile=profile, research=research, centers=8, max_exact_radius=2) as w:
        mine = w.stage0_filter(seeds)
    bad = diff_rows(mine, got_ref, rec)
    assert bad.size == 0, ("product vs reference GPU", bad[:10])
    # the batch reaches every stage: coarse-evaluated regions exist (coarse is 0 unless evaluated)
    assert (got_ref.reshape(-1, rec)[:, 3] == 1).any()


def test_reference_gpu_equals_product_full_batch(ref_gpu):
    """A full 32,768-world batch (262,144 regions), research records, MEGA profile."""
    seeds = consecutive_seeds(32768, 77)
    got_ref = ref_gpu.stage0_batch(seeds, centers=8, profile=bsf.PROFILE_MEGA, research=True)
    with bsf.Worker(capacity=len(seeds), profile=bsf.PROFILE_MEGA, research=True, centers=8,
                    max_exact_radius=2) as w:
        mine = w.stage0_filter(seeds)
    r = got_ref.reshape(-1, 34)
    bad = diff_rows(mine, got_ref, 34)
    assert bad.size == 0, bad[:10]
    coarse = r[:, 4].astype(np.int32) | (r[:, 5].astype(np.int32) << 8)
    assert (coarse >= 85).sum() > 10  # regions pass the coarse gate in a batch this size


def test_reference_gpu_single_centre_matches_product(ref_gpu):
    seeds = consecutive_seeds(4096, 91)
    got_ref = ref_gpu.stage0_batch(seeds, centers=1, profile=bsf.PROFILE_RECORD80, research=True)
    with bsf.Worker(capacity=len(seeds), profile=bsf.PROFILE_RECORD80, research=True, centers=1,
                    max_exact_radius=2) as w:
        mine = w.stage0_filter(seeds)
    assert diff_rows(mine, got_ref, 34).size == 0
