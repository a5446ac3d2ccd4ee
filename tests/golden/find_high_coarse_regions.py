"""Finds regions with large coarse scores for the coarse-scorer fixtures.

Runs the queued MEGA pipeline (GPU) on consecutive 48-bit world seeds and keeps
the coarse-evaluated regions with the highest scores plus a spread of middle
ones, with the GPU's score. tests/test_oracle_golden.py then requires the
oracle's full coarse scorer and its lazy (P17) restatement to give the same
scores on CPU. Usage: python tests/golden/find_high_coarse_regions.py [start] [worlds]
"""
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", ".."))
import betaseedfinder_gb300 as bsf  # noqa: E402


def main():
    start = int(sys.argv[1]) if len(sys.argv) > 1 else 31_415_926_535
    worlds = int(sys.argv[2]) if len(sys.argv) > 2 else 32768
    seeds = np.arange(start, start + worlds, dtype=np.int64)
    with bsf.Worker(capacity=worlds, profile="mega", centers=8, max_exact_radius=24) as w:
        w.mega_search(seeds)
        rr = w.last_region_records(worlds).reshape(-1, 34).astype(np.int64)
    evaluated = np.flatnonzero((rr[:, 3] != 0) & (rr[:, 7] == 0))
    coarse = rr[:, 4] | (rr[:, 5] << 8)
    order = evaluated[np.argsort(-coarse[evaluated], kind="stable")]
    picked = list(order[:8]) + list(order[len(order) // 4:len(order) // 4 + 4])
    out = [{"seed": int(seeds[g // 8]), "cx": bsf.CENTER_CHUNK_X[g % 8], "cz": bsf.CENTER_CHUNK_Z[g % 8],
            "score": int(coarse[g])} for g in picked]
    path = os.path.join(os.path.dirname(__file__), "high_coarse_regions.json")
    json.dump({"start": start, "worlds": worlds, "regions": out}, open(path, "w"), indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
