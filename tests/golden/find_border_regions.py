"""Find regions whose island reaches the side of the radius-7 scan, so that
side-border verification (radii 10, 13, 16, 20, 24) has to widen the scan,
and record them as a fixture for tests/test_gpu_parity_wide.py.

Runs the MEGA pipeline on a GPU (betaseedfinder_gb300) over consecutive seeded
worlds and keeps records whose raw or hot-scan island was border-verified past
its first radius. Usage (on a GPU machine):
    python tests/golden/find_border_regions.py [worlds=4194304] [out=tests/golden/border_regions.json]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import betaseedfinder_gb300 as bsf  # noqa: E402


def main():
    worlds = int(sys.argv[1]) if len(sys.argv) > 1 else 1 << 22
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, "border_regions.json")
    start = 0x5DEECE66D * 4099 % (1 << 47)
    batch = 32768
    found = []
    with bsf.Worker(capacity=batch, profile=bsf.PROFILE_MEGA, centers=8, max_exact_radius=24) as w:
        for off in range(0, worlds, batch):
            seeds = np.arange(start + off, start + off + batch, dtype=np.int64)
            _, recs = w.mega_search(seeds, radius=7)
            for r in recs:
                raw_wide = r.raw_island.found and r.raw_island.radius_used > 7
                hot_wide = r.hot_island.found and r.hot_island.radius_used > 16
                touched = r.island.found and r.island.touches_side
                if raw_wide or hot_wide or touched:
                    found.append({"seed": int(r.seed), "center_chunk_x": r.center_chunk_x,
                                  "center_chunk_z": r.center_chunk_z, "coarse": r.coarse,
                                  "raw_radius": r.raw_island.radius_used if r.raw_island.found else 0,
                                  "hot_radius": r.hot_island.radius_used if r.hot_island.found else 0,
                                  "final_radius": r.island.radius_used, "blocks": r.island.blocks})
    json.dump({"about": "MEGA regions whose side-border verification widened the exact scan (radius 7 "
                        "scan, hot scan at 16), found by find_border_regions.py over %d consecutive worlds "
                        "from %d" % (worlds, start), "regions": found}, open(out, "w"), indent=1)
    print("wrote %s: %d regions" % (out, len(found)))


if __name__ == "__main__":
    main()
