"""Find world seeds whose generator setup hits java.util.Random.nextInt's
rejection loop (the draw r with r - r % bound + bound - 1 overflowing int32).

World setup (BetaTerrain173.java:84-91, WorldChunkManager173.java:24-31): one
terrain Random(seed) feeding 74 octave constructors (noise2 16, noise3 16,
noise1 8, two skipped groups of 4, noise4 10, noise5 16) and three climate
Randoms (seed*9871: 4, seed*39811: 4, seed*543321: 2). Each constructor draws 3
nextDouble and 256 nextInt(256 - i). The scan runs the LCG for many seeds at
once with numpy and flags a seed at its first rejection (its stream is not
followed further). Writes rng_rejection_seeds.json beside this script, with a
SHA-256 of each found world's 76 generator states (permutation bytes, then the
a/b/c offsets as IEEE-754 bits) computed by the reference's own compiled
Random/initPerlin (oracle/_ref, built from the reference checkout).

    python tests/golden/find_rejection_seeds.py [start] [count]
"""
import json
import os
import sys

import numpy as np

MASK = np.uint64((1 << 48) - 1)
MUL = np.uint64(0x5DEECE66D)
ADD = np.uint64(0xB)


def scan(seeds):
    seeds = np.asarray(seeds, dtype=np.int64)
    hit = np.zeros(len(seeds), bool)

    def run(state, constructors):
        for _ in range(constructors):
            for _ in range(6):  # three nextDouble = six next() calls
                state = (state * MUL + ADD) & MASK
            for i in range(256):
                bound = 256 - i
                state = (state * MUL + ADD) & MASK
                if bound & (bound - 1) == 0:
                    continue
                r = (state >> np.uint64(17)).astype(np.int64)        # next(31), non-negative
                t = (r - r % bound + bound - 1)                     # overflows int32 when rejected
                hit[(t > 0x7FFFFFFF)] = True
        return state

    def set_seed(s):
        return (s.astype(np.uint64) ^ MUL) & MASK

    run(set_seed(seeds), 74)
    for k, n in ((9871, 4), (39811, 4), (543321, 2)):
        run(set_seed(seeds * np.int64(k)), n)   # Java long multiply wraps like int64
    return hit


def main():
    start = int(sys.argv[1]) if len(sys.argv) > 1 else 1_000_000
    count = int(sys.argv[2]) if len(sys.argv) > 2 else 20_000
    seeds = np.arange(start, start + count, dtype=np.int64)
    with np.errstate(over="ignore"):
        hit = scan(seeds)
    found = [int(s) for s in seeds[hit]]
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(os.path.dirname(here)))
    import ctypes
    import hashlib
    from oracle import pyoracle as po
    R = po.ref() or (po.build_ref() and po.ref())
    if R is None:
        raise SystemExit("the reference harness (oracle/_ref) is needed to record the states")
    states = {}
    for sd in found:
        hsh = hashlib.sha256()
        for idx in range(76):
            rp = np.zeros(256, np.uint8)
            ra = np.zeros(3)
            R.ref_world_state(sd, idx, rp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                              ra.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            hsh.update(rp.tobytes())
            hsh.update(ra.view(np.uint64).tobytes())
        states[str(sd)] = hsh.hexdigest()
    out = os.path.join(here, "rng_rejection_seeds.json")
    with open(out, "w") as f:
        json.dump({"start": start, "count": count, "seeds": found, "ref_states_sha256": states}, f, indent=1)
    print("%d of %d seeds hit the nextInt rejection loop -> %s" % (len(found), count, out))


if __name__ == "__main__":
    main()
