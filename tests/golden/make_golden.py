#!/usr/bin/env python3
"""Generate tests/golden/reference_vectors.json from the reference's own C++.

Runs in the container that holds the reference checkout: builds oracle/_ref
(the reference headers p20_exact_math.hpp, coarse_exact_core.hpp and
p19_monster_gate.hpp compiled in place by oracle/build_ref.sh) and records
outputs of the reference's functions on seeded inputs. The JSON is committed
so the oracle can be checked against the reference where the checkout is
absent. Doubles are stored as 16-hex-digit IEEE bit patterns.
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vectors.json")


def bits(a):
    return [format(int(v), "016x") for v in np.asarray(a, np.float64).view(np.uint64)]


def ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def main():
    if po.build_ref() is None:
        raise SystemExit("reference checkout not available; cannot regenerate")
    R = po.ref()
    rng = np.random.default_rng(20261203)
    out = {"generator": "tests/golden/make_golden.py", "source": "reference native/src host C++"}

    seeds = [0, 1, -1, 123456789, -4172144997902289642, 2**47 - 1] + [int(s) for s in rng.integers(-2**63, 2**63 - 1, 4)]
    states = []
    for seed in seeds:
        for idx in range(76):
            perm = np.zeros(256, np.uint8)
            abc = np.zeros(3)
            R.ref_world_state(seed, idx, ptr(perm, ctypes.c_uint8), ptr(abc, ctypes.c_double))
            h = hashlib.sha256(perm.tobytes() + abc.tobytes()).hexdigest()
            states.append({"seed": seed, "index": idx, "sha256": h, "abc": bits(abc)})
    out["world_states"] = states

    cols = []
    for _ in range(150):
        seed = int(rng.integers(-2**62, 2**62))
        idx = int(rng.integers(0, 76))
        perm = np.zeros(256, np.uint8)
        abc = np.zeros(3)
        R.ref_world_state(seed, idx, ptr(perm, ctypes.c_uint8), ptr(abc, ctypes.c_double))
        x, z = (float(v) for v in rng.uniform(-70000, 70000, 2))
        sy = float(rng.choice([684.412, 342.206, 171.103, 4.277575, 2.1387875, 0.020886, 1.3368, 0.6684]))
        full = np.zeros(17)
        up = np.zeros(6)
        R.ref_perlin3_full17(ptr(perm, ctypes.c_uint8), ptr(abc, ctypes.c_double), x, sy, z, ptr(full, ctypes.c_double))
        R.ref_perlin3_upper6(ptr(perm, ctypes.c_uint8), ptr(abc, ctypes.c_double), x, sy, z, ptr(up, ctypes.c_double))
        p2 = R.ref_perlin2(ptr(perm, ctypes.c_uint8), ptr(abc, ctypes.c_double), x, z)
        s2 = R.ref_simplex2(ptr(perm, ctypes.c_uint8), ptr(abc, ctypes.c_double), x * 0.01, z * 0.01)
        cols.append({"seed": seed, "index": idx, "x": bits([x])[0], "z": bits([z])[0], "sy": bits([sy])[0],
                     "full17": bits(full), "upper6": bits(up), "perlin2": bits([p2])[0], "simplex2": bits([s2])[0]})
    out["columns"] = cols

    p19 = []
    for _ in range(600):
        f = rng.integers(0, 64, 12).astype(np.int32)
        f[7] %= 2
        f[11] %= 2
        scout = int(rng.integers(0, 256))
        s = R.ref_p19_score(scout, ptr(f, ctypes.c_int))
        e = R.ref_p19_extreme(ptr(f, ctypes.c_int))
        p19.append({"scout": scout, "features": [int(v) for v in f], "score": bits([s])[0], "extreme": int(e)})
    out["p19"] = p19

    coarse = []
    for seed in [123, 456, 252543233732390, 245883435698426, 987654321987]:
        sg = np.zeros(61 * 61 * 17, np.uint8)
        score = R.ref_coarse_score(seed, ptr(sg, ctypes.c_uint8))
        coarse.append({"seed": seed, "score": int(score), "signs_sha256": hashlib.sha256(sg.tobytes()).hexdigest(),
                       "positive": int(sg.sum())})
    out["coarse"] = coarse

    out["splitmix"] = [{"sequence": 123456789, "attempt": a, "seed": str(R.ref_splitmix(123456789, a))}
                       for a in (0, 1, 2, 1000, 2**40)]

    # noise1..5 octave sums of the reference's coarse grid (generateAndScoreHost) at
    # coarse -28..32 around centre (0,0): the lattice points of the 15x15 chunks of a
    # radius-7 region, which the chunk path of BetaTerrain173 samples at the same coordinates
    dp = ctypes.POINTER(ctypes.c_double)
    R.ref_coarse_noise.argtypes = [ctypes.c_int64] + [dp] * 5
    chunk_noise = []
    for seed in [123, -4172144997902289642, 2**48 - 1, 0, 252543233732390] + [int(s) for s in rng.integers(-2**63, 2**63 - 1, 3)]:
        arrs = [np.zeros(61 * 61 * 17), np.zeros(61 * 61 * 17), np.zeros(61 * 61 * 17), np.zeros(61 * 61),
                np.zeros(61 * 61)]
        R.ref_coarse_noise(seed, *[ptr(a, ctypes.c_double) for a in arrs])
        chunk_noise.append({"seed": seed, "sha256": [hashlib.sha256(a.tobytes()).hexdigest() for a in arrs],
                            "n2_col0": bits(arrs[1][:17]), "n5_col0": bits(arrs[4][:1])})
    out["chunk_noise"] = chunk_noise
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=0, separators=(",", ":"))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
