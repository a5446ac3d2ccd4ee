"""ctypes bindings for the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module. It compiles oracle/bsf_oracle.c with gcc on first use (strict
IEEE: -ffp-contract=off, no fast-math) into oracle/_build/, and optionally
loads the reference harness from oracle/_ref/ when it was built here.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_harness.so")
SOURCES = [os.path.join(HERE, "bsf_oracle.c"), os.path.join(HERE, "bsf_oracle.h"),
           os.path.join(HERE, "..", "betaseedfinder_gb300", "csrc", "p19_table.inc")]


def build(force=False):
    """Compile liboracle.so if missing or older than its sources."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB):
        lib_m = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_m for s in SOURCES):
            return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp, SOURCES[0], "-lpthread", "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


def build_ref():
    """Build oracle/_ref from the reference checkout when it is present (this container only)."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.call(["sh", script])
    return REF_LIB if os.path.exists(REF_LIB) else None


class Features(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "fullY88", "fullY96", "fullY104", "fullY112",
        "y88Largest", "y88Width", "y88Depth", "y88Touches",
        "y96Largest", "y96Width", "y96Depth", "y96Touches")]


class Region(ctypes.Structure):
    _fields_ = [("p20", ctypes.c_int32), ("upper", ctypes.c_int32), ("high", ctypes.c_int32),
                ("p19Evaluated", ctypes.c_int32), ("p19Pass", ctypes.c_int32),
                ("p19Extreme", ctypes.c_int32), ("megaReject", ctypes.c_int32),
                ("coarseEvaluated", ctypes.c_int32), ("coarse", ctypes.c_int32),
                ("p19Score", ctypes.c_double), ("f", Features),
                ("upperMask", ctypes.c_uint8 * 256), ("highest", ctypes.c_uint8 * 256)]


class Profile(ctypes.Structure):
    _fields_ = [("p20MinCount", ctypes.c_int), ("upperMinCount", ctypes.c_int),
                ("highMinCount", ctypes.c_int), ("p19MinScore", ctypes.c_double),
                ("coarseMinCells", ctypes.c_int), ("megaTopologyFilter", ctypes.c_int)]


class MatchSettings(ctypes.Structure):
    _fields_ = [("minBlocks", ctypes.c_int), ("minColumns", ctypes.c_int),
                ("minYForMatch", ctypes.c_int), ("minWidth", ctypes.c_int),
                ("minDepth", ctypes.c_int), ("minAvgThickness", ctypes.c_double)]


class Island(ctypes.Structure):
    _fields_ = [("found", ctypes.c_int32), ("blocks", ctypes.c_int32), ("columns", ctypes.c_int32),
                ("minX", ctypes.c_int32), ("maxX", ctypes.c_int32), ("minZ", ctypes.c_int32),
                ("maxZ", ctypes.c_int32), ("minY", ctypes.c_int32), ("maxY", ctypes.c_int32),
                ("centerX", ctypes.c_int32), ("centerZ", ctypes.c_int32),
                ("touchesSide", ctypes.c_int32), ("touchesBottom", ctypes.c_int32),
                ("radiusUsed", ctypes.c_int32), ("sumX", ctypes.c_int64), ("sumZ", ctypes.c_int64)]

    def key(self):
        return (self.found, self.blocks, self.columns, self.minX, self.maxX, self.minZ, self.maxZ,
                self.minY, self.maxY, self.centerX, self.centerZ, self.touchesSide, self.radiusUsed)


class LazyStats(ctypes.Structure):
    _fields_ = [("lowerColumns", ctypes.c_int32), ("rounds", ctypes.c_int32), ("fallbackToFull", ctypes.c_int32)]


class PipelineCounts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "worlds", "regions", "p20Passed", "upperPassed", "highPassed", "p19Passed",
        "megaRejected", "coarseEvaluated", "coarsePassed", "islands")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        P = ctypes.POINTER
        u8p, f64p, i64p, u64p, i32p = (P(ctypes.c_uint8), P(ctypes.c_double), P(ctypes.c_int64),
                                       P(ctypes.c_uint64), P(ctypes.c_int32))
        L.or_world_state.argtypes = [ctypes.c_int64, ctypes.c_int, u8p, f64p]
        L.or_perlin_column17_test.argtypes = [u8p, f64p, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_int, f64p]
        L.or_chunk_stone_bitmap.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, u8p]
        L.or_chunk_stone_bitmap.restype = ctypes.c_uint64
        L.or_bitmap_hash.argtypes = [u8p]
        L.or_bitmap_hash.restype = ctypes.c_uint64
        L.or_chunk_bitmaps.argtypes = [i64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, u8p, u64p, ctypes.c_int]
        L.or_coarse_score_seed.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        L.or_coarse_score.argtypes = [u8p]
        L.or_coarse_signs_seed.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, u8p]
        L.or_coarse_score_lazy_seed.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, P(LazyStats)]
        L.or_p19_score.argtypes = [ctypes.c_int, P(Features)]
        L.or_p19_score.restype = ctypes.c_double
        L.or_p19_extreme.argtypes = [P(Features)]
        L.or_monster_features.argtypes = [u8p, P(Features)]
        L.or_profile_get.argtypes = [ctypes.c_int, P(Profile)]
        L.or_stage0_batch.argtypes = [i64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, u8p, ctypes.c_int]
        L.or_match_defaults.argtypes = [P(MatchSettings)]
        L.or_exact_scan.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, P(MatchSettings), P(Island)]
        L.or_resolve_region.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        P(MatchSettings), P(Island)]
        L.or_preview.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, P(MatchSettings),
                                 P(Island), i32p, i32p, ctypes.c_int]
        L.or_mega_pipeline.argtypes = [i64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, P(MatchSettings),
                                       ctypes.c_int, P(PipelineCounts), P(Island), i64p, ctypes.c_int]
        L.or_splitmix_seed.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.or_splitmix_seed.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def world_state(seed, index):
    perm = np.zeros(256, np.uint8)
    abc = np.zeros(3, np.float64)
    lib().or_world_state(seed, index, _ptr(perm, ctypes.c_uint8), _ptr(abc, ctypes.c_double))
    return perm, abc


def chunk_bitmaps(seeds, chunk_x=0, chunk_z=0, threads=os.cpu_count() or 1):
    seeds = np.ascontiguousarray(seeds, dtype=np.int64)
    n = len(seeds)
    bm = np.zeros((n, 4096), np.uint8)
    h = np.zeros(n, np.uint64)
    lib().or_chunk_bitmaps(_ptr(seeds, ctypes.c_int64), n, chunk_x, chunk_z,
                           _ptr(bm, ctypes.c_uint8), _ptr(h, ctypes.c_uint64), threads)
    return bm, h


def bitmap_hash(bitmap4096):
    bm = np.ascontiguousarray(bitmap4096, dtype=np.uint8)
    return int(lib().or_bitmap_hash(_ptr(bm, ctypes.c_uint8)))


def stage0_batch(seeds, centers=8, profile=1, research=False, threads=os.cpu_count() or 1):
    seeds = np.ascontiguousarray(seeds, dtype=np.int64)
    rec = 34 if research else 16
    out = np.zeros(len(seeds) * centers * rec, np.uint8)
    lib().or_stage0_batch(_ptr(seeds, ctypes.c_int64), len(seeds), centers, profile, int(research),
                          _ptr(out, ctypes.c_uint8), threads)
    return out


def coarse_signs(seed, cx=0, cz=0):
    sg = np.zeros(61 * 61 * 17, np.uint8)
    lib().or_coarse_signs_seed(seed, cx, cz, _ptr(sg, ctypes.c_uint8))
    return sg


def coarse_score(seed, cx=0, cz=0):
    return int(lib().or_coarse_score_seed(seed, cx, cz))


def coarse_score_lazy(seed, cx=0, cz=0):
    """The Java app's component-lazy coarse score (P17) and its generation stats."""
    st = LazyStats()
    score = int(lib().or_coarse_score_lazy_seed(seed, cx, cz, ctypes.byref(st)))
    return score, st


def match_settings(**kw):
    s = MatchSettings()
    lib().or_match_defaults(ctypes.byref(s))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def exact_scan(seed, cx=0, cz=0, radius=7, settings=None):
    s = settings or match_settings()
    out = Island()
    lib().or_exact_scan(seed, cx, cz, radius, ctypes.byref(s), ctypes.byref(out))
    return out


def resolve_region(seed, cx, cz, radius, coarse, settings=None):
    s = settings or match_settings()
    out = Island()
    lib().or_resolve_region(seed, cx, cz, radius, coarse, ctypes.byref(s), ctypes.byref(out))
    return out


def preview(seed, cx=0, cz=0, radius=7, settings=None, capacity=1 << 20):
    s = settings or match_settings()
    out = Island()
    mn = np.zeros(capacity, np.int32)
    mx = np.zeros(capacity, np.int32)
    lib().or_preview(seed, cx, cz, radius, ctypes.byref(s), ctypes.byref(out),
                     _ptr(mn, ctypes.c_int32), _ptr(mx, ctypes.c_int32), capacity)
    if not out.found:
        return out, None, None
    n = (out.maxX - out.minX + 1) * (out.maxZ - out.minZ + 1)
    return out, mn[:n].copy(), mx[:n].copy()


def mega_pipeline(seeds, profile=1, radius=7, settings=None, threads=os.cpu_count() or 1, island_cap=1 << 16):
    seeds = np.ascontiguousarray(seeds, dtype=np.int64)
    s = settings or match_settings()
    counts = PipelineCounts()
    islands = (Island * island_cap)()
    regions = np.zeros(island_cap, np.int64)
    n = lib().or_mega_pipeline(_ptr(seeds, ctypes.c_int64), len(seeds), profile, radius, ctypes.byref(s),
                               threads, ctypes.byref(counts), islands, _ptr(regions, ctypes.c_int64), island_cap)
    return counts, [islands[i] for i in range(n)], regions[:n].copy()


def splitmix_seed(sequence_seed, attempt):
    return int(lib().or_splitmix_seed(sequence_seed & (2**64 - 1), attempt & (2**64 - 1)))


_ref = None


def ref():
    """The reference-harness library, or None when it was not built here."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        L = ctypes.CDLL(REF_LIB)
        P = ctypes.POINTER
        u8p, f64p, i32p = P(ctypes.c_uint8), P(ctypes.c_double), P(ctypes.c_int)
        L.ref_world_state.argtypes = [ctypes.c_int64, ctypes.c_int, u8p, f64p]
        for name, n in (("ref_perlin3", 3), ("ref_perlin2", 2), ("ref_simplex2", 2)):
            f = getattr(L, name)
            f.argtypes = [u8p, f64p] + [ctypes.c_double] * n
            f.restype = ctypes.c_double
        L.ref_perlin3_full17.argtypes = [u8p, f64p, ctypes.c_double, ctypes.c_double, ctypes.c_double, f64p]
        L.ref_perlin3_upper6.argtypes = [u8p, f64p, ctypes.c_double, ctypes.c_double, ctypes.c_double, f64p]
        L.ref_coarse_score.argtypes = [ctypes.c_int64, u8p]
        L.ref_p19_score.argtypes = [ctypes.c_int, i32p]
        L.ref_p19_score.restype = ctypes.c_double
        L.ref_p19_extreme.argtypes = [i32p]
        L.ref_splitmix.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.ref_splitmix.restype = ctypes.c_uint64
        _ref = L
    return _ref


# ---- the reference worker's own GPU kernels (oracle/ref_gpu.cpp) -------------
REF_CUBIN = os.path.join(HERE, "_ref", "ref_worker.cubin")
REF_GPU_LIB = os.path.join(BUILD, "libref_gpu.so")


def build_ref_gpu():
    """Compile the host driver of the reference's GPU kernels (CUDA driver API,
    linked against the oracle for the host P19 step). Returns the library path,
    or None when the reference image oracle/_ref/ref_worker.cubin is absent."""
    if not os.path.exists(REF_CUBIN):
        return None
    build()
    src = os.path.join(HERE, "ref_gpu.cpp")
    deps = [src, os.path.join(HERE, "bsf_oracle.h"), LIB]
    if os.path.exists(REF_GPU_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(REF_GPU_LIB) for d in deps):
        return REF_GPU_LIB
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    tmp = REF_GPU_LIB + ".tmp.%d" % os.getpid()
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", tmp, src, "-I" + HERE,
                           "-I" + os.path.join(cuda, "include"), "-L" + os.path.join(cuda, "lib64", "stubs"),
                           "-lcuda", "-L" + BUILD, "-loracle", "-Wl,-rpath," + BUILD])
    os.replace(tmp, REF_GPU_LIB)
    return REF_GPU_LIB


class RefGpu:
    """The reference worker's stage0stream path on the GPU: its own kernels
    (compiled unmodified into oracle/_ref/ref_worker.cubin) in its own launch
    order, with the host steps restated in oracle/ref_gpu.cpp."""

    def __init__(self, capacity, device=0):
        path = build_ref_gpu()
        if path is None:
            raise FileNotFoundError("reference GPU image not built (oracle/_ref/ref_worker.cubin)")
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.rg_open.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
        L.rg_open.restype = ctypes.c_void_p
        L.rg_stage0_batch.argtypes = [ctypes.c_void_p, P(ctypes.c_int64), ctypes.c_uint32, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, P(ctypes.c_uint8), ctypes.c_char_p,
                                      ctypes.c_size_t]
        L.rg_last_ms.argtypes = [ctypes.c_void_p, P(ctypes.c_double)]
        L.rg_close.argtypes = [ctypes.c_void_p]
        self.L = L
        self.capacity = capacity
        err = ctypes.create_string_buffer(512)
        self.h = L.rg_open(REF_CUBIN.encode(), device, capacity, err, 512)
        if not self.h:
            raise RuntimeError("rg_open: " + err.value.decode())

    def stage0_batch(self, seeds, centers=8, profile=1, research=False):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        rec = 34 if research else 16
        out = np.zeros(len(seeds) * centers * rec, np.uint8)
        err = ctypes.create_string_buffer(512)
        rc = self.L.rg_stage0_batch(self.h, _ptr(seeds, ctypes.c_int64), len(seeds), centers, profile,
                                    int(research), _ptr(out, ctypes.c_uint8), err, 512)
        if rc != 0:
            raise RuntimeError("rg_stage0_batch: " + err.value.decode())
        return out

    def last_ms(self):
        ms = np.zeros(3, np.float64)
        self.L.rg_last_ms(self.h, _ptr(ms, ctypes.c_double))
        return ms

    def close(self):
        if self.h:
            self.L.rg_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
