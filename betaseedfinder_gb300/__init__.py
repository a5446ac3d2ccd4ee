"""BetaSeedFinder GB300: Python host mirror of the worker's C ABI (include/bsf.h).

The compute path is libbsf.so (hand-written sm_103a CUDA kernels). This module
only loads it with ctypes and mirrors the reference's caller-facing interface:
`GpuStage0Scout` / `GpuP20Scout` batch filters (src/GpuStage0Scout.java,
src/GpuP20Scout.java), the exact chunk terrain of `BetaTerrain173`, the exact
island scan and preview of `IslandSearchEngine`, and the batch MEGA search.
There is no CPU fallback: if the extension is missing or no GPU is usable the
calls raise.
"""
import ctypes
import os

import numpy as np

# Served-mode lanes run on separate streams; give each its own hardware queue
# (must happen before the process creates its CUDA context).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbsf.so")
WORKER_PATH = os.path.join(HERE, "_build", "bsf_worker")

PROFILE_GENERAL, PROFILE_MEGA, PROFILE_RECORD60, PROFILE_RECORD80 = 0, 1, 2, 3
PROFILES = {"general": 0, "mega": 1, "record60": 2, "record80": 3}
MODE_QUEUED, MODE_PLAIN, MODE_PLAIN_SCREENED = 0, 1, 2
CENTER_CHUNK_X = (0, 15, 0, 15, -15, -15, 0, 15)
CENTER_CHUNK_Z = (0, 0, 15, 15, 0, 15, -15, -15)


class BsfError(RuntimeError):
    pass


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("capacity", ctypes.c_uint32), ("profile", ctypes.c_int32),
                ("research", ctypes.c_int32), ("centers", ctypes.c_int32), ("max_exact_radius", ctypes.c_int32)]


class MatchSettings(ctypes.Structure):
    _fields_ = [("min_blocks", ctypes.c_int32), ("min_columns", ctypes.c_int32),
                ("min_y_for_match", ctypes.c_int32), ("min_width", ctypes.c_int32),
                ("min_depth", ctypes.c_int32), ("min_avg_thickness", ctypes.c_double)]


class Island(ctypes.Structure):
    _fields_ = [("found", ctypes.c_int32), ("blocks", ctypes.c_int32), ("columns", ctypes.c_int32),
                ("min_x", ctypes.c_int32), ("max_x", ctypes.c_int32), ("min_z", ctypes.c_int32),
                ("max_z", ctypes.c_int32), ("min_y", ctypes.c_int32), ("max_y", ctypes.c_int32),
                ("center_x", ctypes.c_int32), ("center_z", ctypes.c_int32),
                ("touches_side", ctypes.c_int32), ("touches_bottom", ctypes.c_int32),
                ("radius_used", ctypes.c_int32), ("sum_x", ctypes.c_int64), ("sum_z", ctypes.c_int64)]

    def key(self):
        return (self.found, self.blocks, self.columns, self.min_x, self.max_x, self.min_z, self.max_z,
                self.min_y, self.max_y, self.center_x, self.center_z, self.touches_side, self.radius_used)


class MegaRecord(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_int64), ("world_index", ctypes.c_int32), ("center_index", ctypes.c_int32),
                ("center_chunk_x", ctypes.c_int32), ("center_chunk_z", ctypes.c_int32),
                ("p20", ctypes.c_int32), ("upper", ctypes.c_int32), ("high", ctypes.c_int32),
                ("coarse", ctypes.c_int32), ("p19_score", ctypes.c_double), ("island", Island),
                ("raw_island", Island), ("hot_island", Island), ("hot_scanned", ctypes.c_int32),
                ("final_source", ctypes.c_int32), ("p19_pass", ctypes.c_int32), ("p19_extreme", ctypes.c_int32)]


class StageCounts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "worlds", "regions", "p20_passed", "upper_passed", "high_passed", "p19_passed",
        "mega_rejected", "coarse_evaluated", "coarse_passed", "islands", "rng_fallbacks", "lower_columns",
        "screened_tasks", "fallback_tasks")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("profile", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_uint64),
                ("chunk_worlds", ctypes.c_uint32), ("max_lanes", ctypes.c_int32),
                ("preview_lanes", ctypes.c_int32), ("max_preview_radius", ctypes.c_int32)]


class ServerResult(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("status", ctypes.c_int32), ("queue_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double), ("records", ctypes.c_uint32), ("counts", StageCounts),
                ("island", Island), ("preview_columns", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64 * 2), ("completed", ctypes.c_uint64 * 2),
                ("failed", ctypes.c_uint64 * 2), ("p50_ms", ctypes.c_double * 2), ("p99_ms", ctypes.c_double * 2),
                ("p999_ms", ctypes.c_double * 2), ("worlds_completed", ctypes.c_uint64),
                ("hbm_bytes_in_use", ctypes.c_uint64), ("hbm_bytes_peak", ctypes.c_uint64),
                ("hbm_budget", ctypes.c_uint64), ("lanes_open", ctypes.c_uint32 * 2),
                ("max_busy_lanes", ctypes.c_uint32), ("deferred", ctypes.c_uint64), ("evictions", ctypes.c_uint64)]

    def as_dict(self):
        d = {}
        for n, _ in self._fields_:
            v = getattr(self, n)
            d[n] = list(v) if hasattr(v, "__len__") else v
        return d


class SweepCounts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "worlds", "regions", "p20_passed", "upper_passed", "high_passed", "survivors", "rng_fallbacks",
        "screened_tasks", "fallback_tasks")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


REQ_RANGE, REQ_PREVIEW = 0, 1
PENDING = 1

EXPORTS = ["bsf_default_config", "bsf_default_match_settings", "bsf_open", "bsf_close", "bsf_last_error",
           "bsf_set_mode", "bsf_stage0_filter", "bsf_stage0_sweep", "bsf_p20_filter", "bsf_chunk_bitmaps", "bsf_exact_scan",
           "bsf_resolve_region", "bsf_preview", "bsf_mega_search", "bsf_mega_search_device",
           "bsf_mega_search_range", "bsf_mega_search_range_device",
           "bsf_kernel_launches", "bsf_device_summary", "bsf_screen_probe", "bsf_last_stage_ms", "bsf_measure_peaks", "bsf_chunk_bitmaps_noalloc",
           "bsf_autotune", "bsf_set_launch_variants", "bsf_config_footprint", "bsf_handle_footprint",
           "bsf_set_stream_priority", "bsf_set_persistent", "bsf_set_screening", "bsf_set_profile", "bsf_last_region_records", "bsf_default_server_config", "bsf_server_open", "bsf_server_close",
           "bsf_server_last_error", "bsf_server_submit_range", "bsf_server_submit_preview", "bsf_server_poll",
           "bsf_server_records", "bsf_server_preview_columns", "bsf_server_release", "bsf_server_get_stats"]

_lib = None


def load(path=LIB_PATH):
    """Load libbsf.so (build it with betaseedfinder_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise BsfError("libbsf.so not built at %s; run betaseedfinder_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp, i64p, u8p, u64p, i32p = ctypes.c_void_p, P(ctypes.c_int64), P(ctypes.c_uint8), P(ctypes.c_uint64), P(ctypes.c_int32)
    L.bsf_default_config.argtypes = [P(Config)]
    L.bsf_default_match_settings.argtypes = [P(MatchSettings)]
    L.bsf_open.argtypes = [P(Config)]
    L.bsf_open.restype = vp
    L.bsf_close.argtypes = [vp]
    L.bsf_last_error.argtypes = [vp]
    L.bsf_last_error.restype = ctypes.c_char_p
    L.bsf_set_mode.argtypes = [vp, ctypes.c_int32]
    L.bsf_stage0_filter.argtypes = [vp, i64p, ctypes.c_uint32, u8p, ctypes.c_size_t]
    L.bsf_p20_filter.argtypes = [vp, i64p, ctypes.c_uint32, u8p, ctypes.c_size_t]
    L.bsf_stage0_sweep.argtypes = [vp, ctypes.c_int64, ctypes.c_uint64, i64p, ctypes.c_uint64, u64p, P(SweepCounts)]
    L.bsf_chunk_bitmaps.argtypes = [vp, i64p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32, u8p, u64p]
    L.bsf_exact_scan.argtypes = [vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                 P(MatchSettings), P(Island)]
    L.bsf_resolve_region.argtypes = [vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_int32, P(MatchSettings), P(Island)]
    L.bsf_preview.argtypes = [vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                              P(MatchSettings), P(Island), i32p, i32p, ctypes.c_uint32]
    L.bsf_mega_search.argtypes = [vp, i64p, ctypes.c_uint32, ctypes.c_int32, P(MatchSettings), P(MegaRecord),
                                  ctypes.c_uint32, P(ctypes.c_uint32), P(StageCounts)]
    L.bsf_mega_search_device.argtypes = [vp, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, P(MatchSettings),
                                         P(MegaRecord), ctypes.c_uint32, P(ctypes.c_uint32), P(StageCounts),
                                         ctypes.c_void_p]
    L.bsf_mega_search_range.argtypes = [vp, i64p, ctypes.c_uint64, ctypes.c_int32, P(MatchSettings), P(MegaRecord),
                                        ctypes.c_uint32, P(ctypes.c_uint32), P(StageCounts)]
    L.bsf_mega_search_range_device.argtypes = [vp, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32,
                                               P(MatchSettings), P(MegaRecord), ctypes.c_uint32, P(ctypes.c_uint32),
                                               P(StageCounts), ctypes.c_void_p]
    L.bsf_kernel_launches.argtypes = [vp]
    L.bsf_kernel_launches.restype = ctypes.c_uint64
    L.bsf_last_stage_ms.argtypes = [vp, P(ctypes.c_float)]
    L.bsf_measure_peaks.argtypes = [P(ctypes.c_double)]
    L.bsf_autotune.argtypes = [vp, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t]
    L.bsf_set_launch_variants.argtypes = [vp, ctypes.c_int32, ctypes.c_int32]
    L.bsf_config_footprint.argtypes = [P(Config), u64p]
    L.bsf_handle_footprint.argtypes = [vp]
    L.bsf_handle_footprint.restype = ctypes.c_uint64
    L.bsf_set_stream_priority.argtypes = [vp, ctypes.c_int32]
    L.bsf_set_persistent.argtypes = [vp, ctypes.c_int32]
    L.bsf_set_screening.argtypes = [vp, ctypes.c_int32]
    L.bsf_default_server_config.argtypes = [P(ServerConfig)]
    L.bsf_server_open.argtypes = [P(ServerConfig)]
    L.bsf_server_open.restype = vp
    L.bsf_server_close.argtypes = [vp]
    L.bsf_server_last_error.argtypes = [vp]
    L.bsf_server_last_error.restype = ctypes.c_char_p
    L.bsf_server_submit_range.argtypes = [vp, i64p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32, P(MatchSettings),
                                          u64p]
    L.bsf_set_profile.argtypes = [vp, ctypes.c_int32]
    L.bsf_last_region_records.argtypes = [vp, u8p, ctypes.c_size_t]
    L.bsf_server_submit_preview.argtypes = [vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                            P(MatchSettings), u64p]
    L.bsf_server_poll.argtypes = [vp, ctypes.c_uint64, ctypes.c_int32, P(ServerResult)]
    L.bsf_server_records.argtypes = [vp, ctypes.c_uint64, P(MegaRecord), ctypes.c_uint32, P(ctypes.c_uint32)]
    L.bsf_server_preview_columns.argtypes = [vp, ctypes.c_uint64, i32p, i32p, ctypes.c_uint32]
    L.bsf_server_release.argtypes = [vp, ctypes.c_uint64]
    L.bsf_server_get_stats.argtypes = [vp, P(ServerStats)]
    _lib = L
    return L


PROBE_KINDS = ("octave3_fp64_axes", "octave3_df_axes", "octave2_fp64_axes", "octave2_df_axes",
               "simplex_df_geometry", "simplex_fp64_geometry", "climate", "column_shape")


def screen_probe(seeds, samples_per_thread=32, rng=1):
    """Largest |FP32 - FP64| / bound per screening primitive (bsf_screen_probe)."""
    L = load()
    seeds = np.ascontiguousarray(seeds, dtype=np.int64)
    ratio = (ctypes.c_double * len(PROBE_KINDS))()
    counts = (ctypes.c_uint64 * len(PROBE_KINDS))()
    err = ctypes.create_string_buffer(256)
    L.bsf_screen_probe.argtypes = [ctypes.POINTER(ctypes.c_int64), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64), ctypes.c_char_p,
                                   ctypes.c_size_t]
    st = L.bsf_screen_probe(_p(seeds, ctypes.c_int64), len(seeds), samples_per_thread, rng, ratio, counts, err, 256)
    if st != 0:
        raise BsfError("bsf_screen_probe: %s" % err.value.decode())
    return {k: (ratio[i], counts[i]) for i, k in enumerate(PROBE_KINDS)}


def measure_peaks():
    """Measured scalar issue rates of the current GPU: (FP64 adds/s, FP32 adds/s)."""
    ops = (ctypes.c_double * 2)()
    if load().bsf_measure_peaks(ops) != 0:
        raise BsfError("bsf_measure_peaks failed")
    return ops[0], ops[1]


def config_footprint(capacity=32768, profile=PROFILE_MEGA, research=False, centers=8, max_exact_radius=24):
    """Device bytes a Worker with this configuration allocates (no GPU needed)."""
    L = load()
    cfg = Config()
    L.bsf_default_config(ctypes.byref(cfg))
    cfg.capacity = capacity
    cfg.profile = PROFILES.get(profile, profile) if isinstance(profile, str) else profile
    cfg.research, cfg.centers, cfg.max_exact_radius = int(research), centers, max_exact_radius
    b = ctypes.c_uint64(0)
    if L.bsf_config_footprint(ctypes.byref(cfg), ctypes.byref(b)) != 0:
        raise BsfError("bsf_config_footprint: bad config")
    return int(b.value)


def default_match_settings(**overrides):
    s = MatchSettings()
    load().bsf_default_match_settings(ctypes.byref(s))
    for k, v in overrides.items():
        setattr(s, k, v)
    return s


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


class Worker:
    """One GPU worker handle (the C ABI's bsf_handle)."""

    def __init__(self, capacity=32768, profile=PROFILE_MEGA, research=False, centers=8, max_exact_radius=24,
                 device=0):
        L = load()
        cfg = Config()
        L.bsf_default_config(ctypes.byref(cfg))
        cfg.device, cfg.capacity = device, capacity
        cfg.profile = PROFILES.get(profile, profile) if isinstance(profile, str) else profile
        cfg.research, cfg.centers, cfg.max_exact_radius = int(research), centers, max_exact_radius
        self.cfg = cfg
        self._h = L.bsf_open(ctypes.byref(cfg))
        if not self._h:
            raise BsfError("bsf_open failed")
        err = L.bsf_last_error(self._h)
        if err:
            msg = err.decode()
            L.bsf_close(self._h)
            self._h = None
            raise BsfError("bsf_open: " + msg)

    def close(self):
        if self._h:
            load().bsf_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status):
        if status != 0:
            raise BsfError("status %d: %s" % (status, load().bsf_last_error(self._h).decode()))

    @property
    def record_bytes(self):
        return 34 if self.cfg.research else 16

    @property
    def kernel_launches(self):
        return int(load().bsf_kernel_launches(self._h))

    def autotune(self, worlds=4096):
        """Pick the fastest launch shape of the screened kernels; returns the timing report."""
        buf = ctypes.create_string_buffer(512)
        self._check(load().bsf_autotune(self._h, worlds, buf, 512))
        return buf.value.decode()

    def set_launch_variants(self, stage0_variant, coarse_variant):
        self._check(load().bsf_set_launch_variants(self._h, stage0_variant, coarse_variant))

    @property
    def footprint(self):
        """Device bytes this handle holds."""
        return int(load().bsf_handle_footprint(self._h))

    def last_region_records(self, worlds):
        """34-byte research records of every region of the last MEGA batch (`worlds` worlds)."""
        out = np.zeros(worlds * self.cfg.centers * 34, np.uint8)
        self._check(load().bsf_last_region_records(self._h, _p(out, ctypes.c_uint8), out.nbytes))
        return out

    def set_profile(self, profile):
        self._check(load().bsf_set_profile(self._h, PROFILES.get(profile, profile) if isinstance(profile, str)
                                           else profile))

    def set_screening(self, on=True):
        """False: every screened column task takes the exact FP64 fallback path and exact scans the
        all-FP64 fill (verification; results must not change)."""
        self._check(load().bsf_set_screening(self._h, int(bool(on))))

    def set_persistent(self, on=True):
        self._check(load().bsf_set_persistent(self._h, int(bool(on))))

    def set_stream_priority(self, high=True):
        self._check(load().bsf_set_stream_priority(self._h, int(bool(high))))

    def last_stage_ms(self):
        """Per-stage device times of the last batch: setup, Stage0+P19, coarse, exact (ms)."""
        ms = (ctypes.c_float * 4)()
        self._check(load().bsf_last_stage_ms(self._h, ms))
        return list(ms)

    def set_mode(self, mode):
        self._check(load().bsf_set_mode(self._h, mode))

    def stage0_filter(self, seeds):
        """stage0stream response body: count * centers records (numpy uint8)."""
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        out = np.zeros(len(seeds) * self.cfg.centers * self.record_bytes, np.uint8)
        self._check(load().bsf_stage0_filter(self._h, _p(seeds, ctypes.c_int64), len(seeds),
                                             _p(out, ctypes.c_uint8), out.nbytes))
        return out

    def stage0_sweep(self, start_seed, count, cap=None):
        """Stage0 scout sweep over `count` consecutive seeds from start_seed: the
        surviving worlds' seeds (numpy int64, sweep order, at most cap), the total
        survivor count and the stage pass counters."""
        cap = int(count) if cap is None else int(cap)
        out = np.zeros(max(cap, 1), np.int64)
        n = ctypes.c_uint64(0)
        c = SweepCounts()
        start = int(start_seed)
        start = start - (1 << 64) if start >= (1 << 63) else start
        self._check(load().bsf_stage0_sweep(self._h, start, int(count), _p(out, ctypes.c_int64), cap,
                                            ctypes.byref(n), ctypes.byref(c)))
        return out[:min(cap, n.value)].copy(), n.value, c.as_dict()

    def p20_filter(self, seeds):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        out = np.zeros(len(seeds), np.uint8)
        self._check(load().bsf_p20_filter(self._h, _p(seeds, ctypes.c_int64), len(seeds),
                                          _p(out, ctypes.c_uint8), out.nbytes))
        return out

    def chunk_bitmaps(self, seeds, chunk_x=0, chunk_z=0):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        bm = np.zeros((len(seeds), 4096), np.uint8)
        h = np.zeros(len(seeds), np.uint64)
        self._check(load().bsf_chunk_bitmaps(self._h, _p(seeds, ctypes.c_int64), len(seeds), chunk_x, chunk_z,
                                             _p(bm, ctypes.c_uint8), _p(h, ctypes.c_uint64)))
        return bm, h

    def exact_scan(self, seed, center_chunk_x=0, center_chunk_z=0, radius=7, settings=None):
        out = Island()
        s = settings or default_match_settings()
        self._check(load().bsf_exact_scan(self._h, seed, center_chunk_x, center_chunk_z, radius, ctypes.byref(s),
                                          ctypes.byref(out)))
        return out

    def resolve_region(self, seed, center_chunk_x, center_chunk_z, radius, coarse, settings=None):
        out = Island()
        s = settings or default_match_settings()
        self._check(load().bsf_resolve_region(self._h, seed, center_chunk_x, center_chunk_z, radius, coarse,
                                              ctypes.byref(s), ctypes.byref(out)))
        return out

    def preview(self, seed, center_chunk_x=0, center_chunk_z=0, radius=7, settings=None, capacity=1 << 20):
        out = Island()
        s = settings or default_match_settings()
        mn = np.zeros(capacity, np.int32)
        mx = np.zeros(capacity, np.int32)
        self._check(load().bsf_preview(self._h, seed, center_chunk_x, center_chunk_z, radius, ctypes.byref(s),
                                       ctypes.byref(out), _p(mn, ctypes.c_int32), _p(mx, ctypes.c_int32), capacity))
        if not out.found:
            return out, None, None
        n = (out.max_x - out.min_x + 1) * (out.max_z - out.min_z + 1)
        return out, mn[:n].copy(), mx[:n].copy()

    def mega_search(self, seeds, radius=7, settings=None, records_cap=4096):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        s = settings or default_match_settings()
        recs = (MegaRecord * records_cap)()
        n = ctypes.c_uint32(0)
        counts = StageCounts()
        self._check(load().bsf_mega_search(self._h, _p(seeds, ctypes.c_int64), len(seeds), radius, ctypes.byref(s),
                                           recs, records_cap, ctypes.byref(n), ctypes.byref(counts)))
        return counts, [recs[i] for i in range(n.value)]

    def mega_search_device(self, d_seeds_ptr, count, radius=7, settings=None, records_cap=4096, stream=None):
        s = settings or default_match_settings()
        recs = (MegaRecord * records_cap)()
        n = ctypes.c_uint32(0)
        counts = StageCounts()
        self._check(load().bsf_mega_search_device(self._h, ctypes.c_void_p(d_seeds_ptr), count, radius,
                                                  ctypes.byref(s), recs, records_cap, ctypes.byref(n),
                                                  ctypes.byref(counts), ctypes.c_void_p(stream or 0)))
        return counts, [recs[i] for i in range(n.value)]


    def mega_search_range(self, seeds, radius=7, settings=None, records_cap=1 << 16):
        """Pipelined MEGA search over a seed array of any length (bsf_mega_search_range)."""
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        s = settings or default_match_settings()
        recs = (MegaRecord * records_cap)()
        n = ctypes.c_uint32(0)
        counts = StageCounts()
        self._check(load().bsf_mega_search_range(self._h, _p(seeds, ctypes.c_int64), len(seeds), radius,
                                                 ctypes.byref(s), recs, records_cap, ctypes.byref(n),
                                                 ctypes.byref(counts)))
        return counts, [recs[i] for i in range(n.value)]

    def mega_search_range_device(self, d_seeds_ptr, count, radius=7, settings=None, records_cap=1 << 16, stream=None):
        s = settings or default_match_settings()
        recs = (MegaRecord * records_cap)()
        n = ctypes.c_uint32(0)
        counts = StageCounts()
        self._check(load().bsf_mega_search_range_device(self._h, ctypes.c_void_p(d_seeds_ptr), count, radius,
                                                        ctypes.byref(s), recs, records_cap, ctypes.byref(n),
                                                        ctypes.byref(counts), ctypes.c_void_p(stream or 0)))
        return counts, [recs[i] for i in range(n.value)]


class Server:
    """Served mode (bsf_server_*): continuous batching of range searches and
    previews over device-resident lanes, admitted by HBM footprint."""

    def __init__(self, profile=PROFILE_MEGA, hbm_budget_bytes=0, chunk_worlds=8192, max_lanes=4,
                 preview_lanes=2, max_preview_radius=16, device=0):
        L = load()
        cfg = ServerConfig()
        L.bsf_default_server_config(ctypes.byref(cfg))
        cfg.device = device
        cfg.profile = PROFILES.get(profile, profile) if isinstance(profile, str) else profile
        cfg.hbm_budget_bytes, cfg.chunk_worlds, cfg.max_lanes = hbm_budget_bytes, chunk_worlds, max_lanes
        cfg.preview_lanes = preview_lanes
        cfg.max_preview_radius = max_preview_radius
        self._s = L.bsf_server_open(ctypes.byref(cfg))
        if not self._s:
            raise BsfError("bsf_server_open failed")
        err = L.bsf_server_last_error(self._s)
        if err:
            L.bsf_server_close(self._s)
            self._s = None
            raise BsfError("bsf_server_open: " + err.decode())

    def close(self):
        if self._s:
            load().bsf_server_close(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status):
        if status < 0:
            raise BsfError("status %d: %s" % (status, load().bsf_server_last_error(self._s).decode()))
        return status

    def last_error(self):
        return load().bsf_server_last_error(self._s).decode()

    def submit_range(self, seeds, radius=7, settings=None, profile=None):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        t = ctypes.c_uint64(0)
        s = settings or default_match_settings()
        prof = -1 if profile is None else (PROFILES.get(profile, profile) if isinstance(profile, str) else profile)
        self._check(load().bsf_server_submit_range(self._s, _p(seeds, ctypes.c_int64), len(seeds), radius, prof,
                                                   ctypes.byref(s), ctypes.byref(t)))
        return int(t.value)

    def submit_preview(self, seed, center_chunk_x=0, center_chunk_z=0, radius=7, settings=None):
        t = ctypes.c_uint64(0)
        s = settings or default_match_settings()
        self._check(load().bsf_server_submit_preview(self._s, seed, center_chunk_x, center_chunk_z, radius,
                                                     ctypes.byref(s), ctypes.byref(t)))
        return int(t.value)

    def poll(self, ticket, wait_ms=0):
        """ServerResult when finished, None while pending."""
        r = ServerResult()
        st = self._check(load().bsf_server_poll(self._s, ticket, wait_ms, ctypes.byref(r)))
        return None if st == PENDING else r

    def wait(self, ticket, timeout_s=600.0):
        """Block until the ticket finishes; raises BsfError after timeout_s."""
        import time
        deadline = time.monotonic() + timeout_s
        while True:
            r = self.poll(ticket, 200)
            if r is not None:
                return r
            if time.monotonic() > deadline:
                raise BsfError("request %d not finished after %.0f s" % (ticket, timeout_s))

    def records(self, ticket, cap=1 << 16):
        recs = (MegaRecord * cap)()
        n = ctypes.c_uint32(0)
        self._check(load().bsf_server_records(self._s, ticket, recs, cap, ctypes.byref(n)))
        return [recs[i] for i in range(n.value)]

    def preview_columns(self, ticket, cells):
        mn = np.zeros(max(cells, 1), np.int32)
        mx = np.zeros(max(cells, 1), np.int32)
        self._check(load().bsf_server_preview_columns(self._s, ticket, _p(mn, ctypes.c_int32),
                                                      _p(mx, ctypes.c_int32), max(cells, 1)))
        return mn[:cells], mx[:cells]

    def release(self, ticket):
        self._check(load().bsf_server_release(self._s, ticket))

    def stats(self):
        st = ServerStats()
        self._check(load().bsf_server_get_stats(self._s, ctypes.byref(st)))
        return st


class GpuStage0Scout:
    """Mirror of src/GpuStage0Scout.java: filter(seeds, count) -> BatchResult arrays."""

    def __init__(self, capacity=32768, profile="general", research=True, centers=8):
        self.worker = Worker(capacity=capacity, profile=profile, research=research, centers=centers,
                             max_exact_radius=1)
        self.centers = centers

    def center_count(self):
        return self.centers

    def center_chunk_x(self, i):
        return CENTER_CHUNK_X[i]

    def center_chunk_z(self, i):
        return CENTER_CHUNK_Z[i]

    def result_index(self, world_index, center_index):
        return world_index * self.centers + center_index

    def filter(self, seeds, count=None):
        seeds = np.asarray(seeds, dtype=np.int64)[: (len(seeds) if count is None else count)]
        raw = self.worker.stage0_filter(seeds)
        return decode_records(raw, self.worker.record_bytes)

    def close(self):
        self.worker.close()


def decode_records(raw, record_bytes):
    """Decode stage0stream records into the Java BatchResult field arrays (GpuStage0Scout.java:290-335)."""
    r = np.asarray(raw, np.uint8).reshape(-1, record_bytes)
    u16 = lambda o: r[:, o].astype(np.int32) | (r[:, o + 1].astype(np.int32) << 8)
    out = {
        "p20Counts": r[:, 0].copy(), "fullUpperCounts": r[:, 1].copy(), "highReentryCounts": r[:, 2].copy(),
        "p19Pass": r[:, 3].copy(), "coarseScores": u16(4), "p19ExtremeBypass": r[:, 6].copy(),
        "megaTopologyRejected": r[:, 7].copy(),
        "p19Scores": np.ascontiguousarray(r[:, 8:16]).view(np.float64).ravel(),
    }
    if record_bytes == 34:
        out.update({"p19FullY88": u16(16), "p19FullY96": u16(18), "p19FullY104": u16(20), "p19FullY112": u16(22),
                    "p19Y88LargestCluster": u16(24), "p19Y88Width": r[:, 26].copy(), "p19Y88Depth": r[:, 27].copy(),
                    "p19Y88TouchesBorder": r[:, 28].copy(), "p19Y96LargestCluster": u16(29),
                    "p19Y96Width": r[:, 31].copy(), "p19Y96Depth": r[:, 32].copy(),
                    "p19Y96TouchesBorder": r[:, 33].copy()})
    return out


def splitmix_seed(sequence_seed, attempt):
    """deterministicSeedForAttempt (src/IslandSearchEngine.java:2551-2556), as a signed int64."""
    m = (1 << 64) - 1
    z = (sequence_seed + attempt * 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    z ^= z >> 31
    return z - (1 << 64) if z >= 1 << 63 else z
