"""Host-only checks of the C-ABI boundary: the library builds, loads and exports
every entry point declared in include/bsf.h; argument validation and the worker
CLI's error paths work without a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

import betaseedfinder_gb300 as bsf
from betaseedfinder_gb300 import build as bsf_build

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "bsf.h")


@pytest.fixture(scope="module")
def lib():
    bsf_build.build()
    return bsf.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bsf_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_mirrored_entry_points():
    names = declared_functions()
    for n in bsf.EXPORTS:
        assert n in names, n


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_default_config_and_settings_match_reference_defaults(lib):
    cfg = bsf.Config()
    lib.bsf_default_config(ctypes.byref(cfg))
    assert (cfg.capacity, cfg.profile, cfg.centers, cfg.max_exact_radius) == (32768, bsf.PROFILE_MEGA, 8, 24)
    s = bsf.default_match_settings()
    # SearchSettings.java:39-45
    assert (s.min_blocks, s.min_columns, s.min_y_for_match, s.min_width, s.min_depth) == (1000, 100, 60, 10, 10)
    assert s.min_avg_thickness == 2.0


def test_open_rejects_bad_config_without_touching_the_gpu(lib):
    cfg = bsf.Config()
    lib.bsf_default_config(ctypes.byref(cfg))
    cfg.centers = 3
    h = lib.bsf_open(ctypes.byref(cfg))
    assert h
    assert b"centers" in lib.bsf_last_error(h)
    seeds = (ctypes.c_int64 * 1)(1)
    out = (ctypes.c_uint8 * 16)()
    assert lib.bsf_stage0_filter(h, seeds, 1, out, 16) == -3  # BSF_E_STATE
    lib.bsf_close(h)


def test_null_handle_is_rejected(lib):
    assert lib.bsf_set_mode(None, 0) == -1
    assert lib.bsf_last_error(None) == b"null handle"


def test_worker_cli_error_paths(lib):
    exe = bsf.WORKER_PATH
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stderr
    r = subprocess.run([exe, "bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and r.stderr.startswith("ERROR: unknown mode")
    r = subprocess.run([exe, "stage0stream", "32768", "nonsense"], capture_output=True, text=True)
    assert r.returncode == 1 and "hunt profile must be" in r.stderr
    r = subprocess.run([exe, "stage0stream", "32768", "general", "lean12"], capture_output=True, text=True)
    assert r.returncode == 1 and "telemetry must be research or lean" in r.stderr


def test_splitmix_matches_oracle():
    from oracle import pyoracle as po
    for a in (0, 1, 7, 2 ** 40 + 3):
        v = bsf.splitmix_seed(123456789, a)
        assert v & ((1 << 64) - 1) == po.splitmix_seed(123456789, a)


def test_config_footprint_sums_the_handle_buffers(lib):
    small = bsf.config_footprint(capacity=1, centers=1, max_exact_radius=4)
    big = bsf.config_footprint(capacity=8192)
    assert 0 < small < big < bsf.config_footprint(capacity=32768)
    # the state cache grows with capacity, one generator set per world
    assert bsf.config_footprint(capacity=16384) - big > 8192 * 20000
    cfg = bsf.Config()
    lib.bsf_default_config(ctypes.byref(cfg))
    cfg.max_exact_radius = 25
    out = ctypes.c_uint64(0)
    assert lib.bsf_config_footprint(ctypes.byref(cfg), ctypes.byref(out)) == -1


def test_server_config_validation_without_a_gpu(lib):
    cfg = bsf.ServerConfig()
    lib.bsf_default_server_config(ctypes.byref(cfg))
    assert (cfg.chunk_worlds, cfg.max_lanes, cfg.max_preview_radius) == (8192, 4, 16)
    cfg.max_lanes = 0
    s = lib.bsf_server_open(ctypes.byref(cfg))
    assert s and b"max_lanes" in lib.bsf_server_last_error(s)
    t = ctypes.c_uint64(0)
    seeds = (ctypes.c_int64 * 1)(1)
    assert lib.bsf_server_submit_range(s, seeds, 1, 7, -1, None, ctypes.byref(t)) == -3  # BSF_E_STATE
    r = bsf.ServerResult()
    assert lib.bsf_server_poll(s, 1, 0, ctypes.byref(r)) == -1  # unknown ticket
    lib.bsf_server_close(s)


@pytest.mark.parametrize("value,prec,expected", [
    ("1.03125", 4, "1.0313"), ("2.675", 2, "2.68"), ("12.5", 4, "12.5000"), ("0.5", 0, "1"),
    ("-1.25", 1, "-1.3"), ("99.99995", 4, "100.0000"), ("nan", 6, "NaN"), ("0.000123456", 6, "0.000123"),
])
def test_candidate_log_formats_numbers_like_java(lib, value, prec, expected):
    """hunter_candidates.csv numbers follow Java's String.format("%.nf"): the
    shortest decimal digits of the double, rounded half-up (2.675 -> 2.68)."""
    out = subprocess.run([bsf.WORKER_PATH, "javafmt", value, str(prec)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == expected
