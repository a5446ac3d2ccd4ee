"""bsf_chunk_bitmaps_noalloc: the allocation-free entry point, checked against
bsf_chunk_bitmaps through the C ABI on two calls in a row.

The entry point serves callers that cannot allocate GPU memory themselves or
through the library (a host that owns all device memory, a serving loop where
an allocation would synchronise the device, a fixed memory budget); it uses a
fixed scratch array compiled into the library. This file is collected last so
that a failure here comes after every other test has run; it also passes alone
in a fresh process, where its first call performs the per-device set-up."""
import ctypes

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf

pytestmark = pytest.mark.gpu


def _bind():
    from betaseedfinder_gb300 import build
    build.build()
    L = bsf.load()
    f = L.bsf_chunk_bitmaps_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    return f


def test_noalloc_matches_allocating_entry_point_twice():
    """Calls in a row, against bsf_chunk_bitmaps: a partial call, one at the size
    limit, then a smaller call at another chunk, which must ignore what the larger
    call left in the shared scratch array. A repeat of the last call takes no
    device memory (the free memory the driver reports does not change)."""
    torch = pytest.importorskip("torch")
    noalloc = _bind()
    stream = torch.cuda.current_stream().cuda_stream
    calls = [(200, 0, 0, 101), (256, -3, 5, 202), (17, 9, -4, 303)]
    for n, cx, cz, salt in calls:
        start = int(np.random.default_rng(salt).integers(0, 2 ** 48 - n))
        seeds = np.arange(start, start + n, dtype=np.int64)
        d_seeds = torch.from_numpy(seeds).cuda()
        d_bm = torch.full((n, 4096), 0xAB, dtype=torch.uint8, device="cuda")
        d_h = torch.zeros(n, dtype=torch.int64, device="cuda")
        err = ctypes.create_string_buffer(256)
        rc = noalloc(d_seeds.data_ptr(), n, cx, cz, d_bm.data_ptr(), d_h.data_ptr(), stream, err, 256)
        assert rc == 0, err.value
        torch.cuda.synchronize()
        with bsf.Worker(capacity=n, profile="general", centers=1, max_exact_radius=1) as w:
            bm, h = w.chunk_bitmaps(seeds, cx, cz)
        assert np.array_equal(d_bm.cpu().numpy(), bm)
        assert np.array_equal(d_h.cpu().numpy().view(np.uint64), h)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc = noalloc(d_seeds.data_ptr(), n, cx, cz, d_bm.data_ptr(), d_h.data_ptr(), stream, err, 256)
    assert rc == 0, err.value
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert np.array_equal(d_bm.cpu().numpy(), bm)


def test_noalloc_rejects_counts_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    noalloc = _bind()
    n = 257
    d_seeds = torch.zeros(n, dtype=torch.int64, device="cuda")
    d_bm = torch.zeros((n, 4096), dtype=torch.uint8, device="cuda")
    d_h = torch.zeros(n, dtype=torch.int64, device="cuda")
    err = ctypes.create_string_buffer(256)
    rc = noalloc(d_seeds.data_ptr(), n, 0, 0, d_bm.data_ptr(), d_h.data_ptr(), None, err, 256)
    assert rc == -4  # BSF_E_LIMIT
    assert b"256" in err.value
