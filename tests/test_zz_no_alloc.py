"""The allocation-free trigger scan (gbwt_pfp_trigger_scan_noalloc).

It exists for callers that cannot allocate device memory themselves -- for
example code that runs inside a host framework which hands out a fixed
device-memory budget, or behind an allocator that must not be re-entered.
Those callers pass their own device buffers for the text and the phrase
ends; the entry point's scratch is a library-wide device array.

The test calls it through the C ABI, twice in a row on the same buffers
(the shared scratch keeps the previous call's contents), and checks both
results against the storage-based entry point gbwt_pfp_trigger_scan, exactly
(integer positions).  The file sorts last so that a stop-at-first-failure
run has executed every other test before this one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fn(pkg):
    lib = pkg._lib()
    f = lib.gbwt_pfp_trigger_scan_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    f.restype = ctypes.c_int64
    return f


@pytest.mark.parametrize("W,P,small", [(5, 16, False), (35, 81, True), (5, 23, False), (7, 13, False)])
def test_noalloc_matches_storage_entry_point(pkg, wl, W, P, small):
    torch = pytest.importorskip("torch")
    fn = _fn(pkg)
    text = wl.dna_copies(base_len=96 * 1024, copies=12, sub_rate=1e-3, seed=W + P)
    with pkg.Storage(len(text)) as st:
        want = st.trigger_scan(text, W, P, small)
    dT = torch.from_numpy(text).cuda()
    cap = len(text) + 2
    dD = torch.zeros(cap, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    flags = pkg.FLAG_SMALL_ALPHABET if small else 0
    for call in range(2):
        dD.fill_(-1)
        torch.cuda.synchronize()
        z = fn(dT.data_ptr(), len(text), W, P, flags, dD.data_ptr(), cap, stream)
        assert z == len(want), (call, z, len(want))
        got = dD[:z].cpu().numpy().astype(np.int64)
        assert np.array_equal(got, want), call


@pytest.mark.parametrize("n", [20 * (1 << 20) + 12345, 32 * (1 << 20)])
def test_noalloc_large_text_matches_oracle(pkg, wl, orc, n):
    # more than 4096 CTAs of 4 KiB: the per-CTA counts are scanned in several tiles
    # (reduce, scan of the tile partials, down-sweep); 32 MiB is an exact multiple of
    # one scan tile's 16 MiB.  Compared with the oracle's trigger scan directly.
    torch = pytest.importorskip("torch")
    fn = _fn(pkg)
    base = wl.config1_text()
    text = np.resize(base, n).astype(np.uint8)
    text[::7919] = 5                                  # the copies are not identical
    want = orc.trigger_scan(text, 5, 16)
    dT = torch.from_numpy(text).cuda()
    cap = n + 1                                       # z <= n - W + 1 always fits
    dD = torch.zeros(cap, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    for call in range(2):
        dD.fill_(-1)
        torch.cuda.synchronize()
        z = fn(dT.data_ptr(), n, 5, 16, 0, dD.data_ptr(), cap, stream)
        assert z == len(want), (call, z, len(want))
        assert np.array_equal(dD[:z].cpu().numpy().astype(np.int64), want), call


def test_noalloc_limits_and_errors(pkg):
    torch = pytest.importorskip("torch")
    fn = _fn(pkg)
    buf = torch.full((64,), 3, dtype=torch.uint8, device="cuda")
    out = torch.zeros(64, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    # beyond the stated maximum size: rejected before any device work
    assert fn(buf.data_ptr(), (1 << 30) + 1, 5, 16, 0, out.data_ptr(), 64, stream) == pkg.BAD_PARAMETER
    # output too small for the phrase ends
    assert fn(buf.data_ptr(), 64, 1, 1, 0, out.data_ptr(), 2, stream) == pkg.BAD_PARAMETER
    # invalid byte
    buf[10] = 0
    assert fn(buf.data_ptr(), 64, 5, 16, 0, out.data_ptr(), 64, stream) == pkg.BAD_PARAMETER
    # a valid call afterwards still works (the scratch is cleared per call)
    buf[10] = 3
    assert fn(buf.data_ptr(), 64, 5, 16, 0, out.data_ptr(), 64, stream) >= 1
