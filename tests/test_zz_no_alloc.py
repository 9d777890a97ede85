"""The allocation-free weight gather (sfb_winweights2galweights_noalloc)
against the allocating entry point, called through the C ABI.

Tolerance: exact equality.  Both entry points run the same gather kernel on
the same doubles, so every weight must be bit-identical.
"""

import ctypes as C

import numpy as np
import pytest

from helpers import catalogue

pytestmark = pytest.mark.gpu

capi = pytest.importorskip("sfbgpu._capi")


def _inputs(nside, nr, ngal, seed):
    rng = np.random.default_rng(seed)
    rb = np.linspace(500.0, 1000.0, nr + 1)
    npix = 12 * nside * nside
    W = np.asfortranarray(rng.random((nr, npix)))      # element (bin, pix) at bin + nr*pix
    rtp, _ = catalogue(ngal, 500.0, 1000.0, seed=seed + 1)
    rtp[0, :4] = [500.0, 1000.0, rb[3], rb[nr - 1]]
    gal = np.ascontiguousarray(rtp.T)
    return W, rb, gal


def _call(fn, nside, W, rb, gal):
    out = np.full(gal.shape[0], np.nan)
    st = fn(nside, C.c_void_p(W.ctypes.data), W.shape[0], C.c_void_p(rb.ctypes.data),
            C.c_void_p(gal.ctypes.data), gal.shape[0], C.c_void_p(out.ctypes.data))
    return st, out


def test_noalloc_matches_allocating_entry_twice():
    # nside 64, nr 30: 1.47M-double table, so 400k galaxies take three staged chunks
    nside, nr = 64, 30
    W, rb, gal = _inputs(nside, nr, 400_000, 21)
    st, ref = _call(capi.lib.sfb_winweights2galweights, nside, W, rb, gal)
    assert st == capi.SFB_OK, capi.last_error()
    for _ in range(2):
        st, out = _call(capi.lib.sfb_winweights2galweights_noalloc, nside, W, rb, gal)
        assert st == capi.SFB_OK, capi.last_error()
        np.testing.assert_array_equal(out, ref)


def test_noalloc_error_word_is_cleared_between_calls():
    nside, nr = 16, 8
    W, rb, gal = _inputs(nside, nr, 10_000, 31)
    bad = gal.copy()
    bad[5, 0] = 1001.0
    st, _ = _call(capi.lib.sfb_winweights2galweights_noalloc, nside, W, rb, bad)
    assert st == capi.SFB_ERANGE
    st, out = _call(capi.lib.sfb_winweights2galweights_noalloc, nside, W, rb, gal)
    assert st == capi.SFB_OK, capi.last_error()
    st, ref = _call(capi.lib.sfb_winweights2galweights, nside, W, rb, gal)
    assert st == capi.SFB_OK
    np.testing.assert_array_equal(out, ref)


def test_noalloc_rejects_table_beyond_scratch():
    nside, nr = 128, 11          # 11 * 196608 + 12 doubles > 2080736
    rb = np.linspace(500.0, 1000.0, nr + 1)
    W = np.zeros((nr, 12 * nside * nside), order="F")
    gal = np.array([[700.0, 1.0, 1.0]])
    st, _ = _call(capi.lib.sfb_winweights2galweights_noalloc, nside, W, rb, gal)
    assert st == capi.SFB_EINVAL
    assert "static scratch maximum" in capi.last_error()


def test_noalloc_runs_with_device_memory_taken():
    """The property the entry point exists for: with nearly all device memory
    held by another allocator (here a PyTorch tensor), the allocating entry
    point fails with SFB_ENOMEM while the allocation-free one still returns
    the same weights."""
    torch = pytest.importorskip("torch")
    nside, nr = 64, 30
    W, rb, gal = _inputs(nside, nr, 2_000_000, 41)      # the allocating call needs ~76 MB
    st, ref = _call(capi.lib.sfb_winweights2galweights, nside, W, rb, gal)
    assert st == capi.SFB_OK, capi.last_error()
    st, _ = _call(capi.lib.sfb_winweights2galweights_noalloc, nside, W, rb, gal[:10])   # set-up done
    assert st == capi.SFB_OK, capi.last_error()
    torch.cuda.synchronize()
    keep = 32 << 20
    hold = None
    try:
        free, _ = torch.cuda.mem_get_info()
        hold = torch.empty(max(free - keep, 0), dtype=torch.uint8, device="cuda")
        free_after, _ = torch.cuda.mem_get_info()
        assert free_after < 64 << 20
        st, _ = _call(capi.lib.sfb_winweights2galweights, nside, W, rb, gal)
        assert st == capi.SFB_ENOMEM
        for _ in range(2):
            st, out = _call(capi.lib.sfb_winweights2galweights_noalloc, nside, W, rb, gal)
            assert st == capi.SFB_OK, capi.last_error()
            np.testing.assert_array_equal(out, ref)
        # no device memory taken by the calls (the driver may release some of its own)
        assert torch.cuda.mem_get_info()[0] >= free_after
    finally:
        del hold
        torch.cuda.empty_cache()
