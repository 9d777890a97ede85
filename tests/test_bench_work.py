"""The algorithmic work bench.py reports: the rings holding galaxies
(`sky_rings`, with the oracle's ang2pix standing in for the GPU one) and the
per-stage counts built on them (`stage_work`)."""

import importlib.util
import os
import types

import numpy as np
import pytest

from oracle import healpix as oh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


STUB = types.SimpleNamespace(ang2pix_ring=lambda ns, th, ph: np.asarray(oh.ang2pix_ring(ns, th, ph)))


def _ring_lengths(ns):
    return np.array([4 * i if i < ns else (4 * ns if i <= 3 * ns else 4 * (4 * ns - i)) for i in range(1, 4 * ns)])


@pytest.mark.parametrize("ns", [4, 16])
def test_sky_rings_full_sky(ns):
    b = _bench()
    rng = np.random.default_rng(ns)
    n = 200 * 12 * ns * ns
    th, ph = np.arccos(rng.uniform(-1, 1, n)), rng.uniform(0, 2 * np.pi, n)
    pix, rings, live = b.sky_rings(STUB, ns, th, ph)
    assert pix == 12 * ns * ns and live == 12 * ns * ns and rings == 4 * ns - 1


def test_sky_rings_cap_and_band():
    b = _bench()
    ns = 16
    lens = _ring_lengths(ns)
    rng = np.random.default_rng(3)
    # northern cap z > 0.5: rings counted from the pixels the galaxies fall in
    th, ph = np.arccos(rng.uniform(0.5, 1, 200_000)), rng.uniform(0, 2 * np.pi, 200_000)
    pix, rings, live = b.sky_rings(STUB, ns, th, ph)
    gp = np.asarray(oh.ang2pix_ring(ns, th, ph))
    starts = np.concatenate([[0], np.cumsum(lens)])
    ring_of = np.searchsorted(starts, gp, side="right") - 1          # 0-based ring of each galaxy
    used = np.unique(ring_of)
    assert live == lens[used].sum()
    k = used.max() + 1                                                # pairs 0 .. k-1 (all northern)
    assert rings == 2 * k and pix == 2 * lens[:k].sum()
    # a band |z| < 0.3: the span starts past the pole
    th = np.arccos(rng.uniform(-0.3, 0.3, 200_000))
    pix, rings, live = b.sky_rings(STUB, ns, th, ph)
    ring_of = np.searchsorted(starts, np.asarray(oh.ang2pix_ring(ns, th, ph)), side="right") - 1
    pairs = np.unique(np.minimum(ring_of, 4 * ns - 2 - ring_of))
    lo, hi = pairs.min(), pairs.max()
    assert rings == 2 * (hi - lo + 1) - (1 if hi == 2 * ns - 1 else 0)
    assert live == lens[np.unique(ring_of)].sum()


def test_stage_work_counts_the_rings_with_data():
    b = _bench()
    nm, ngal, nbasis = 328, 10_000_000, 327
    npix = 12 * b.NSIDE ** 2
    sky = (npix // 2, 640, npix // 4)
    full = dict((st, b.stage_work(st, "mixed", nm, ngal, nbasis)) for st in ("deposit", "leg_analysis"))
    part = dict((st, b.stage_work(st, "mixed", nm, ngal, nbasis, sky=sky)) for st in ("deposit", "leg_analysis"))
    # maps are written as double-float pairs, 8 B per value
    assert part["deposit"][1] == pytest.approx(40.0 * ngal + 8.0 * nbasis * npix / 4)
    assert full["deposit"][1] == pytest.approx(40.0 * ngal + 8.0 * nbasis * npix)
    assert part["leg_analysis"][1] < full["leg_analysis"][1]
    # the FP64 path computes every ring: the sky does not change its counts
    assert b.stage_work("deposit", "fp64", nm, ngal, nbasis, sky=sky) == b.stage_work("deposit", "fp64", nm, ngal,
                                                                                       nbasis)


def test_batched_mock_generator():
    """The batched-mocks bench: uneven sizes in [1e6, 2e7], offsets over the concatenation, every
    mock inside the window's support (cap and radial range), independent seeds per mock, and the
    inverse-CDF radial draw matching the rejection sampler of the single-catalogue bench."""
    b = _bench()
    sizes = b.mock_sizes(64)
    assert sizes.min() >= 1_000_000 and sizes.max() <= 20_000_000 and len(np.unique(sizes)) > 60
    small = np.array([20_000, 0, 50_000, 7])
    gal = np.full((small.sum(), 3), np.nan)
    w = np.full(small.sum(), np.nan)
    off = b.fill_mocks(small, gal, w)
    assert list(off) == [0, 20_000, 20_000, 70_000, 70_007]
    assert np.all(np.isfinite(gal)) and np.all(np.isfinite(w))
    assert gal[:, 0].min() >= b.RMIN and gal[:, 0].max() <= b.RMAX
    assert gal[:, 1].max() <= np.radians(b.CAP_DEG) + 1e-12 and gal[:, 1].min() >= 0.0
    assert np.all((gal[:, 2] >= 0) & (gal[:, 2] < 2 * np.pi)) and np.all((w >= 0.5) & (w < 1.5))
    assert not np.allclose(gal[:7, 0], gal[20_000:20_007, 0])
    # radial distribution against the rejection sampler (histogram within Poisson noise)
    b.NGAL_MEAN = 200_000
    ref, _ = b.make_catalogue(seed=5)
    edges = np.linspace(b.RMIN, b.RMAX, 9)
    h1 = np.histogram(gal[20_000:70_000, 0], edges)[0] / 50_000
    h2 = np.histogram(ref[:, 0], edges)[0] / ref.shape[0]
    assert np.all(np.abs(h1 - h2) < 5 * np.sqrt(h2 / 50_000) + 1e-3)


class _FakeTensor:
    """Host stand-in for the pinned torch tensors of the batched extra (no device here)."""

    def __init__(self, a):
        self.a = a

    def pin_memory(self):
        return self

    def numpy(self):
        return self.a

    def data_ptr(self):
        return self.a.ctypes.data

    def __getitem__(self, sl):
        return _FakeTensor(self.a[sl])


def test_batched_extra_plumbing():
    """batched_mocks_bench on the host with a stand-in library: every mock reaches the batched call with
    its offsets and n-bar, the per-mock rows come back in order, and the single-call comparison reads
    the same galaxies (pointer arithmetic of the row slices)."""
    import ctypes as C
    b = _bench()
    from sfbgpu import _capi as capi
    nlm = 5

    def as_arr(ptr, n):
        return np.ctypeslib.as_array(C.cast(ptr.value, C.POINTER(C.c_double)), (n,))

    def signature(gal, w, nbar):
        # a row that depends on every galaxy of the mock: sums of r, w and r*w, scaled by 1/nbar
        s = np.array([gal[:, 0].sum(), w.sum(), (gal[:, 0] * w).sum(), len(w), 1.0 / nbar])
        return np.stack([s, -s], axis=1).ravel()

    class Lib:
        def sfb_cat2amln_batched(self, h, gp, wp, op, nm, nbp, win, outp):
            off = np.ctypeslib.as_array(C.cast(op.value, C.POINTER(C.c_int64)), (nm + 1,))
            nb = as_arr(nbp, nm)
            gal = as_arr(gp, 3 * off[-1]).reshape(-1, 3)
            w = as_arr(wp, off[-1])
            out = as_arr(outp, nm * 2 * nlm).reshape(nm, 2 * nlm)
            for k in range(nm):
                out[k] = signature(gal[off[k]:off[k + 1]], w[off[k]:off[k + 1]], nb[k])
            return 0

        def sfb_cat2amln(self, h, gp, wp, n, nbar, win, outp):
            out = np.ctypeslib.as_array(C.cast(outp.value, C.POINTER(C.c_double)), (2 * nlm,))
            out[:] = signature(as_arr(gp, 3 * n).reshape(-1, 3), as_arr(wp, n), nbar)
            return 0

    fake_capi = types.SimpleNamespace(lib=Lib(), check=capi.check, Window=capi.Window, C=C, _dp=capi._dp,
                                      SFB_WINDOW_SEPARABLE=capi.SFB_WINDOW_SEPARABLE)
    fake_torch = types.SimpleNamespace(
        float64=np.float64, cuda=types.SimpleNamespace(synchronize=lambda: None),
        empty=lambda shape, dtype=None: _FakeTensor(np.empty(shape, np.float64)),
        from_numpy=lambda a: _FakeTensor(a))
    b.mock_sizes = lambda n, seed=7: np.array([3000, 1000, 2500])[:n]
    plan = types.SimpleNamespace(handle=None)
    rec = b.batched_mocks_bench(3, 2, fake_capi, fake_torch, plan, np.ones(12), np.ones((2, 3)), 10.0, nlm)
    assert rec["mocks"] == 3 and rec["galaxies"] == 6500 and rec["repeats"] == 2
    assert rec["rows_vs_single_calls_max_rel_diff"] == 0.0
    assert rec["h2d_bytes_per_batch"] == 32 * 6500 and rec["d2h_bytes_per_batch"] == 16 * nlm * 3
