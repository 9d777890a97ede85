"""Mixed precision (FP32 ring FFT, split-BF16 tcgen05 contractions, FP64
deposit/tables/projection/window) against the FP64 GPU path and the oracle.

Error measure: max|mixed - fp64| / max|fp64| over all a_nlm (global), and the
per-mode relative error over modes with |a| above 1e-3 max|a| (recorded)."""

import numpy as np
import pytest

import sfbgpu
from helpers import catalogue, modes_dict, record, rel_err
from oracle import sfb as osfb

pytestmark = pytest.mark.gpu


def _setup(kmax, rmin, rmax, nside, ngal, seed):
    a = sfbgpu.AnlmModes(kmax, rmin, rmax, nside=nside)
    rtp, w = catalogue(ngal, rmin, rmax, seed=seed, weights=True)
    wm = sfbgpu.ConfigurationSpaceModes(rmin, rmax, 100, nside)
    phi = np.exp(-((wm.r - 0.5 * (rmin + rmax)) / (0.3 * (rmax - rmin))) ** 2)
    mask = sfbgpu.gen_mask(nside, 0.75)
    win = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, a)
    nbar = ngal / sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    return a, rtp, w, win, nbar


# the mixed path's accuracy bar: ||a_mixed - a_ref|| / ||a_ref|| <= 1e-7
MIXED_TOL = 1e-7


@pytest.mark.parametrize("cfg", [(0.03, 500.0, 1000.0, 16, 50_000, 1), (0.05, 500.0, 1000.0, 32, 200_000, 2)])
def test_mixed_vs_fp64(cfg):
    kmax, rmin, rmax, nside, ngal, seed = cfg
    a, rtp, w, win, nbar = _setup(*cfg)
    f64 = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="fp64")
    mix = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed")
    e = rel_err(mix, f64)
    big = np.abs(f64) > 1e-3 * np.max(np.abs(f64))
    per_mode = float(np.max(np.abs(mix - f64)[big] / np.abs(f64)[big]))
    record(f"mixed_vs_fp64_kmax{kmax}_nside{nside}", e, per_mode_rel_above_1em3=per_mode)
    assert e < MIXED_TOL


def test_mixed_vs_reference_algorithm():
    a, rtp, w, win, nbar = _setup(0.03, 500.0, 1000.0, 16, 50_000, 3)
    md = modes_dict(a)
    ref = osfb.cat2amln(rtp, md, nbar, ("separable", win.mask, win.w_ln), w)
    mix = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed")
    e = rel_err(mix, ref)
    record("mixed_vs_reference_algorithm", e)
    assert e < MIXED_TOL


def test_bounded_wait_times_out_and_context_survives():
    """A device wait with no arrival expires, is reported as SFB_ETIMEOUT, and
    the next transform still runs (failure detection without a GPU fault)."""
    from sfbgpu import _capi as capi
    assert capi.lib.sfb_selftest_wait_timeout() == capi.SFB_ETIMEOUT
    a = sfbgpu.AnlmModes(0.02, 500.0, 1000.0, nside=8)
    rtp, w = catalogue(1000, a.rmin, a.rmax, seed=4)
    out = sfbgpu.cat2amln(rtp, a, 1e-4, None, None, precision="mixed")
    assert np.all(np.isfinite(out))
