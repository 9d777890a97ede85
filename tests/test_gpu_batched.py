"""Batched mock catalogues (sfb_cat2amln_batched) and their band-power
covariance, at a small geometry: every mock's a_nlm must equal the single-
catalogue call, and the band powers (amln2clnn, reference
src/SphericalFourierBesselDecompositions.jl:133-150) of the batch feed a
sample covariance that matches the one formed from separate calls."""

import numpy as np
import pytest

import sfbgpu
from helpers import modes_dict, record, rel_err
from oracle import sfb as osfb

pytestmark = pytest.mark.gpu


def _mocks(a, sizes, seed):
    """Seeded Poisson-like mocks in a polar cap x Gaussian shell (r^2 weighting by rejection)."""
    rng = np.random.default_rng(seed)
    cats, ws = [], []
    for n in sizes:
        r = [np.zeros(0)]
        while sum(len(x) for x in r) < n:
            x = rng.uniform(a.rmin, a.rmax, 4 * n + 100)
            keep = rng.random(x.size) * a.rmax ** 2 <= x ** 2 * np.exp(-((x - 750.0) / 150.0) ** 2) * 1.0
            r.append(x[keep])
        r = np.concatenate(r)[:n]
        mu = rng.uniform(np.cos(np.radians(60.0)), 1.0, n)
        ph = rng.uniform(0.0, 2 * np.pi, n)
        cats.append(np.stack([r, np.arccos(mu), ph]))
        ws.append(rng.uniform(0.5, 1.5, n))
    return cats, ws


def _window(a):
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, 100, a.nside)
    phi = np.exp(-((wm.r - 750.0) / 150.0) ** 2)
    th, _ = sfbgpu.pix2ang_ring(a.nside, np.arange(wm.npix))
    mask = (th < np.radians(60.0)).astype(float)
    return wm, phi, mask


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_mocks_equal_single_calls(precision):
    a = sfbgpu.AnlmModes(0.05, 500.0, 1000.0, nside=32)
    wm, phi, mask = _window(a)
    win = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, a)
    veff = sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    sizes = [40_000, 0, 125_000, 7, 80_000]                # uneven, an empty and a tiny mock
    cats, ws = _mocks(a, sizes, 41)
    nbars = [max(n, 1) / veff for n in sizes]
    batch = sfbgpu.cat2amln_batched(cats, a, nbars, win, ws, precision=precision)
    tol = 1e-12 if precision == "fp64" else 1e-9
    for k in range(len(sizes)):
        single = sfbgpu.cat2amln(cats[k], a, nbars[k], win, ws[k], precision=precision)
        e = rel_err(batch[k], single)
        record(f"batched_vs_single_{precision}_mock{k}", e, ngal=sizes[k])
        assert e < tol, (k, e)


def test_batched_band_power_covariance():
    """Band powers of a batch of mocks and their sample covariance; the first
    mock's spectrum against the oracle's amln2clnn."""
    a = sfbgpu.AnlmModes(0.03, 500.0, 1000.0, nside=16)
    wm, phi, mask = _window(a)
    win = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, a)
    veff = sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    rng = np.random.default_rng(5)
    sizes = list(rng.integers(20_000, 60_000, 12))
    cats, ws = _mocks(a, sizes, 43)
    nbars = [n / veff for n in sizes]
    anlm = sfbgpu.cat2amln_batched(cats, a, nbars, win, ws, precision="fp64")
    cm = sfbgpu.ClnnModes(a, dnmax=1)
    clnn = sfbgpu.amln2clnn(anlm, cm)                     # (nmocks, nlnn)
    single = np.array([sfbgpu.amln2clnn(anlm[k], cm) for k in range(len(sizes))])
    assert rel_err(clnn, single) < 1e-14
    cov = np.cov(clnn, rowvar=False)
    cov_ref = np.cov(single, rowvar=False)
    assert rel_err(cov, cov_ref) < 1e-12
    md = modes_dict(a)
    e = rel_err(clnn[0], osfb.amln2clnn(anlm[0], anlm[0], cm.lnn, md))
    record("batched_band_power_vs_oracle", e)
    assert e < 1e-14
