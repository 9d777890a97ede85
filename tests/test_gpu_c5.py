"""The adjoint configuration at full size: kmax 0.15, r in [500, 2500],
nside 512, 512 radial shells, an FP32 N(0, 1) field and a 5e6-galaxy
catalogue, loss L = sum |a_nlm - t_nlm|^2 with seeded Gaussian targets.

* field: the mixed forward of the FP32 field against the FP64 forward (L2 and
  max-norm, 1e-7); dL/d(field) from field2anlm_vjp (FP64) against central
  differences of the FP64 forward along a random direction on four shells,
  1e-5 relative (L is quadratic, so the differences are exact up to
  rounding);
* weights: dL/dw from cat2amln_vjp against central differences of the FP64
  cat2amln along a random direction in the 5e6 weights, 1e-5 relative.

The small-size checks against the oracle's reference algorithm are in
test_gpu_adjoint.py."""

import numpy as np
import pytest

import sfbgpu
from helpers import catalogue, record

pytestmark = pytest.mark.gpu

NSIDE, NR, KMAX, RMIN, RMAX = 512, 512, 0.15, 500.0, 2500.0


@pytest.fixture(scope="module")
def c5():
    a = sfbgpu.AnlmModes(KMAX, RMIN, RMAX, nside=NSIDE)
    wm = sfbgpu.ConfigurationSpaceModes(RMIN, RMAX, NR, NSIDE)
    return a, wm


def _loss(x, t):
    d = x - t
    return float(np.sum(d.real * d.real + d.imag * d.imag))


def test_c5_field_gradient(c5):
    a, wm = c5
    npix = 12 * NSIDE * NSIDE
    rng = np.random.default_rng(50)
    delta = np.asfortranarray(rng.standard_normal((NR, npix), dtype=np.float32))
    n = sfbgpu.getnlmsize(a)
    t = rng.normal(size=n) + 1j * rng.normal(size=n)
    a64 = sfbgpu.field2anlm(delta, wm, a, precision="fp64")
    amx = sfbgpu.field2anlm(delta, wm, a, precision="mixed")
    e2 = float(np.linalg.norm(amx - a64) / np.linalg.norm(a64))
    emax = float(np.abs(amx - a64).max() / np.abs(a64).max())
    record("c5_field2anlm_mixed_vs_fp64", e2, maxnorm=emax, nlmsize=int(n))
    assert e2 < 1e-7 and emax < 1e-7

    g = sfbgpu.field2anlm_vjp(2.0 * (a64 - t), wm, a, dtype=np.float64, precision="fp64")
    shells = [3, 100, 300, NR - 1]
    v = rng.normal(size=(len(shells), npix))
    eps = 1e-3
    f = np.asfortranarray(delta, dtype=np.float64)
    del delta
    base = f[shells].copy()
    f[shells] = base + eps * v
    lp = _loss(sfbgpu.field2anlm(f, wm, a, precision="fp64"), t)
    f[shells] = base - eps * v
    lm = _loss(sfbgpu.field2anlm(f, wm, a, precision="fp64"), t)
    fd = (lp - lm) / (2 * eps)
    an = float(np.sum(g[shells] * v))
    e = abs(fd - an) / abs(fd)
    record("c5_field_gradient_vs_central_differences", e, shells=len(shells), eps=eps)
    assert e < 1e-5


def test_c5_weight_gradient(c5):
    a, _ = c5
    ngal = 5_000_000
    rtp, w = catalogue(ngal, RMIN, RMAX, seed=51, weights=True)
    nbar = ngal / (4 / 3 * np.pi * (RMAX ** 3 - RMIN ** 3))
    rng = np.random.default_rng(52)
    n = sfbgpu.getnlmsize(a)
    t = rng.normal(size=n) + 1j * rng.normal(size=n)
    opts = dict(precision="fp64", radial="poly")
    a0 = sfbgpu.cat2amln(rtp, a, nbar, None, w, **opts)
    g = sfbgpu.cat2amln_vjp(rtp, a, nbar, 2.0 * (a0 - t), **opts)
    u = rng.normal(size=ngal)
    eps = 1e-3
    lp = _loss(sfbgpu.cat2amln(rtp, a, nbar, None, w + eps * u, **opts), t)
    lm = _loss(sfbgpu.cat2amln(rtp, a, nbar, None, w - eps * u, **opts), t)
    fd = (lp - lm) / (2 * eps)
    an = float(np.dot(g, u))
    e = abs(fd - an) / abs(fd)
    record("c5_weight_gradient_vs_central_differences", e, ngal=ngal, eps=eps)
    assert np.all(np.isfinite(g)) and e < 1e-5
