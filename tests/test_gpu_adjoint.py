"""Adjoints of the transforms (FP64): dot-product tests <J x, y> = <x, J^T y>
for map2alm (niter refinement included), cat2amln (the galaxy weights) and
field2anlm (the shell x pixel field), and gradients of the loss
L = sum |a_nlm - t_nlm|^2 against central finite differences — of this
library's forward transform (L is quadratic, so the differences are exact up
to rounding) and of the oracle's reference algorithm."""

import numpy as np
import pytest

import sfbgpu
from helpers import catalogue, modes_dict, record
from oracle import sfb as osfb

pytestmark = pytest.mark.gpu


def _rdot(a, b):
    """Real inner product of complex vectors viewed as (re, im) pairs."""
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.sum(a.real * b.real + a.imag * b.imag))


def _rel(x, y):
    return abs(x - y) / max(abs(x), abs(y))


@pytest.mark.parametrize("nmaps,nside,lmax,niter", [(3, 16, 31, 3), (1, 16, 40, 3), (2, 8, 23, 0), (4, 32, 40, 3)])
def test_map2alm_adjoint_dot(nmaps, nside, lmax, niter):
    a = sfbgpu.AnlmModes.from_nmax_lmax(1, lmax, 500.0, 1000.0, nside=nside, cache=True)
    rng = np.random.default_rng(nmaps + nside)
    f = rng.normal(size=(nmaps, 12 * nside * nside))
    ab = rng.normal(size=(nmaps, (lmax + 1) * (lmax + 2) // 2)) + 1j * rng.normal(size=(nmaps, (lmax + 1) * (lmax + 2) // 2))
    alm = sfbgpu.cat2anlm.map2alm(f, a, niter=niter, radial="spline")
    fb = sfbgpu.cat2anlm.map2alm_adjoint(ab, a, niter=niter, radial="spline")
    lhs, rhs = _rdot(alm, ab), float(np.sum(f * fb))
    e = _rel(lhs, rhs)
    record(f"map2alm_adjoint_dot_{nmaps}maps_nside{nside}_lmax{lmax}_niter{niter}", e)
    assert e < 1e-12


def _setup_cat(seed=21):
    a = sfbgpu.AnlmModes(0.03, 500.0, 1000.0, nside=16)
    rtp, w = catalogue(20_000, a.rmin, a.rmax, seed=seed, weights=True, rpad=20.0)
    nbar = rtp.shape[1] / (4 / 3 * np.pi * (a.rmax ** 3 - a.rmin ** 3))
    return a, rtp, w, nbar


def test_cat2amln_vjp_dot():
    """a(w) is linear in w for a zero window: <a(dw), abar> = <dw, vjp(abar)>."""
    a, rtp, w, nbar = _setup_cat()
    rng = np.random.default_rng(3)
    dw = rng.normal(size=w.size)
    ab = rng.normal(size=sfbgpu.getnlmsize(a)) + 1j * rng.normal(size=sfbgpu.getnlmsize(a))
    a_dw = sfbgpu.cat2amln(rtp, a, nbar, None, dw, precision="fp64", radial="poly")
    g = sfbgpu.cat2amln_vjp(rtp, a, nbar, ab, precision="fp64", radial="poly")
    e = _rel(_rdot(a_dw, ab), float(np.dot(dw, g)))
    record("cat2amln_vjp_dot", e)
    assert e < 1e-11


def test_field2anlm_vjp_dot():
    a = sfbgpu.AnlmModes(0.03, 500.0, 1000.0, nside=16)
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, 40, a.nside)
    rng = np.random.default_rng(4)
    f = rng.normal(size=(wm.nr, wm.npix)).astype(np.float32).astype(float)
    ab = rng.normal(size=sfbgpu.getnlmsize(a)) + 1j * rng.normal(size=sfbgpu.getnlmsize(a))
    an = sfbgpu.field2anlm(f, wm, a)
    fb = sfbgpu.field2anlm_vjp(ab, wm, a)
    assert fb.shape == f.shape
    e = _rel(_rdot(an, ab), float(np.sum(f * fb)))
    record("field2anlm_vjp_dot", e)
    assert e < 1e-11


def test_cat2amln_weight_gradient_finite_differences():
    """dL/dw_i for L = sum |a - t|^2 (separable window) against central
    differences of L through this library's forward transform (exact for a
    quadratic) and through the oracle's reference algorithm (spline radial
    functions; the poly basis differs from them by ~1e-7)."""
    a, rtp, w, nbar = _setup_cat(22)
    md = modes_dict(a)
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, 50, a.nside)
    phi = np.exp(-((wm.r - 750.0) / 200.0) ** 2)
    mask = sfbgpu.gen_mask(a.nside, 0.6)
    _, wln = osfb.win_rhat_ln_separable(phi, mask, a.rmin, a.rmax, 50, md)
    win = sfbgpu.SeparableArray(mask, wln, "mask", "w_ln")
    rng = np.random.default_rng(9)
    a0 = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="fp64", radial="poly")
    t = a0 + 0.3 * np.abs(a0).max() * (rng.normal(size=a0.size) + 1j * rng.normal(size=a0.size))

    def loss(wv):
        return float(np.sum(np.abs(sfbgpu.cat2amln(rtp, a, nbar, win, wv, precision="fp64", radial="poly") - t) ** 2))

    g = sfbgpu.cat2amln_vjp(rtp, a, nbar, 2.0 * (a0 - t), precision="fp64", radial="poly")
    idx = rng.choice(w.size, 5, replace=False)
    h = 0.25
    for i in idx:
        wp, wmn = w.copy(), w.copy()
        wp[i] += h
        wmn[i] -= h
        fd = (loss(wp) - loss(wmn)) / (2 * h)
        e = _rel(fd, g[i])
        record("cat2amln_weight_gradient_vs_fd", e, galaxy=int(i))
        assert e < 1e-6, (i, fd, g[i])

    def loss_oracle(wv):
        return float(np.sum(np.abs(osfb.cat2amln(rtp, md, nbar, ("separable", mask, wln), wv) - t) ** 2))

    for i in idx[:2]:
        wp, wmn = w.copy(), w.copy()
        wp[i] += h
        wmn[i] -= h
        fd = (loss_oracle(wp) - loss_oracle(wmn)) / (2 * h)
        e = _rel(fd, g[i])
        record("cat2amln_weight_gradient_vs_oracle_fd", e, galaxy=int(i))
        assert e < 1e-5, (i, fd, g[i])


def test_field2anlm_gradient_finite_differences():
    a = sfbgpu.AnlmModes(0.03, 500.0, 1000.0, nside=16)
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, 30, a.nside)
    rng = np.random.default_rng(6)
    f = rng.normal(size=(wm.nr, wm.npix))
    a0 = sfbgpu.field2anlm(f, wm, a)
    t = a0 + 0.2 * np.abs(a0).max() * (rng.normal(size=a0.size) + 1j * rng.normal(size=a0.size))
    g = sfbgpu.field2anlm_vjp(2.0 * (a0 - t), wm, a)
    h = 0.5
    for _ in range(4):
        s, p = int(rng.integers(wm.nr)), int(rng.integers(wm.npix))
        fp, fm = f.copy(), f.copy()
        fp[s, p] += h
        fm[s, p] -= h
        lp = float(np.sum(np.abs(sfbgpu.field2anlm(fp, wm, a) - t) ** 2))
        lm = float(np.sum(np.abs(sfbgpu.field2anlm(fm, wm, a) - t) ** 2))
        fd = (lp - lm) / (2 * h)
        e = _rel(fd, g[s, p])
        record("field2anlm_gradient_vs_fd", e)
        assert e < 1e-6, (s, p, fd, g[s, p])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_field2anlm_fp32_field_and_shell_streaming(precision, monkeypatch):
    """An FP32 field (sfb_field2anlm_typed) gives exactly what its FP64 copy
    gives; the FP32 gradient is the FP64 one rounded; and a field streamed
    through the device six shells at a time (SFBGPU_FIELD_MAX_BYTES of six
    FP32 shells) matches the resident field to the rounding of the radial
    sum's grouping (1e-12).  Six shells per chunk keep the mixed transform on
    the same refinement scheme as the resident 24-shell batch (a batch of at
    most four maps takes the full refinement passes, a different rounding)."""
    a = sfbgpu.AnlmModes(0.03, 500.0, 1000.0, nside=16)
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, 24, a.nside)
    rng = np.random.default_rng(31)
    f32 = rng.normal(size=(wm.nr, wm.npix)).astype(np.float32)
    r64 = sfbgpu.field2anlm(f32.astype(float), wm, a, precision=precision)
    r32 = sfbgpu.field2anlm(f32, wm, a, precision=precision)
    np.testing.assert_array_equal(r32, r64)
    ab = rng.normal(size=r64.size) + 1j * rng.normal(size=r64.size)
    g64 = sfbgpu.field2anlm_vjp(ab, wm, a, precision=precision)
    g32 = sfbgpu.field2anlm_vjp(ab, wm, a, dtype=np.float32, precision=precision)
    assert g32.dtype == np.float32
    np.testing.assert_array_equal(g32, g64.astype(np.float32))
    monkeypatch.setenv("SFBGPU_FIELD_MAX_BYTES", str(6 * 4 * wm.npix))
    b = sfbgpu.AnlmModes(0.03, 500.0, 1000.0, nside=16)
    s32 = sfbgpu.field2anlm(f32, wm, b, precision=precision)
    gs = sfbgpu.field2anlm_vjp(ab, wm, b, precision=precision)
    gs32 = sfbgpu.field2anlm_vjp(ab, wm, b, dtype=np.float32, precision=precision)
    e = float(np.max(np.abs(s32 - r32)) / np.max(np.abs(r32)))
    eg = float(np.max(np.abs(gs - g64)) / np.max(np.abs(g64)))
    record(f"field2anlm_streamed_vs_resident_{precision}", e, vjp=eg)
    assert e < 1e-12 and eg < 1e-12
    np.testing.assert_array_equal(gs32, gs.astype(np.float32))
