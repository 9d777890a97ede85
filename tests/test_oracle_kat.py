"""The oracle pinned against the reference's own known-answer tests and the
closed-form fixtures in tests/golden (CPU only)."""

import os

import numpy as np
import pytest

import sfbgpu
from helpers import catalogue, modes_dict, rel_err, round_sig, ylm
from oracle import healpix as ohp, sfb as osfb, sht as osht

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_kat.npz"))


def test_ylm_closed_forms():
    """reference test/test_toplevel.jl:20-51 (Condon-Shortley phase), extended to l = 2."""
    th, ph = GOLD["ylm_theta"], GOLD["ylm_phi"]
    for (l, m), val in zip(GOLD["ylm_lm"], GOLD["ylm_val"]):
        assert np.allclose(osht.ylm(int(l), int(m), th, ph), val, rtol=1e-14, atol=1e-15)


def test_healpix_golden_centres():
    for ns, th, ph in ((1, GOLD["hp1_theta"], GOLD["hp1_phi"]), (2, GOLD["hp2_theta"], GOLD["hp2_phi"])):
        t, p = ohp.pix2ang_ring(ns, np.arange(12 * ns * ns))
        assert np.allclose(t, th, atol=1e-14) and np.allclose(p, ph, atol=1e-14)
        assert np.array_equal(ohp.ang2pix_ring(ns, th, ph), np.arange(12 * ns * ns))


@pytest.mark.parametrize("nside", [1, 2, 3, 8, 64])
def test_healpix_round_trip(nside):
    pix = np.arange(12 * nside * nside)
    th, ph = ohp.pix2ang_ring(nside, pix)
    assert np.array_equal(ohp.ang2pix_ring(nside, th, ph), pix)
    th2, ph2 = sfbgpu.pix2ang_ring(nside, pix)
    assert np.allclose(th, th2, atol=1e-13) and np.allclose(np.mod(ph - ph2 + 1, 2 * np.pi) - 1, 0, atol=1e-13)


def test_map2alm_recovers_bandlimited_alm():
    nside, lmax = 16, 16
    S = osht.SHT(nside, lmax)
    rng = np.random.default_rng(2)
    alm = rng.normal(size=(lmax + 1, lmax + 1)) + 1j * rng.normal(size=(lmax + 1, lmax + 1))
    alm = np.tril(alm)
    alm[:, 0] = alm[:, 0].real
    back = S.map2alm(S.synthesis(alm), niter=3)
    assert rel_err(back, alm) < 1e-6
    assert rel_err(S.map2alm(S.synthesis(alm), niter=0), alm) < 1e-2


@pytest.mark.parametrize("niter", [0, 3])
def test_map2alm_matches_dense_definition_at_3nside(niter):
    """The oracle's map2alm at lmax = 3 nside - 1 (the regime no reference test reaches) against the
    same Jacobi iteration written with dense matrices of scipy's spherical harmonics at the pixel
    centres: analysis A f = (4 pi / npix) Y^H f, synthesis S a = Re(Y (c a)) with c = 1 for m = 0 and 2
    for m > 0 (a real map), a <- a + A (f - S a).  Independent of the oracle's Legendre recursion,
    ring FFTs, aliasing and phases; a random (not band-limited) map."""
    from scipy.special import sph_harm_y
    nside = 16
    lmax = 3 * nside - 1
    S = osht.SHT(nside, lmax)
    th, ph = ohp.pix2ang_ring(nside, np.arange(S.npix))
    lm = np.array([(l, m) for m in range(lmax + 1) for l in range(m, lmax + 1)])
    ls, ms = lm[:, 0], lm[:, 1]
    Y = sph_harm_y(ls[None, :], ms[None, :], th[:, None], ph[:, None])
    w = 4 * np.pi / S.npix
    c = np.where(ms == 0, 1.0, 2.0)
    f = np.random.default_rng(11).normal(size=S.npix)
    a = w * (Y.conj().T @ f)
    for _ in range(niter):
        a = a + w * (Y.conj().T @ (f - (Y @ (c * a)).real))
    got = S.map2alm(f, niter=niter)[ls, ms]
    assert rel_err(got, a) < 1e-12


def test_point_source_kat_oracle():
    """reference test/test_cat2anlm.jl:153-196 (nside 256, nmax 2, lmax 3, nr 100).

    field2anlm is linear and a zero shell contributes nothing, so each point
    source is evaluated with the one-shell configuration around its shell
    (same r_i and dr), which is the same formula with one SHT."""
    a = sfbgpu.AnlmModes.from_nmax_lmax(2, 3, 500.0, 1000.0, nside=256)
    md = modes_dict(a)
    nr, ns = 100, 256
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, nr, ns)
    S = osht.SHT(ns, a.lmax)
    Op = 4 * np.pi / wm.npix
    for j, i in ((0, 0), (3 * ns * ns + 7, 41)):
        f = np.zeros((1, wm.npix))
        f[0, j] = 1
        ri = wm.r[i]
        an1 = round_sig(osfb.field2anlm(f, ri - wm.dr / 2, ri + wm.dr / 2, 1, md, sht=S), 6)
        th, ph = ohp.pix2ang_ring(ns, j)
        an0 = np.empty_like(an1)
        for k in range(1, sfbgpu.getnlmsize(a) + 1):
            n, l, m = sfbgpu.getnlm(a, k)
            an0[k - 1] = round_sig(wm.dr * ri ** 2 * a.basisfunctions(n, l, ri)
                                   * np.conj(ylm(l, m, th, ph)) * Op, 6)
        assert np.linalg.norm(an0 - an1) <= 1e-5 * max(np.linalg.norm(an0), np.linalg.norm(an1))


def test_basis_function_kat_oracle():
    """reference test/test_cat2anlm.jl:32-67."""
    a = sfbgpu.AnlmModes(0.02, 0.0, 1000.0, nside=32)
    md = modes_dict(a)
    nr = 200
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, nr, 32)
    th, ph = ohp.pix2ang_ring(32, np.arange(wm.npix))
    S = osht.SHT(32, a.lmax)
    for idx in np.random.default_rng(1).integers(1, sfbgpu.getnlmsize(a) + 1, 4):
        n, l, m = sfbgpu.getnlm(a, int(idx))
        y = ylm(l, m, th, ph)
        yr = y.real if m == 0 else np.sqrt(2) * (-1) ** m * y.real
        W = osfb.win_rhat_ln_dense(np.outer(a.basisfunctions(n, l, wm.r), yr), a.rmin, a.rmax, nr, md)
        an = -osfb.cat2amln(np.zeros((3, 0)), md, 3e-4, ("dense", W), np.zeros(0), sht=S)
        k = int(idx) - 1
        assert abs(an[k] - (1 if m == 0 else (-1) ** m / np.sqrt(2))) < 1e-3
        assert np.max(np.abs(np.delete(an, k))) <= 2e-3


def test_field2anlm_v1_v2_oracle():
    """reference test/test_cat2anlm.jl:235-258."""
    a = sfbgpu.AnlmModes.from_nmax_lmax(4, 6, 500.0, 1000.0, nside=16)
    md = modes_dict(a)
    nr = 60
    f = np.random.default_rng(3).random((nr, 12 * 16 * 16))
    W = osfb.win_rhat_ln_dense(f, a.rmin, a.rmax, nr, md)
    v1 = -osfb.cat2amln(np.zeros((3, 0)), md, 1.0, ("dense", W), np.zeros(0))
    v2 = osfb.field2anlm(f, a.rmin, a.rmax, nr, md)
    assert np.allclose(v1, v2, rtol=np.sqrt(np.finfo(float).eps), atol=0)


def test_anlm2field_round_trip_oracle():
    """reference test/test_cat2anlm.jl:261-289."""
    a = sfbgpu.AnlmModes.from_nmax_lmax(4, 6, 500.0, 1000.0, nside=16)
    md = modes_dict(a)
    nr = 60
    f1 = np.random.default_rng(4).random((nr, 12 * 16 * 16))
    a1 = osfb.field2anlm(f1, a.rmin, a.rmax, nr, md)
    f2 = osfb.anlm2field(a1, a.rmin, a.rmax, nr, md)
    a2 = osfb.field2anlm(f2, a.rmin, a.rmax, nr, md)
    f3 = osfb.anlm2field(a2, a.rmin, a.rmax, nr, md)
    assert np.linalg.norm(f2 - f3) <= 1e-4 * np.linalg.norm(f2)
    assert np.linalg.norm(a1 - a2) <= 1e-4 * np.linalg.norm(a1)


def test_cat2amln_oracle_linearity_and_order():
    """cat2amln is linear in the weights and independent of galaxy order."""
    a = sfbgpu.AnlmModes(0.02, 500.0, 1000.0, nside=8)
    md = modes_dict(a)
    rtp, w = catalogue(2000, a.rmin, a.rmax, seed=5, weights=True)
    zero = ("separable", np.zeros(12 * 64), np.zeros((a.lmax + 1, a.nmax)))
    x1 = osfb.cat2amln(rtp, md, 1e-4, zero, w)
    x2 = osfb.cat2amln(rtp, md, 1e-4, zero, 2 * w)
    p = np.random.default_rng(6).permutation(rtp.shape[1])
    x3 = osfb.cat2amln(rtp[:, p], md, 1e-4, zero, w[p])
    assert rel_err(x2, 2 * x1) < 1e-14
    assert rel_err(x3, x1) < 1e-13


def test_splitmix64_known_answers():
    """The counter-based draws of apply_window: the published SplitMix64
    output sequence for state 1234567 (Steele, Lea, Flood 2014 reference
    generator), and uniforms in [0, 1) on the 2^-53 grid."""
    z = osfb.splitmix64(1234567, 5)
    assert [int(v) for v in z] == [6457827717110365317, 3203168211198807973, 9817491932198370423,
                                   4593380528125082431, 16408922859458223821]
    u = osfb.splitmix64_uniform(7, 100_000)
    assert u.min() >= 0.0 and u.max() < 1.0
    assert np.all(u * 2.0 ** 53 == np.floor(u * 2.0 ** 53))
    assert abs(u.mean() - 0.5) < 0.005


def test_apply_window_oracle_matches_reference_loop():
    """The vectorised oracle against a per-galaxy loop written as the
    reference's apply_window (src/windows.jl:169-216), on a catalogue that
    includes r == rmin, r == rmax, r beyond, and window values <= 0."""
    nside, nr, rmin, rmax = 8, 12, 500.0, 1000.0
    dr = (rmax - rmin) / nr
    rng = np.random.default_rng(3)
    win = rng.uniform(-0.2, 1.0, (nr, 12 * nside * nside))
    rtp, _ = catalogue(3000, rmin, rmax, seed=4, rpad=30.0)
    rtp[0, :3] = [rmin, rmax, rmin + 3 * dr]
    u = rng.random(rtp.shape[1])
    got = osfb.apply_window(rtp, win, rmin, rmax, dr, nside, u)
    oow = 1.0 / np.max(win)
    keep = []
    for i in range(rtp.shape[1]):
        r, th, ph = rtp[:, i]
        if not (rmin <= r <= rmax):
            continue
        ir = int(np.ceil((r - rmin) / dr))
        if ir == 0:
            ir = 1
        elif ir > nr:
            continue
        pix = int(ohp.ang2pix_ring(nside, np.array([th]), np.array([ph]))[0])
        if u[i] <= win[ir - 1, pix] * oow:
            keep.append(i)
    assert np.array_equal(got, rtp[:, keep])
    assert 0 < got.shape[1] < rtp.shape[1]
