"""Mixed precision (double-float maps and ring spectra, sliced-BF16 tcgen05
DFT and Legendre contractions, FP64 tables/projection/window terms) against
the FP64 GPU path and the oracle.

Error measures, both held to MIXED_TOL = 1e-7 in every case: the L2 relative
error ||a_mixed - a_ref||_2 / ||a_ref||_2 over the whole a_nlm vector and the
global max-norm error max|a_mixed - a_ref| / max|a_ref|.  The catalogues are
drawn from the window itself, so the data term and the window term cancel to
shot noise, as in a survey, which is the case that amplifies rounding."""

import numpy as np
import pytest

import sfbgpu
from helpers import catalogue, modes_dict, record, rel_err
from oracle import sfb as osfb

pytestmark = pytest.mark.gpu


def window_catalogue(ngal, rmin, rmax, fsky, seed, rmid=None, rsig=None):
    """Galaxies drawn from nbar * phi(r) * mask: r ~ r^2 phi(r) by rejection,
    directions uniform in the polar cap of gen_mask(fsky); weights U[0.5, 1.5]."""
    rng = np.random.default_rng(seed)
    rmid = 0.5 * (rmin + rmax) if rmid is None else rmid
    rsig = 0.3 * (rmax - rmin) if rsig is None else rsig
    f = lambda r: r * r * np.exp(-((r - rmid) / rsig) ** 2)
    fmax = f(np.linspace(rmin, rmax, 4001)).max() * 1.001
    rs, have = [], 0
    while have < ngal:
        r = rng.uniform(rmin, rmax, 2 * (ngal - have) + 1000)
        r = r[rng.random(r.size) * fmax <= f(r)]
        rs.append(r)
        have += r.size
    r = np.concatenate(rs)[:ngal]
    mu = rng.uniform(1.0 - 2.0 * fsky, 1.0, ngal)
    ph = rng.uniform(0.0, 2 * np.pi, ngal)
    return np.stack([r, np.arccos(mu), ph]), rng.uniform(0.5, 1.5, ngal), (lambda rr: np.exp(-((rr - rmid) / rsig) ** 2))


def _setup(kmax, rmin, rmax, nside, ngal, seed, kind="separable"):
    a = sfbgpu.AnlmModes(kmax, rmin, rmax, nside=nside)
    rtp, w, phif = window_catalogue(ngal, rmin, rmax, 0.75, seed)
    wm = sfbgpu.ConfigurationSpaceModes(rmin, rmax, 100, nside)
    phi = phif(wm.r)
    mask = sfbgpu.gen_mask(nside, 0.75)
    nbar = ngal / sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    if kind == "separable":
        win = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, a)
    elif kind == "dense":
        # separable part plus a direction-dependent radial tilt
        th, _ = sfbgpu.pix2ang_ring(nside, np.arange(wm.npix))
        tilt = 1.0 + 0.2 * np.cos(th)[None, :] * ((wm.r - 0.5 * (rmin + rmax)) / (rmax - rmin))[:, None]
        win = sfbgpu.win_rhat_ln(phi[:, None] * mask[None, :] * tilt, wm, a)
    else:
        win = None
    return a, rtp, w, win, nbar


def _errors(x, ref):
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref)), rel_err(x, ref)


# the mixed path's accuracy bar
MIXED_TOL = 1e-7


@pytest.mark.parametrize("cfg,kind", [((0.03, 500.0, 1000.0, 16, 50_000, 1), "separable"),
                                      ((0.05, 500.0, 1000.0, 32, 200_000, 2), "separable"),
                                      ((0.03, 500.0, 1000.0, 16, 50_000, 5), "dense"),
                                      ((0.03, 500.0, 1000.0, 16, 50_000, 6), "zero")])
def test_mixed_vs_fp64(cfg, kind):
    kmax, rmin, rmax, nside, ngal, seed = cfg
    a, rtp, w, win, nbar = _setup(*cfg, kind=kind)
    f64 = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="fp64")
    mix = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed")
    e2, emax = _errors(mix, f64)
    record(f"mixed_vs_fp64_{kind}_kmax{kmax}_nside{nside}", e2, maxnorm=emax)
    assert e2 < MIXED_TOL and emax < MIXED_TOL


@pytest.mark.parametrize("zlim", [(-0.3, 0.3), (-1.0, -0.4)])
def test_mixed_vs_fp64_partial_sky(zlim):
    """Surveys that leave rings empty at the start of the ring range (a band
    |z| < 0.3) or in the north (a southern cap): the ring DFT skips tiles of
    zero rows and the first analysis pass skips the zero ring chunks, which
    must leave the a_nlm unchanged."""
    z0, z1 = zlim
    a = sfbgpu.AnlmModes(0.05, 500.0, 1000.0, nside=32)
    rng = np.random.default_rng(12)
    n = 150_000
    r = np.cbrt(rng.uniform(a.rmin ** 3, a.rmax ** 3, n))
    rtp = np.stack([r, np.arccos(rng.uniform(z0, z1, n)), rng.uniform(0, 2 * np.pi, n)])
    w = rng.uniform(0.5, 1.5, n)
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, 100, a.nside)
    th, _ = sfbgpu.pix2ang_ring(a.nside, np.arange(wm.npix))
    mask = ((np.cos(th) > z0) & (np.cos(th) < z1)).astype(float)
    phi = np.ones(wm.nr)
    win = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, a)
    nbar = n / sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    f64 = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="fp64")
    mix = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed")
    e2, emax = _errors(mix, f64)
    record(f"mixed_vs_fp64_partial_sky_z{z0}_{z1}", e2, maxnorm=emax)
    assert e2 < MIXED_TOL and emax < MIXED_TOL


@pytest.mark.parametrize("env,val,name", [("SFBGPU_DFT_IMAGE_MAX_BYTES", "0", "polar_twiddles_gathered"),
                                          ("SFBGPU_DFT_AIMG", "0", "rows_sliced_in_producers"),
                                          ("SFBGPU_DFT_POLAR_GATHER", "1", "polar_gather_with_a_image"),
                                          ("SFBGPU_MOMENTS_SMEM", "0", "moments_in_registers")])
def test_kernel_variants_agree(monkeypatch, env, val, name):
    """The ring DFT takes its twiddle operand from the precomputed image and
    its map rows from the A image written by the slicing pass; the variants
    gather the polar twiddles from the ring tables (past the image budget, or
    by choice beside the A image) or slice the map rows in the DFT's producer
    warps, and the deposit's moments sum in registers or in shared memory.
    All do the same arithmetic, so the a_nlm agree to the run-to-run rounding
    of the deposit (the order of the galaxies within a bin)."""
    cfg = (0.05, 500.0, 1000.0, 32, 200_000, 8)
    a, rtp, w, win, nbar = _setup(*cfg)
    img = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed")
    monkeypatch.setenv(env, val)
    b = sfbgpu.AnlmModes(*cfg[:3], nside=cfg[3])
    alt = sfbgpu.cat2amln(rtp, b, nbar, win, w, precision="mixed")
    f64 = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="fp64")
    e_ia = _errors(alt, img)[0]
    record(f"dft_default_vs_{name}", e_ia)
    assert e_ia < 1e-9
    assert _errors(alt, f64)[0] < MIXED_TOL and _errors(img, f64)[0] < MIXED_TOL


def test_gram_refinement_matches_full_passes(monkeypatch):
    """The refinement passes of the mixed transform use the Gram matrices of
    the alias-free rings plus synthesis / fold / analysis over the aliased
    rings only; the full passes over every ring (SFBGPU_GRAM_REFINEMENT=0)
    compute the same a_lm up to rounding."""
    cfg = (0.05, 500.0, 1000.0, 32, 200_000, 9)
    a, rtp, w, win, nbar = _setup(*cfg)
    gram = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed")
    monkeypatch.setenv("SFBGPU_GRAM_REFINEMENT", "0")
    b = sfbgpu.AnlmModes(*cfg[:3], nside=cfg[3])
    full = sfbgpu.cat2amln(rtp, b, nbar, win, w, precision="mixed")
    f64 = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="fp64")
    e_gf = _errors(gram, full)[0]
    e_g, e_f = _errors(gram, f64)[0], _errors(full, f64)[0]
    record("gram_vs_full_refinement", e_gf, gram_vs_fp64=e_g, full_vs_fp64=e_f)
    assert e_g < MIXED_TOL and e_f < MIXED_TOL and e_gf < MIXED_TOL


def test_mixed_vs_reference_algorithm():
    a, rtp, w, win, nbar = _setup(0.03, 500.0, 1000.0, 16, 50_000, 3)
    md = modes_dict(a)
    ref = osfb.cat2amln(rtp, md, nbar, ("separable", win.mask, win.w_ln), w)
    mix = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed")
    e2, emax = _errors(mix, ref)
    record("mixed_vs_reference_algorithm", e2, maxnorm=emax)
    assert e2 < MIXED_TOL and emax < MIXED_TOL


def test_mixed_full_size():
    """The full-size geometry (kmax 0.1, r in [500, 2500], nside 256, 7520
    (n, l) pairs) with 2e6 galaxies in a 60-degree cap x Gaussian shell."""
    a = sfbgpu.AnlmModes(0.1, 500.0, 2500.0, nside=256)
    ngal = 2_000_000
    fsky = (1 - np.cos(np.radians(60.0))) / 2
    rtp, w, phif = window_catalogue(ngal, 500.0, 2500.0, fsky, 7, rmid=1500.0, rsig=400.0 * np.sqrt(2))
    wm = sfbgpu.ConfigurationSpaceModes(500.0, 2500.0, 1000, 256)
    phi = phif(wm.r)
    mask = sfbgpu.gen_mask(256, fsky)
    nbar = ngal / sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    win = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, a, radial="poly")
    f64 = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="fp64", radial="poly")
    mix = sfbgpu.cat2amln(rtp, a, nbar, win, w, precision="mixed", radial="poly")
    e2, emax = _errors(mix, f64)
    record("mixed_vs_fp64_full_size_nside256_kmax0.1", e2, maxnorm=emax)
    # ~1e6 coefficients: the largest single error, relative to the largest
    # coefficient, is held to the same bar as the L2 error
    assert e2 < MIXED_TOL and emax < MIXED_TOL


def test_field2anlm_mixed_vs_fp64():
    """field2anlm on a plan in mixed precision (tensor-core shell transforms of
    the FP32-rounded field, FP64 radial sum) against the FP64 plan."""
    a = sfbgpu.AnlmModes(0.05, 500.0, 1000.0, nside=32)
    wm = sfbgpu.ConfigurationSpaceModes(a.rmin, a.rmax, 64, a.nside)
    rng = np.random.default_rng(11)
    f = rng.normal(size=(wm.nr, wm.npix)).astype(np.float32).astype(float)
    f64 = sfbgpu.field2anlm(f, wm, a, precision="fp64")
    mix = sfbgpu.field2anlm(f, wm, a, precision="mixed")
    e2, emax = _errors(mix, f64)
    record("field2anlm_mixed_vs_fp64", e2, maxnorm=emax)
    assert e2 < MIXED_TOL and emax < MIXED_TOL


def test_bounded_wait_times_out_and_context_survives():
    """A device wait with no arrival expires, is reported as SFB_ETIMEOUT, and
    the next transform still runs (failure detection without a GPU fault)."""
    from sfbgpu import _capi as capi
    assert capi.lib.sfb_selftest_wait_timeout() == capi.SFB_ETIMEOUT
    a = sfbgpu.AnlmModes(0.02, 500.0, 1000.0, nside=8)
    rtp, w = catalogue(1000, a.rmin, a.rmax, seed=4)
    out = sfbgpu.cat2amln(rtp, a, 1e-4, None, None, precision="mixed")
    assert np.all(np.isfinite(out))
