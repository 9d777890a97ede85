"""Host-side mode tables: k_nl roots, normalisation, splines, index maps (CPU)."""

import os

import numpy as np
import pytest

import sfbgpu
from sfbgpu.gnl import sphericalbesselj
from sfbgpu.spline import build_ypp, eval_spline

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_kat.npz"))


def test_knl_rmin0_golden():
    a = sfbgpu.AnlmModes.from_nmax_lmax(5, 3, 0.0, 1000.0, cache=False)
    # the reference stops the double-secant iteration at xrtol = 1e-10
    assert np.allclose(a.knl, GOLD["knl_rmin0_rmax1000"], rtol=1e-9, atol=0)


def _boundary_det(l, k, rmin, rmax):
    """Potential-boundary condition as a 2 x 2 determinant of spherical Bessel functions (scipy's
    spherical_jn / spherical_yn, not the Bessel-J/Y form the root search uses): g' - l g / r = 0 at
    rmin and g' + (l + 1) g / r = 0 at rmax for g = c j_l(kr) + d y_l(kr), i.e.
    j_{l-1}(k rmax) y_{l+1}(k rmin) - j_{l+1}(k rmin) y_{l-1}(k rmax) = 0 (j_{-1} = cos x / x,
    y_{-1} = sin x / x)."""
    from scipy.special import spherical_jn, spherical_yn
    xa, xb = k * rmin, k * rmax
    with np.errstate(all="ignore"):
        jm = np.cos(xb) / xb if l == 0 else spherical_jn(l - 1, xb)
        ym = np.sin(xb) / xb if l == 0 else spherical_yn(l - 1, xb)
        return jm * spherical_yn(l + 1, xa) - spherical_jn(l + 1, xa) * ym


@pytest.mark.parametrize("kmax,rmin,rmax,lstep,npts", [(0.05, 500.0, 1000.0, 1, 100001),
                                                      (0.1, 500.0, 2500.0, 19, 40001)])
def test_knl_are_all_boundary_roots_below_kmax(kmax, rmin, rmax, lstep, npts):
    """The modes the scan-and-secant search selects are exactly the roots of the boundary determinant
    in (0, kmax], found independently (sign changes on a fine k grid, then Brent): same count for
    every l checked (no root missed or added) and the same values to 1e-9 (C1 geometry: every l;
    the bench geometry: every 19th l)."""
    from scipy.optimize import brentq
    a = sfbgpu.AnlmModes(kmax, rmin, rmax, cache=False)
    k = np.linspace(1e-4, kmax, npts)
    for l in range(0, a.lmax + 1, lstep):
        d = _boundary_det(l, k, rmin, rmax)
        ok = np.isfinite(d)
        kk, sg = k[ok], np.sign(d[ok])
        idx = np.nonzero(sg[:-1] * sg[1:] < 0)[0]
        roots = np.array([brentq(lambda q: _boundary_det(l, q, rmin, rmax), kk[i], kk[i + 1], xtol=1e-15,
                                 rtol=1e-14) for i in idx])
        got = a.knl[:, l]
        got = got[np.isfinite(got)]
        assert len(got) == len(roots) == int(a.nmax_l[l]), (l, len(got), len(roots))
        if len(roots):
            assert np.max(np.abs(got - roots) / roots) < 1e-9, l


def test_modes_structure_and_index_bijection():
    """reference test/test_modes.jl:13-37."""
    m = sfbgpu.AnlmModes(0.01, 100.0, 10000.0, cache=False)
    assert 2 * m.nside >= m.lmax
    assert max(m.lmax_n) == m.lmax and max(m.nmax_l) == m.nmax
    assert len(m.lmax_n) == m.nmax and len(m.nmax_l) == m.lmax + 1
    assert m.knl.shape == (m.nmax, m.lmax + 1)
    for n in range(1, m.nmax + 1):
        for l in range(int(m.lmax_n[n - 1]) + 1):
            for mm in range(l + 1):
                assert sfbgpu.getnlm(m, sfbgpu.getidx(m, n, l, mm)) == (n, l, mm)
    assert sfbgpu.getidx(m, m.nmax, int(m.lmax_n[-1]), int(m.lmax_n[-1])) == sfbgpu.getnlmsize(m)


@pytest.mark.parametrize("rmin", [0.0, 500.0])
@pytest.mark.parametrize("kmax", [0.01, 0.03])
def test_gnl_orthonormality(rmin, kmax):
    """reference test/test_gnl.jl:11-45 (potential boundary, atol 1e-6)."""
    rmax = 2467.10
    a = sfbgpu.AnlmModes(kmax, rmin, rmax)
    ls = sorted(set([l for l in range(6) if l <= a.lmax] + [a.lmax]))
    for l in ls:
        nmaxl = int(a.nmax_l[l])
        for n1 in range(1, nmaxl + 1):
            for n2 in range(n1, min(n1 + 3, nmaxl) + 1):
                x, wq = np.polynomial.legendre.leggauss(16 * (n1 + n2))
                r = (rmin + rmax) / 2 + (rmax - rmin) / 2 * x
                dr = wq * (rmax - rmin) / 2
                d = np.sum(dr * r ** 2 * a.basisfunctions(n1, l, r) * a.basisfunctions(n2, l, r))
                assert abs(d - (1.0 if n1 == n2 else 0.0)) < 1e-6, (l, n1, n2, d)
    assert np.all(a.knl[np.isfinite(a.knl)] <= kmax)


def test_spline_interpolates_and_matches_exact():
    a = sfbgpu.AnlmModes(0.03, 500.0, 1000.0)
    bf = a.basisfunctions
    for (n, l), (x, y, ypp) in list(bf.spline.items())[::7]:
        assert np.allclose(eval_spline(x, y, ypp, x[:-1]), y[:-1], rtol=0, atol=1e-15 * np.max(np.abs(y)))
        r = np.linspace(a.rmin, a.rmax, 3001)
        # the reference spline's parabolic end slopes leave a few 1e-6 of max|g| near rmin, rmax
        inner = (r > a.rmin + 5 * (x[1] - x[0])) & (r < a.rmax - 5 * (x[1] - x[0]))
        assert np.max(np.abs(bf(n, l, r) - bf.exact(n, l, r))) < 1e-5 * np.max(np.abs(y))
        assert np.max(np.abs(bf(n, l, r[inner]) - bf.exact(n, l, r[inner]))) < 1e-6 * np.max(np.abs(y))
        # boundary extrapolation (reference src/Splines.jl:72-77)
        assert bf(n, l, a.rmin - 5) == y[0] and bf(n, l, a.rmax + 5) == y[-1]


def test_spline_matches_clamped_spline_with_parabola_slopes():
    """The reference spline is the clamped cubic spline whose end slopes are the
    slopes of the parabolas through the first/last three knots
    (src/Splines.jl:179-182,232-263); scipy's clamped spline is an
    independent solver of the same system."""
    from scipy.interpolate import CubicSpline
    rng = np.random.default_rng(0)
    x = np.sort(rng.uniform(0, 3, 40))
    y = np.sin(2 * x) + 0.1 * x
    def pslope(i, j, k):
        return ((y[k] - y[i]) * (x[j] - x[i]) ** 2 - (y[j] - y[i]) * (x[k] - x[i]) ** 2) / (
            (x[k] - x[i]) * (x[j] - x[k]) * (x[j] - x[i]))
    cs = CubicSpline(x, y, bc_type=((1, pslope(0, 1, 2)), (1, pslope(-1, -2, -3))))
    ypp = build_ypp(x, y)
    assert np.allclose(ypp, cs(x, 2), rtol=1e-10, atol=1e-10)
    r = np.linspace(x[0], x[-1], 777)
    assert np.allclose(eval_spline(x, y, ypp, r), cs(r), rtol=1e-12, atol=1e-12)


def test_spherical_bessel_small_x_rule():
    assert sphericalbesselj(0, 1e-20) == 1.0 and sphericalbesselj(3, 1e-20) == 0.0


def test_clnnmodes_order_and_index():
    """reference src/modes.jl:333-401: sorted by l, then n2-n1, then n1; index round trip."""
    a = sfbgpu.AnlmModes(0.03, 500.0, 1000.0, cache=False)
    cm = sfbgpu.ClnnModes(a, dnmax=3)
    lnn = cm.lnn
    keys = [(l, n2 - n1, n1) for l, n1, n2 in lnn.T]
    assert keys == sorted(keys)
    assert np.all(lnn[2] >= lnn[1]) and np.all(lnn[2] - lnn[1] <= 3)
    for i in range(1, sfbgpu.getlnnsize(cm) + 1):
        l, n1, n2 = sfbgpu.getlnn(cm, i)
        assert sfbgpu.getidx_lnn(cm, l, n1, n2) == i == sfbgpu.getidx_lnn(cm, l, n2, n1)
