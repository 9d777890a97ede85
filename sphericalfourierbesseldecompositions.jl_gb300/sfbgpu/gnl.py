"""g_nl(r) = c_nl j_l(k_nl r) + d_nl y_l(k_nl r) for the potential boundary.

Host-side setup of the radial basis, as the Julia side of the boundary
computes it before calling the GPU plan:

* k_nl: roots of the potential-boundary condition, found by the reference's
  scan-then-double-secant search (reference
  ``src/SphericalBesselGNLs.jl:72-166,197-214,219-228,294-336``);
* c_nl, d_nl: the analytic normalisation (``:404-421``, sign rule ``:418``);
* spline cache: knots ``rmin:Δr:rmax+Δr/2`` with
  ``nr = 3 + 12*ceil(2k(rmax-rmin))`` (``:558-579``), cubic spline per (n,l).

Bessel functions come from scipy (AMOS for real order, the same library
family the reference's SpecialFunctions uses).  The reference's 1024-bit Arb
fallback on AMOS overflow is replaced by the overflow-free ratio form of the
root function; at the workloads this package targets no overflow occurs.
"""

import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
from scipy import special

from .spline import build_ypp_batched, eval_spline

__all__ = ["POTENTIAL", "calc_knl_kmax", "calc_knl_nmax", "calc_cnl_dnl",
           "sphericalbesselj", "sphericalbessely", "SphericalBesselGNL"]

POTENTIAL = "potential"


def sphericalbesselj(l, x):
    """j_l(x) = sqrt(pi/2x) J_{l+1/2}(x) with the small-x rule of SpecialFunctions."""
    x = np.asarray(x, float)
    with np.errstate(all="ignore"):
        bj = special.jv(l + 0.5, x)
        v = np.sqrt(np.pi / (2 * x)) * bj
    small = np.abs(x) <= math.sqrt(np.finfo(float).eps)
    return np.where(small, 1.0 if l == 0 else 0.0, v)


def sphericalbessely(l, x):
    """y_l(x) = sqrt(pi/2x) Y_{l+1/2}(x); -inf at x == 0 (bes_yl, :389-393)."""
    x = np.asarray(x, float)
    with np.errstate(all="ignore"):
        v = np.sqrt(np.pi / (2 * x)) * special.yv(l + 0.5, x)
    return np.where(x == 0, -np.inf, v)


def _sign(v):
    return 0.0 if v == 0 else (1.0 if v > 0 else -1.0)


def knl_zero_function_potential(k, l, rmin, rmax):
    """Potential-boundary root function (reference :219-228)."""
    scale = k ** 3 / (1 + abs(k) ** 3)
    jlmax = special.jv(l - 0.5, k * rmax)
    if k * rmin == 0:
        return jlmax
    with np.errstate(all="ignore"):
        ylmin_raw = special.yv(l + 1.5, k * rmin)
    ylmax = special.yv(l - 0.5, k * rmax) * scale
    jlmin = special.jv(l + 1.5, k * rmin)
    if np.isfinite(ylmin_raw):
        ylmin = ylmin_raw * scale
        return jlmax * ylmin - jlmin * ylmax
    # AMOS overflow of y_{l+3/2}(k rmin): divide the function by ylmin*scale,
    # which is negative there, so the ratio form keeps the sign pattern.  The
    # remaining term jlmin/ylmin * ylmax underflows to zero in this regime.
    return -jlmax


def doublesecant_method(fn, a, b, maxevals=1000, xrtol=float(np.finfo(float).eps)):
    """Bracketed double-secant root refinement (reference :72-128)."""
    fa = fn(a)
    fb = fn(b)
    assert _sign(fa) * _sign(fb) <= 0
    neval = 0
    while a != b and neval < maxevals:
        m = (fb - fa) / (b - a)
        c = b - fb / m
        if abs(c - b) <= xrtol * c or abs(c - a) <= xrtol * c:
            return c
        fc = fn(c)
        d = b - (fb + fc) / m
        if _sign(fa) * _sign(fc) <= 0:
            b, fb = c, fc
        elif _sign(fb) * _sign(fc) <= 0:
            a, fa = c, fc
        else:
            a, fa, b, fb = c, fc, c, fc
        if a <= d <= b:
            fd = fn(d)
            if _sign(fa) * _sign(fd) <= 0:
                b, fb = d, fd
            elif _sign(fb) * _sign(fd) <= 0:
                a, fa = d, fd
            else:
                a, fa, b, fb = d, fd, d, fd
        neval += 1
    return float("nan")


def calc_next_fn_zero(func, x, delta, maxevals=1000, xrtol=1e-10):
    """Step by delta until the sign changes, then refine (reference :131-166)."""
    f = func(x)
    xnew = x + delta
    fnew = func(xnew)
    while _sign(fnew) == _sign(f):
        x, f = xnew, fnew
        xnew += delta
        fnew = func(xnew)
    xnew = doublesecant_method(func, x, xnew, maxevals=maxevals, xrtol=xrtol)
    if not math.isfinite(xnew):
        raise ArithmeticError("root search did not converge")
    return xnew


def calc_zeros(func, xmin, xmax, delta):
    """All zeros in [xmin, xmax] (reference :197-214)."""
    out = []
    while xmin <= xmax:
        x = calc_next_fn_zero(func, xmin, delta)
        if xmin <= x <= xmax:
            out.append(x)
        xmin = x + delta
    return out


def calc_first_n_zeros(func, nmax, delta, xmin):
    """First nmax zeros at or above xmin (reference :175-188)."""
    out = np.full(nmax, np.nan)
    for n in range(nmax):
        out[n] = calc_next_fn_zero(func, xmin, delta)
        xmin = out[n] + delta
    return out


def _map_l(fn, lvals):
    nthreads = min(len(lvals), os.cpu_count() or 1) or 1
    if nthreads <= 1:
        return [fn(l) for l in lvals]
    with ThreadPoolExecutor(nthreads) as ex:
        return list(ex.map(fn, lvals))


def calc_knl_kmax(kmax, rmin, rmax, nmax=None, lmax=None):
    """k_nl <= kmax for every l (reference calc_knl_zeros(kmax, ...), :309-336).

    Returns an (nmax_calc, lmax_calc+1) array, NaN where no root exists.
    """
    nmax_calc = math.ceil(kmax * rmax / math.pi) + 1
    lmax_calc = math.ceil(kmax * rmax)
    big = 2 ** 62
    nmax_req = big if nmax is None else nmax
    lmax_req = big if lmax is None else lmax
    kmax_lim = lmax_req > lmax_calc and nmax_req > nmax_calc
    nmax_u = min(nmax_req, nmax_calc)
    lmax_u = min(lmax_req, lmax_calc)
    delta = math.pi / rmax / 4

    def one_l(l):
        kmin = (l + 1.5) / rmax
        return calc_zeros(lambda k: knl_zero_function_potential(k, l, rmin, rmax), kmin, kmax, delta)

    roots = _map_l(one_l, list(range(lmax_u + 1)))
    knl = np.full((nmax_u, lmax_u + 1), np.nan)
    for l, kn in enumerate(roots):
        if len(kn) > nmax_u:
            raise ValueError("nmax too small")
        if kmax_lim and l == lmax_u:
            assert len(kn) == 0
        knl[:len(kn), l] = kn
    fin = knl[np.isfinite(knl)]
    assert np.all(fin > 0)
    return knl


def calc_knl_nmax(nmax, lmax, rmin, rmax):
    """First nmax roots for each l <= lmax (reference calc_knl_zeros(nmax, lmax, ...), :294-306)."""
    delta = math.pi / rmax / 4

    def one_l(l):
        xmin = (l + 1.5) / rmax
        return calc_first_n_zeros(lambda k: knl_zero_function_potential(k, l, rmin, rmax), nmax, delta, xmin)

    cols = _map_l(one_l, list(range(lmax + 1)))
    knl = np.stack(cols, axis=1)
    assert np.all(knl > 0)
    return knl


def _sphbes_gnl(q, l, c, d):
    """c j_l(q) + d y_l(q) (reference calc_sphbes_gnl, :396-401)."""
    jl = sphericalbesselj(l, q)
    if d == 0:
        return c * jl
    yl = sphericalbessely(l, q)
    return c * jl + d * yl


def calc_cnl_dnl(knl, rmin, rmax):
    """Potential-boundary normalisation (reference :404-421,530-555)."""
    nmax, L1 = knl.shape
    cnl = np.full(knl.shape, np.nan)
    dnl = np.full(knl.shape, np.nan)
    for n1 in range(nmax):
        n = n1 + 1
        for l in range(L1):
            k = knl[n1, l]
            if not np.isfinite(k):
                continue
            with np.errstate(all="ignore"):
                ymin = special.yv(l + 1.5, k * rmin) if k * rmin != 0 else -np.inf
                dc = -special.jv(l + 1.5, k * rmin) / ymin
            g_rmin = float(_sphbes_gnl(k * rmin, l, 1.0, dc))
            g_rmax = float(_sphbes_gnl(k * rmax, l, 1.0, dc))
            num_one = (rmax ** 3 * g_rmax ** 2 - rmin ** 3 * g_rmin ** 2) / 2
            assert num_one >= 0
            e = n + (1 - (1 if l == 0 else 0)) * (1 - (1 if n == 1 else 0))
            c = (-1.0) ** e / math.sqrt(num_one)
            cnl[n1, l] = c
            dnl[n1, l] = dc * c
    return cnl, dnl


def spline_knots(k, rmin, rmax):
    """Knot grid of one g_nl spline (reference gen_gnl_cache, :571-573)."""
    nr = 3 + 12 * math.ceil(2 * k * (rmax - rmin))
    dr = (rmax - rmin) / nr
    return rmin + dr * np.arange(nr + 1)


class SphericalBesselGNL:
    """Radial basis with cached splines (reference ``SphericalBesselGNL``, :584-656).

    ``self(n, l, r)`` evaluates the cached spline, as ``GNLs.evaluate`` does
    (reference ``src/GNLs.jl:105-107``); n is 1-based, l 0-based.
    """

    def __init__(self, knl, cnl, dnl, rmin, rmax, cache=True):
        self.knl = knl
        self.cnl = cnl
        self.dnl = dnl
        self.rmin = float(rmin)
        self.rmax = float(rmax)
        self.nmax, L1 = knl.shape
        self.lmax = L1 - 1
        self.spline = {}
        if cache:
            self._build_cache()

    def exact(self, n, l, r):
        """Uncached evaluation c j_l(kr) + d y_l(kr) (reference evaluate, :651-656)."""
        k = self.knl[n - 1, l]
        return _sphbes_gnl(k * np.asarray(r, float), l, self.cnl[n - 1, l], self.dnl[n - 1, l])

    def _build_cache(self):
        pairs = [(n1 + 1, l) for n1 in range(self.nmax) for l in range(self.lmax + 1)
                 if np.isfinite(self.knl[n1, l])]
        xs = [spline_knots(self.knl[n - 1, l], self.rmin, self.rmax) for n, l in pairs]

        def knot_values(i):
            n, l = pairs[i]
            return self.exact(n, l, xs[i])

        ys = _map_l(knot_values, list(range(len(pairs))))
        ypps = build_ypp_batched(xs, ys)
        for (n, l), x, y, ypp in zip(pairs, xs, ys, ypps):
            self.spline[(n, l)] = (x, np.asarray(y, float), ypp)

    def __call__(self, n, l, r):
        if (n, l) in self.spline:
            x, y, ypp = self.spline[(n, l)]
            return eval_spline(x, y, ypp, r)
        return self.exact(n, l, r)
