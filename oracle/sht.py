"""Spherical-harmonic transforms on HEALPix RING maps (TEST INFRASTRUCTURE).

Restates the transform the reference obtains from Healpix.jl/libsharp
(``mymap2alm!`` -> ``map2alm!(map, alm; niter=3)``, reference
``src/healpix_helpers.jl:50-56``):

* analysis  a_lm = (4pi/npix) sum_p f_p conj(Y_lm(p))      (uniform weights)
* synthesis f_p  = sum_lm a_lm Y_lm(p) for a real map (m>=0 stored)
* refinement alm <- alm + A(f - S(alm)), ``niter`` times (Jacobi iteration).

Y_lm = lambda_lm(theta) e^{i m phi} with the Condon-Shortley phase, the
convention of the reference's ``sphericalharmonicsy`` (``src/math.jl:10-21``,
pinned by ``test/test_toplevel.jl:2-17``).

Analysis uses the exact per-ring DFT (bins m mod nph, so aliasing on short
polar rings is exact); synthesis folds every m onto the ring's nph bins and
applies an inverse DFT, then the refinement runs in pixel space.  Arrays:
alm[..., l, m] complex with m <= l, maps[..., npix] float.
"""

import numpy as np

from .healpix import ring_info

_SCALE = 600  # exponent step of the scaled Legendre recursion


def legendre_table(lmax, z, sth):
    """lambda_lm(theta) for all rings: array [m, l, ring] (zero for l < m).

    Three-term recursion in l with a power-of-two scale carried per ring so
    that lambda_mm ~ sin^m(theta) never underflows before the recursion in l
    brings it back; values below the double range are flushed to zero.
    """
    z = np.atleast_1d(np.asarray(z, float))
    sth = np.atleast_1d(np.asarray(sth, float))
    R = len(z)
    out = np.zeros((lmax + 1, lmax + 1, R))
    # lambda_mm with separate mantissa and binary exponent
    mant = np.full(R, 1.0 / np.sqrt(4 * np.pi))
    expo = np.zeros(R, np.int64)
    for m in range(lmax + 1):
        if m > 0:
            mant = mant * (-np.sqrt((2 * m + 1) / (2.0 * m))) * sth
            small = (np.abs(mant) < 2.0 ** -_SCALE) & (mant != 0)
            mant = np.where(small, np.ldexp(mant, _SCALE), mant)
            expo = np.where(small, expo - _SCALE, expo)
        v_prev2 = np.zeros(R)
        v_prev = mant.copy()
        e = expo.copy()
        out[m, m] = np.ldexp(v_prev, e)
        for l in range(m + 1, lmax + 1):
            a = np.sqrt((4.0 * l * l - 1) / (l * l - m * m))
            b = np.sqrt(((l - 1) ** 2 - m * m) / (4.0 * (l - 1) ** 2 - 1)) if l - 1 > m else 0.0
            v = a * (z * v_prev - b * v_prev2)
            big = np.abs(v) > 2.0 ** _SCALE
            if np.any(big):
                v = np.where(big, np.ldexp(v, -_SCALE), v)
                v_prev = np.where(big, np.ldexp(v_prev, -_SCALE), v_prev)
                e = np.where(big, e + _SCALE, e)
            out[m, l] = np.ldexp(v, e)
            v_prev2, v_prev = v_prev, v
    return out


class SHT:
    """Batched analysis/synthesis for one (nside, lmax)."""

    def __init__(self, nside, lmax):
        self.nside = nside
        self.lmax = lmax
        self.info = ring_info(nside)
        self.npix = self.info["npix"]
        self.w = 4 * np.pi / self.npix
        self.lam = legendre_table(lmax, self.info["z"], self.info["sth"])   # [m, l, ring]
        # group rings by length for batched FFTs
        self.groups = {}
        for r, n in enumerate(self.info["nph"]):
            self.groups.setdefault(int(n), []).append(r)

    def ring_fourier(self, maps):
        """F[..., ring, m] = w sum_j f_j e^{-i m phi_j}, m = 0..lmax."""
        maps = np.asarray(maps, float)
        lead = maps.shape[:-1]
        L = self.lmax
        m = np.arange(L + 1)
        F = np.zeros(lead + (self.info["nring"], L + 1), complex)
        for n, rings in self.groups.items():
            rings = np.array(rings)
            starts = self.info["start"][rings]
            idx = starts[:, None] + np.arange(n)[None, :]
            seg = maps[..., idx]                          # [..., nr_g, n]
            c = np.fft.fft(seg, axis=-1)
            bins = c[..., m % n]                          # [..., nr_g, L+1]
            phase = np.exp(-1j * np.outer(self.info["phi0"][rings], m))
            F[..., rings, :] = self.w * bins * phase
        return F

    def analysis(self, maps):
        """Plain quadrature (niter = 0)."""
        F = self.ring_fourier(maps)
        # alm[..., l, m] = sum_r lam[m, l, r] F[..., r, m]
        return np.einsum("mlr,...rm->...lm", self.lam, F)

    def synthesis(self, alm):
        alm = np.asarray(alm, complex)
        lead = alm.shape[:-2]
        L = self.lmax
        G = np.einsum("mlr,...lm->...rm", self.lam, alm)       # [..., ring, m]
        G[..., 0] = G[..., 0].real
        maps = np.zeros(lead + (self.npix,))
        m = np.arange(L + 1)
        for n, rings in self.groups.items():
            rings = np.array(rings)
            phi0 = self.info["phi0"][rings]
            Gr = G[..., rings, :]                                 # [..., nr_g, L+1]
            pos = Gr * np.exp(1j * np.outer(phi0, m))
            neg = np.conj(Gr[..., 1:]) * np.exp(-1j * np.outer(phi0, m[1:]))
            c = np.zeros(lead + (len(rings), n), complex)
            # fold every frequency onto the ring's n DFT bins
            c2 = c.reshape((-1, len(rings), n))
            np.add.at(c2, (slice(None), slice(None), m % n), pos.reshape((-1, len(rings), L + 1)))
            np.add.at(c2, (slice(None), slice(None), (-m[1:]) % n), neg.reshape((-1, len(rings), L)))
            c = c2.reshape(lead + (len(rings), n))
            vals = (np.fft.ifft(c, axis=-1) * n).real
            starts = self.info["start"][rings]
            idx = starts[:, None] + np.arange(n)[None, :]
            maps[..., idx] = vals
        return maps

    def map2alm(self, maps, niter=3):
        """Analysis with Jacobi refinement (Healpix.jl map2alm!, default niter=3)."""
        maps = np.asarray(maps, float)
        alm = self.analysis(maps)
        for _ in range(niter):
            alm = alm + self.analysis(maps - self.synthesis(alm))
        return alm

    def alm2map(self, alm):
        return self.synthesis(alm)


def ylm(l, m, theta, phi):
    """Complex Y_lm with Condon-Shortley phase for m >= 0 (test helper)."""
    th = np.asarray(theta, float)
    lam = legendre_table(l, np.cos(th).ravel(), np.sin(th).ravel())[m, l].reshape(th.shape)
    return lam * np.exp(1j * m * np.asarray(phi))
