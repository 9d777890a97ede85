"""Generate tests/golden/golden_kat.npz: closed-form known answers.

The reference ships no golden vectors and cannot run here (no Julia), so the
fixtures are known answers that follow from the mathematics, computed with
code independent of both the oracle and the package:

* k_nl for the potential boundary with rmin = 0: the condition reduces to
  j_{l-1}(k rmax) = 0 (reference src/SphericalBesselGNLs.jl:219-223), i.e.
  l = 0: cos(x) = 0, l = 1: sin(x) = 0, l = 2: tan(x) = x, l = 3: zeros of
  j_2 (found with scipy's brentq on scipy.special.spherical_jn);
* HEALPix pixel centres for nside = 1 and 2 from the ring construction
  written out by hand (Gorski et al. 2005, Table/Fig. 4 geometry);
* Y_lm closed forms for l <= 2 with the Condon-Shortley phase
  (reference test/test_toplevel.jl:2-17 for l <= 1).

Run:  python tests/golden/make_golden.py
"""

import os

import numpy as np
from scipy import optimize, special

HERE = os.path.dirname(os.path.abspath(__file__))


def knl_rmin0(rmax=1000.0, nmax=5):
    out = np.zeros((nmax, 4))
    out[:, 0] = (np.arange(1, nmax + 1) - 0.5) * np.pi / rmax
    out[:, 1] = np.arange(1, nmax + 1) * np.pi / rmax
    for l, order in ((2, 1), (3, 2)):
        f = lambda x: special.spherical_jn(order, x)
        roots = []
        x = 1e-3
        while len(roots) < nmax:
            if f(x) * f(x + 0.01) < 0:
                roots.append(optimize.brentq(f, x, x + 0.01, xtol=1e-15, rtol=1e-15))
            x += 0.01
        out[:, l] = np.array(roots) / rmax
    return out


def healpix_centres():
    # nside = 1: three rings of 4 pixels at z = 2/3, 0, -2/3
    th1 = np.repeat([np.arccos(2 / 3), np.pi / 2, np.arccos(-2 / 3)], 4)
    ph1 = np.concatenate([np.pi / 4 + np.pi / 2 * np.arange(4), np.pi / 2 * np.arange(4),
                          np.pi / 4 + np.pi / 2 * np.arange(4)])
    # nside = 2: rings z = 1 - 1/12 (4 px), 2/3, 1/3, 0, -1/3, -2/3 (8 px each), -(1 - 1/12) (4 px)
    zs = [11 / 12, 2 / 3, 1 / 3, 0.0, -1 / 3, -2 / 3, -11 / 12]
    counts = [4, 8, 8, 8, 8, 8, 4]
    # first-pixel phi: cap rings pi/4; belt rings alternate pi/8, 0, pi/8, 0, pi/8
    phi0 = [np.pi / 4, np.pi / 8, 0.0, np.pi / 8, 0.0, np.pi / 8, np.pi / 4]
    th2, ph2 = [], []
    for z, c, p0 in zip(zs, counts, phi0):
        th2 += [np.arccos(z)] * c
        ph2 += list(p0 + 2 * np.pi / c * np.arange(c))
    return th1, ph1, np.array(th2), np.array(ph2)


def ylm_closed(theta, phi):
    c, s = np.cos(theta), np.sin(theta)
    e = np.exp(1j * phi)
    return {
        (0, 0): np.full_like(e, 1 / np.sqrt(4 * np.pi)),
        (1, 0): np.sqrt(3 / (4 * np.pi)) * c + 0j,
        (1, 1): -np.sqrt(3 / (8 * np.pi)) * s * e,
        (2, 0): np.sqrt(5 / (16 * np.pi)) * (3 * c ** 2 - 1) + 0j,
        (2, 1): -np.sqrt(15 / (8 * np.pi)) * s * c * e,
        (2, 2): np.sqrt(15 / (32 * np.pi)) * s ** 2 * e ** 2,
    }


def main():
    th1, ph1, th2, ph2 = healpix_centres()
    theta = np.array([0.1, 0.7, 1.3, 2.2, 3.0])
    phi = np.array([0.0, 1.0, 2.5, 4.0, 6.0])
    Y = ylm_closed(theta, phi)
    np.savez(os.path.join(HERE, "golden_kat.npz"),
             knl_rmin0_rmax1000=knl_rmin0(),
             hp1_theta=th1, hp1_phi=ph1, hp2_theta=th2, hp2_phi=ph2,
             ylm_theta=theta, ylm_phi=phi,
             ylm_lm=np.array(list(Y.keys())), ylm_val=np.array(list(Y.values())))


if __name__ == "__main__":
    main()
