"""HEALPix helpers the host API needs (pixel centres for masks and fixtures).

RING scheme, 0-based pixel indices (Healpix.jl's ``pix2angRing`` takes the
same index plus one).  Pixel classification of galaxies happens on the GPU
(``sfb_ang2pix_ring`` / the binning kernel), not here.
"""

import numpy as np

__all__ = ["nside2npix", "npix2nside", "pix2ang_ring"]


def nside2npix(nside):
    return 12 * int(nside) ** 2


def npix2nside(npix):
    ns = int(round(np.sqrt(npix / 12)))
    if 12 * ns * ns != npix:
        raise ValueError("npix is not 12*nside^2")
    return ns


def pix2ang_ring(nside, pix):
    """(theta, phi) of the centres of 0-based RING pixels (Gorski et al. 2005)."""
    ns = int(nside)
    npix = 12 * ns * ns
    ncap = 2 * ns * (ns - 1)
    pix = np.asarray(pix, np.int64)
    theta = np.empty(pix.shape)
    phi = np.empty(pix.shape)
    north = pix < ncap
    south = pix >= npix - ncap
    eq = ~(north | south)
    if np.any(north):
        p = pix[north]
        i = (1 + np.floor(np.sqrt(1 + 2 * p)).astype(np.int64)) >> 1
        # guard the integer square root against rounding
        i = np.where(2 * i * (i - 1) > p, i - 1, i)
        i = np.where(2 * (i + 1) * i <= p, i + 1, i)
        j = p - 2 * i * (i - 1)
        omz = i * i * (4.0 / npix)
        theta[north] = np.arctan2(np.sqrt(omz * (2 - omz)), 1 - omz)
        phi[north] = (j + 0.5) * (np.pi / 2) / i
    if np.any(eq):
        p = pix[eq] - ncap
        i = p // (4 * ns) + ns
        j = p % (4 * ns)
        fodd = np.where(((i + ns) & 1) == 1, 1.0, 0.5)
        z = (2 * ns - i) * (8.0 * ns / npix)
        theta[eq] = np.arctan2(np.sqrt((1 - z) * (1 + z)), z)
        phi[eq] = (j + 1 - fodd) * (np.pi / 2) / ns
    if np.any(south):
        p = npix - 1 - pix[south]
        i = (1 + np.floor(np.sqrt(1 + 2 * p)).astype(np.int64)) >> 1
        i = np.where(2 * i * (i - 1) > p, i - 1, i)
        i = np.where(2 * (i + 1) * i <= p, i + 1, i)
        jr = p - 2 * i * (i - 1)              # counted from the end of the ring
        j = 4 * i - 1 - jr
        omz = i * i * (4.0 / npix)
        theta[south] = np.arctan2(np.sqrt(omz * (2 - omz)), -(1 - omz))
        phi[south] = (j + 0.5) * (np.pi / 2) / i
    return theta, phi
