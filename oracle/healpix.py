"""HEALPix RING-scheme geometry for the oracle (TEST INFRASTRUCTURE).

Written from the published HEALPix construction (Gorski et al. 2005): rings
i = 1..4*nside-1 from the north pole; polar rings carry 4i pixels, the
equatorial belt 4*nside.  Pixel indices here are 0-based; Healpix.jl's
``ang2pixRing`` returns the same index plus one (reference call sites
``src/cat2anlm.jl:230,263``).
"""

import numpy as np

INV_HALFPI = 2.0 / np.pi


def nside2npix(nside):
    return 12 * nside * nside


def ring_info(nside):
    """Per ring (0-based ring r = i-1): nph, first pixel, z = cos(theta),
    1 - |z| where exact, sin(theta), and phi of the ring's first pixel."""
    ns = nside
    npix = nside2npix(ns)
    nring = 4 * ns - 1
    i = np.arange(1, nring + 1)
    nph = np.empty(nring, np.int64)
    start = np.empty(nring, np.int64)
    z = np.empty(nring)
    sth = np.empty(nring)
    phi0 = np.empty(nring)
    fact2 = 4.0 / npix
    fact1 = (2 * ns) * fact2
    for k, ii in enumerate(i):
        if ii < ns:                                  # north cap
            nph[k] = 4 * ii
            start[k] = 2 * ii * (ii - 1)
            omz = ii * ii * fact2                     # 1 - z, exact for the cap
            z[k] = 1.0 - omz
            sth[k] = np.sqrt(omz * (2.0 - omz))
            phi0[k] = np.pi / (4 * ii)
        elif ii <= 3 * ns:                           # equatorial belt
            nph[k] = 4 * ns
            start[k] = 2 * ns * (ns - 1) + (ii - ns) * 4 * ns
            z[k] = (2 * ns - ii) * fact1
            sth[k] = np.sqrt((1.0 - z[k]) * (1.0 + z[k]))
            fodd = 1.0 if ((ii + ns) & 1) else 0.5
            phi0[k] = (1.0 - fodd) * np.pi / (2 * ns)
        else:                                        # south cap
            jj = 4 * ns - ii
            nph[k] = 4 * jj
            start[k] = npix - 2 * jj * (jj + 1)
            omz = jj * jj * fact2
            z[k] = -(1.0 - omz)
            sth[k] = np.sqrt(omz * (2.0 - omz))
            phi0[k] = np.pi / (4 * jj)
    return dict(nph=nph, start=start, z=z, sth=sth, phi0=phi0, nring=nring, npix=npix)


def pix2ang_ring(nside, pix):
    """Pixel-centre (theta, phi) of 0-based RING pixels."""
    info = ring_info(nside)
    pix = np.asarray(pix, np.int64)
    r = np.searchsorted(info["start"], pix, side="right") - 1
    j = pix - info["start"][r]
    theta = np.arctan2(info["sth"][r], info["z"][r])
    phi = info["phi0"][r] + 2 * np.pi * j / info["nph"][r]
    return theta, phi


def _fmodulo(v, m):
    out = np.fmod(v, m)
    out = np.where(out < 0, out + m, out)
    return np.where(out >= m, 0.0, out)


def ang2pix_ring(nside, theta, phi):
    """0-based RING pixel containing (theta, phi) (HEALPix paper algorithm)."""
    theta = np.asarray(theta, float)
    phi = np.asarray(phi, float)
    ns = nside
    npix = nside2npix(ns)
    ncap = 2 * ns * (ns - 1)
    z = np.cos(theta)
    za = np.abs(z)
    tt = _fmodulo(phi * INV_HALFPI, 4.0)          # in [0, 4)
    out = np.empty(z.shape, np.int64)

    eq = za <= 2.0 / 3.0
    if np.any(eq):
        ze = z[eq]
        te = tt[eq]
        temp1 = ns * (0.5 + te)
        temp2 = ns * ze * 0.75
        jp = np.floor(temp1 - temp2).astype(np.int64)      # ascending edge line
        jm = np.floor(temp1 + temp2).astype(np.int64)      # descending edge line
        ir = ns + 1 + jp - jm                              # ring from z = 2/3
        kshift = 1 - (ir & 1)
        t1 = jp + jm - ns + kshift + 1 + 8 * ns
        ip = (t1 >> 1) % (4 * ns)
        # same guard as the GPU kernel against a rounding step outside the belt
        out[eq] = np.clip(ncap + (ir - 1) * 4 * ns + ip, 0, npix - 1)
    pc = ~eq
    if np.any(pc):
        zp = z[pc]
        tp_all = tt[pc]
        zap = za[pc]
        tp = tp_all - np.floor(tp_all)
        tmp = ns * np.sqrt(3.0 * (1.0 - zap))
        jp = np.floor(tp * tmp).astype(np.int64)
        jm = np.floor((1.0 - tp) * tmp).astype(np.int64)
        ir = jp + jm + 1                                   # ring from the nearest pole
        ip = np.floor(tp_all * ir).astype(np.int64)
        ip = ip % (4 * ir)
        out[pc] = np.where(zp > 0, 2 * ir * (ir - 1) + ip, npix - 2 * ir * (ir + 1) + ip)
    return out
