"""Shared test helpers: oracle mode dicts, seeded catalogues, error measures."""

import json
import os

import numpy as np


def modes_dict(amodes, nside=None):
    """The oracle's view of an AnlmModes (same tables the GPU plan receives)."""
    return dict(nmax=amodes.nmax, lmax=amodes.lmax, lmax_n=[int(v) for v in amodes.lmax_n],
                nside=amodes.nside if nside is None else nside, splines=amodes.basisfunctions.spline,
                noff=amodes._noff)


def catalogue(n, rmin, rmax, seed=1, weights=False, rpad=0.0):
    """r ~ r^2 on [rmin - rpad, rmax + rpad], isotropic directions (full sky)."""
    rng = np.random.default_rng(seed)
    a, b = max(rmin - rpad, 0.0), rmax + rpad
    u = rng.random(n)
    r = (a ** 3 + u * (b ** 3 - a ** 3)) ** (1 / 3)
    th = np.arccos(rng.uniform(-1, 1, n))
    ph = rng.uniform(0, 2 * np.pi, n)
    w = rng.uniform(0.5, 1.5, n) if weights else None
    return np.stack([r, th, ph]), w


def rel_err(a, b):
    """max |a - b| / max |b| (global relative error)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def ylm(l, m, theta, phi):
    """Complex Y_lm with Condon-Shortley phase (scipy, either API generation)."""
    from scipy import special
    if hasattr(special, "sph_harm_y"):
        return special.sph_harm_y(l, m, theta, phi)
    return special.sph_harm(m, l, phi, theta)


def round_sig(z, digits=6):
    """Julia's round(x, sigdigits=digits), applied to real and imaginary parts."""
    def r(x):
        x = np.asarray(x, float)
        out = np.zeros_like(x)
        nz = x != 0
        e = np.floor(np.log10(np.abs(x[nz])))
        f = 10.0 ** (digits - 1 - e)
        out[nz] = np.round(x[nz] * f) / f
        return out
    z = np.asarray(z)
    return r(z.real) + 1j * r(z.imag)


def record(name, value, **extra):
    """Append a measured parity figure to $SFB_PARITY_REPORT (JSON lines), if set."""
    path = os.environ.get("SFB_PARITY_REPORT")
    if not path:
        return
    with open(path, "a") as f:
        f.write(json.dumps({"case": name, "rel_err": float(value), **extra}) + "\n")
