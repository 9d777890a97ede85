"""Voxelisation and window helpers (host side).

``ConfigurationSpaceModes`` (reference ``src/windows.jl:80-114``),
``window_r``/``get_rbounds`` (``:125-134``), ``integrate_window``
(``:219-228``), ``SeparableArray`` (``src/SeparableArrays.jl:46-110``) and the
window generators the reference tests use (``gen_mask`` and a subset of
``make_window``, ``src/SphericalFourierBesselDecompositions.jl:221-234,300-494``).
"""

import numpy as np

from .healpix import nside2npix, pix2ang_ring

__all__ = ["ConfigurationSpaceModes", "window_r", "get_rbounds", "integrate_window", "SeparableArray",
           "gen_mask", "make_window"]


class ConfigurationSpaceModes:
    """Radial shells x HEALPix pixels (reference src/windows.jl:98-103)."""

    def __init__(self, rmin, rmax, nr, nside):
        self.rmin = float(rmin)
        self.rmax = float(rmax)
        self.nr = int(nr)
        self.nside = int(nside)
        self.dr = (self.rmax - self.rmin) / self.nr
        self.r = np.linspace(self.rmin + self.dr / 2, self.rmax - self.dr / 2, self.nr)   # midpoints
        self.npix = nside2npix(self.nside)

    @classmethod
    def from_amodes(cls, amodes, nr):
        """ConfigurationSpaceModes(amodes, nr) (reference src/windows.jl:112-114)."""
        return cls(amodes.rmin, amodes.rmax, nr, amodes.nside)


def window_r(wmodes):
    return wmodes.r, wmodes.dr


def get_rbounds(wmodes):
    return np.linspace(wmodes.rmin, wmodes.rmax, wmodes.nr + 1)


class SeparableArray:
    """Lazy outer product arr1 (x) arr2 (reference src/SeparableArrays.jl:46-110).

    ``SeparableArray(phi, mask, name1="phi", name2="mask")`` is a separable
    window W[r, p] = phi[r] mask[p]; ``win_rhat_ln`` of it returns
    ``SeparableArray(mask, w_ln, name1="mask", name2="w_ln")``.
    """

    def __init__(self, arr1, arr2, name1="arr1", name2="arr2"):
        self.arr1 = np.asarray(arr1, float)
        self.arr2 = np.asarray(arr2, float)
        self.name1 = name1
        self.name2 = name2

    def __getattr__(self, name):
        d = self.__dict__
        if name == d.get("name1"):
            return d["arr1"]
        if name == d.get("name2"):
            return d["arr2"]
        raise AttributeError(name)

    @property
    def shape(self):
        return self.arr1.shape + self.arr2.shape

    def dense(self):
        return np.multiply.outer(self.arr1, self.arr2)

    def __getitem__(self, idx):
        return self.dense()[idx]


def integrate_window(win, wmodes):
    """V_eff = dr dOmega sum_r r^2 sum_p W[r, p] (reference src/windows.jl:219-228)."""
    W = win.dense() if isinstance(win, SeparableArray) else np.asarray(win, float)
    npix = W.shape[1]
    return wmodes.dr * (4 * np.pi / npix) * np.sum(W.sum(axis=1) * wmodes.r ** 2)


def gen_mask(nside, fsky):
    """Polar-cap mask with theta <= acos(1 - 2 fsky) (reference src/SphericalFourierBesselDecompositions.jl:221-234)."""
    npix = nside2npix(nside)
    theta, _ = pix2ang_ring(nside, np.arange(npix))
    return (theta <= np.arccos(1 - 2 * fsky)).astype(float)


def make_window(wmodes, *features):
    """Subset of the reference's window DSL: :fullsky, :ang_75/_half/_quarter/_eighth/_sixteenth,
    :radial, :radial_expmrr0, :separable, :dense (reference :300-494)."""
    win = np.ones((wmodes.nr, wmodes.npix))
    fsky = {"ang_75": 0.75, "ang_half": 0.5, "ang_quarter": 0.25, "ang_eighth": 1 / 8, "ang_sixteenth": 1 / 16}

    def normalise(w):
        if isinstance(w, SeparableArray):
            w.arr2 /= np.max(w.arr2)
            w.arr1 /= np.max(np.multiply.outer(w.arr1, w.arr2))
            return w
        return w / np.max(w)

    for feat in features:
        feat = feat.lstrip(":")
        if feat == "fullsky":
            pass
        elif feat in fsky:
            mask = gen_mask(wmodes.nside, fsky[feat])
            if isinstance(win, SeparableArray):
                win.arr2 *= mask
            else:
                win = win * mask[None, :]
        elif feat in ("radial", "radial_expmrr0"):
            if feat == "radial":
                phi = np.exp(-(wmodes.r / (wmodes.rmax * 0.55)) ** 2)
            else:
                phi = np.exp(-wmodes.r / ((wmodes.rmin + wmodes.rmax) / 2 / 3))
            if isinstance(win, SeparableArray):
                win.arr1 *= phi
            else:
                win = win * phi[:, None]
        elif feat == "separable":
            win = SeparableArray(win.mean(axis=1), win.mean(axis=0), name1="phi", name2="mask")
        elif feat == "dense":
            win = win.dense() if isinstance(win, SeparableArray) else np.array(win)
        else:
            raise ValueError(f"Unsupported feature {feat}.")
        win = normalise(win)
    return win
