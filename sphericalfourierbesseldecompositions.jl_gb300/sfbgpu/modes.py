"""Mode selection and the a_nlm ordering (host side).

``AnlmModes`` follows the reference struct (``src/modes.jl:92-175``): modes
with k_nl <= kmax, ``nmax_l``/``lmax_n`` and the coefficient order "m
fastest, then l, then n" with m >= 0 (``src/modes.jl:80-82``).  Indices n are
1-based, l and m 0-based, and ``getidx`` returns a 1-based index exactly as
the reference does; ``getidx0`` is the 0-based position in a Python array.
"""

import math

import numpy as np

from .gnl import SphericalBesselGNL, calc_cnl_dnl, calc_knl_kmax, calc_knl_nmax

__all__ = ["AnlmModes", "ClnnModes", "estimate_nside", "getlmsize", "getnlmsize", "getidx",
           "getidx0", "getnlm", "isvalidnlm", "getlnnsize", "getlnn", "getidx_lnn"]


def estimate_nside(lmax):
    """2^max(2, ceil(log2((2 lmax + 1)/2))) (reference src/modes.jl:68)."""
    return 2 ** max(2, math.ceil(math.log2((2 * lmax + 1) / 2)))


def getlmsize(lmax):
    """Number of (l, m>=0) pairs up to lmax (reference src/modes.jl:178-180)."""
    return lmax * (lmax + 1) // 2 + lmax + 1


class AnlmModes:
    """Modes and basis functions of an SFB decomposition.

    ``AnlmModes(kmax, rmin, rmax, nside=None)`` or
    ``AnlmModes.from_nmax_lmax(nmax, lmax, rmin, rmax, nside=None)``
    (reference ``src/modes.jl:122-175``).
    """

    def __init__(self, kmax, rmin, rmax, nside=None, nmax=None, lmax=None, cache=True):
        kmax = float(kmax)
        rmin = float(rmin)
        rmax = float(rmax)
        if not rmin < rmax:
            raise ValueError("rmin >= rmax")
        knl_full = calc_knl_kmax(kmax, rmin, rmax, nmax=nmax, lmax=lmax)
        with np.errstate(invalid="ignore"):
            modes = knl_full <= kmax
        nmax_f = _findlast(modes[:, 0])
        if nmax_f < 1:
            raise ValueError("no radial mode below kmax")
        lmax_n = [_findlast(modes[n, :]) - 1 for n in range(nmax_f)]
        lmax_f = _findlast(modes[0, :]) - 1
        nmax_l = [_findlast(modes[:, l]) for l in range(lmax_f + 1)]
        if not all(v > 0 for v in nmax_l):
            raise ValueError("nmax_l out of range")
        assert all(v >= 0 for v in lmax_n)
        self._setup(rmin, rmax, knl_full, nmax_f, lmax_f, nmax_l, lmax_n, nside, cache)

    @classmethod
    def from_nmax_lmax(cls, nmax, lmax, rmin, rmax, nside=None, cache=True):
        """All modes n <= nmax, l <= lmax (reference src/modes.jl:161-175)."""
        self = cls.__new__(cls)
        rmin = float(rmin)
        rmax = float(rmax)
        knl = calc_knl_nmax(nmax, lmax, rmin, rmax)
        self._setup(rmin, rmax, knl, nmax, lmax, [nmax] * (lmax + 1), [lmax] * nmax, nside, cache)
        return self

    def _setup(self, rmin, rmax, knl_full, nmax, lmax, nmax_l, lmax_n, nside, cache):
        cnl, dnl = calc_cnl_dnl(knl_full, rmin, rmax)
        self.rmin = rmin
        self.rmax = rmax
        self.basisfunctions = SphericalBesselGNL(knl_full, cnl, dnl, rmin, rmax, cache=cache)
        self.nmax = int(nmax)
        self.lmax = int(lmax)
        self.nmax_l = np.asarray(nmax_l, dtype=np.int64)
        self.lmax_n = np.asarray(lmax_n, dtype=np.int64)
        self.nside = int(estimate_nside(lmax) if nside is None else nside)
        fin = knl_full[np.isfinite(knl_full)]
        self.kmax = float(fin.max())
        self.knl = knl_full[:nmax, :lmax + 1].copy()
        # cumulative offsets of each n block in the a_nlm vector
        sizes = [getlmsize(int(l)) for l in self.lmax_n]
        self._noff = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)

    def __repr__(self):
        return (f"AnlmModes(kmax={self.kmax}, rmin={self.rmin}, rmax={self.rmax}, nmax={self.nmax}, "
                f"lmax={self.lmax}, nside={self.nside}, num_modes={int(np.isfinite(self.knl).sum())})")

    # -- (n, l) pairs in the coefficient order ---------------------------------
    def pairs(self):
        """(n, l) with l <= lmax_n[n], n slowest: the order of a_nlm blocks."""
        return [(n, l) for n in range(1, self.nmax + 1) for l in range(int(self.lmax_n[n - 1]) + 1)]


def _findlast(mask):
    idx = np.nonzero(mask)[0]
    return int(idx[-1]) + 1 if len(idx) else 0   # 1-based like Julia's findlast, 0 if none


def getnlmsize(amodes, nmax=None):
    """Length of the a_nlm vector (reference src/modes.jl:183-189)."""
    nmax = amodes.nmax if nmax is None else nmax
    return int(amodes._noff[nmax])


def isvalidnlm(amodes, n, l, m):
    """reference src/modes.jl:192-200"""
    if n > amodes.nmax:
        return False
    if l > amodes.lmax_n[n - 1]:
        return False
    return abs(m) <= l


def getidx(amodes, n, l, m):
    """1-based a_nlm index (reference src/modes.jl:223-232)."""
    assert n >= 1 and l >= 0 and m >= 0
    return 1 + int(amodes._noff[n - 1]) + getlmsize(l - 1) + m


def getidx0(amodes, n, l, m):
    """0-based position of a_nlm in a Python array."""
    return getidx(amodes, n, l, m) - 1


def getnlm(amodes, idx):
    """(n, l, m) of a 1-based index (reference src/modes.jl:203-220)."""
    n = 1
    nmodes = getlmsize(int(amodes.lmax_n[n - 1]))
    while idx > nmodes:
        idx -= nmodes
        n += 1
        nmodes = getlmsize(int(amodes.lmax_n[n - 1]))
    l = 0
    nmodes = l + 1
    while idx > nmodes:
        idx -= nmodes
        l += 1
        nmodes = l + 1
    return n, l, idx - 1


class ClnnModes:
    """(l, n1, n2) ordering of the pseudo-SFB power spectrum
    (reference ``src/modes.jl:281-401``): entries with |k_n2 - k_n1| <= dkmax
    and |n2 - n1| <= dnmax, sorted by l, then n2 - n1, then n1; for one
    AnlmModes (auto-correlation) n2 >= n1."""

    def __init__(self, amodesA, amodesB=None, dkmax=np.inf, dnmax=2 ** 62):
        self.symmetric = amodesB is None
        self.amodesA = amodesA
        self.amodesB = amodesA if amodesB is None else amodesB
        A, B = self.amodesA, self.amodesB
        lmax = min(A.lmax, B.lmax)
        rows = []
        dk_out, dn_out = -np.inf, 0
        for l in range(lmax + 1):
            for nA in range(1, int(A.nmax_l[l]) + 1):
                for nB in range((nA if self.symmetric else 1), int(B.nmax_l[l]) + 1):
                    dk = B.knl[nB - 1, l] - A.knl[nA - 1, l]
                    if abs(dk) <= dkmax and abs(nB - nA) <= dnmax:
                        rows.append((l, nA, nB))
                        dk_out = max(abs(dk), dk_out)
                        dn_out = max(abs(nB - nA), dn_out)
        rows.sort(key=lambda t: (t[0], t[2] - t[1], t[1]))
        self.lnn = np.array(rows, dtype=np.int64).reshape(-1, 3).T.copy()     # 3 x nlnn, like Julia's lnn
        self.dkmax = dk_out
        self.dnmax = dn_out
        self._index = {tuple(c): i for i, c in enumerate(self.lnn.T.tolist())}

    @property
    def amodes(self):
        return self.amodesA


def getlnnsize(cmodes):
    return cmodes.lnn.shape[1]


def getlnn(cmodes, idx):
    """(l, n1, n2) of a 1-based index (reference src/modes.jl:388-393)."""
    l, n1, n2 = cmodes.lnn[:, idx - 1]
    return int(l), int(n1), int(n2)


def getidx_lnn(cmodes, l, n1, n2):
    """1-based index of (l, n1, n2) (reference src/modes.jl:398-...)."""
    if cmodes.symmetric and n1 > n2:
        n1, n2 = n2, n1
    return cmodes._index[(l, n1, n2)] + 1
