"""Reference algorithms of the catalogue -> a_nlm path (TEST INFRASTRUCTURE).

Every function takes plain arrays (the same tables the GPU plan receives)
and follows one reference function:

* ``spline_eval``    Spline1D{3} evaluation, src/Splines.jl:64-101,327-364
* ``cat2amln``       src/cat2anlm.jl:257-310 (sortout :50-71, scatter :95-103)
* ``field2anlm``     field2anlm_v2, src/cat2anlm.jl:323-357
* ``anlm2field``     src/cat2anlm.jl:383-422
* ``win_rhat_ln``    src/windows.jl:244-257 (dense), :260-270 (separable)
* ``integrate_window`` src/windows.jl:219-228
* ``amln2clnn``      src/SphericalFourierBesselDecompositions.jl:114-150
* ``winweights2galweights`` src/cat2anlm.jl:218-238
* ``win_lnn``        src/windows.jl:382-422 (W00 from map2alm at 2 lmax, trapezoidal radial sum)
* ``calc_wmix``      src/windows.jl:299-366, 273-296, 451-465 (exact Racah 3j symbols)
* ``apply_window``   src/windows.jl:169-216 (the uniform draws passed in;
  ``splitmix64_uniform`` restates the library's counter-based stream)

``modes`` arguments are dicts with ``nmax``, ``lmax``, ``lmax_n`` (list over n),
``nside``, ``splines`` {(n, l): (x, y, ypp)} and ``noff`` (offset of each n
block in the a_nlm vector), built by the tests from the host-side mode tables.
"""

import numpy as np

from .healpix import ang2pix_ring, nside2npix
from .sht import SHT


def spline_eval(x, y, ypp, r):
    """Cubic spline with boundary extrapolation (Splines.jl:64-101,327-364)."""
    N = len(x)
    r = np.asarray(r, float)
    i = np.searchsorted(x, r, side="right") - 1
    i = np.clip(i, 0, N - 2)
    x0 = x[i]
    h = x[i + 1] - x0
    t = (r - x0) / h
    h2 = h * h
    b = h2 * ypp[i] / 2
    a = h2 * (ypp[i + 1] - ypp[i]) / 6
    d = y[i]
    c = y[i + 1] - a - b - d
    val = d + t * (c + t * (b + t * a))
    val = np.where(r < x[0], y[0], val)
    return np.where(r > x[-1], y[-1], val)


def _idx0(modes, n, l, m):
    return int(modes["noff"][n - 1]) + l * (l + 1) // 2 + m


def nlmsize(modes):
    return int(modes["noff"][modes["nmax"]])


def pairs(modes):
    return [(n, l) for n in range(1, modes["nmax"] + 1) for l in range(modes["lmax_n"][n - 1] + 1)]


def cat2amln(rtp, modes, nbar, window, weight=None, niter=3, sht=None, pair_subset=None):
    """a_nlm of a catalogue, reference algorithm (src/cat2anlm.jl:257-310).

    rtp: (3, N) array of r, theta, phi.  window: ("dense", W[npix, lmax+1, nmax])
    or ("separable", mask[npix], W_ln[lmax+1, nmax]).  Returns complex nlmsize.
    ``pair_subset`` restricts the (n, l) loop (used to time a bounded sample).
    """
    rtp = np.asarray(rtp, float)
    N = rtp.shape[1]
    weight = np.ones(N) if weight is None else np.asarray(weight, float)
    # sortout: sort by r, stable (src/cat2anlm.jl:50-71)
    p = np.argsort(rtp[0], kind="stable")
    r, th, ph, w = rtp[0, p], rtp[1, p], rtp[2, p], weight[p]
    nside = modes["nside"]
    lmax = modes["lmax"]
    npix = nside2npix(nside)
    dOmega = 4 * np.pi / npix
    pix = ang2pix_ring(nside, th, ph)
    if sht is None:
        sht = SHT(nside, lmax)
    if lmax > 4 * nside:
        raise ValueError("alm.lmax > 4*nside is a poor choice")
    anlm = np.full(nlmsize(modes), np.nan + 1j * np.nan)
    todo = pairs(modes) if pair_subset is None else list(pair_subset)
    chunk = 64
    for c0 in range(0, len(todo), chunk):
        batch = todo[c0:c0 + chunk]
        maps = np.empty((len(batch), npix))
        for b, (n, l) in enumerate(batch):
            x, y, ypp = modes["splines"][(n, l)]
            vals = w * spline_eval(x, y, ypp, r)
            m = np.bincount(pix, weights=vals, minlength=npix).astype(float)
            m *= 1 / (nbar * dOmega)
            if window[0] == "dense":
                m = m - window[1][:, l, n - 1]
            else:
                m = m - window[1] * window[2][l, n - 1]
            maps[b] = m
        alm = sht.map2alm(maps, niter=niter)
        for b, (n, l) in enumerate(batch):
            i0 = _idx0(modes, n, l, 0)
            anlm[i0:i0 + l + 1] = alm[b, l, :l + 1]
    if pair_subset is None:
        assert np.all(np.isfinite(anlm))
    return anlm


def field2anlm(f, rmin, rmax, nr, modes, niter=3, sht=None):
    """field2anlm_v2 (src/cat2anlm.jl:323-357): per-shell map2alm, radial sum."""
    f = np.asarray(f, float)
    dr = (rmax - rmin) / nr
    rs = np.linspace(rmin + dr / 2, rmax - dr / 2, nr)
    if sht is None:
        sht = SHT(modes["nside"], modes["lmax"])
    alm = sht.map2alm(f, niter=niter)                  # [nr, l, m]
    out = np.zeros(nlmsize(modes), complex)
    for (n, l) in pairs(modes):
        x, y, ypp = modes["splines"][(n, l)]
        g = spline_eval(x, y, ypp, rs) * rs ** 2 * dr
        i0 = _idx0(modes, n, l, 0)
        out[i0:i0 + l + 1] += g @ alm[:, l, :l + 1]
    return out


def anlm2field(fnlm, rmin, rmax, nr, modes, sht=None):
    """anlm2field (src/cat2anlm.jl:383-422): radial sum per shell, alm2map."""
    dr = (rmax - rmin) / nr
    rs = np.linspace(rmin + dr / 2, rmax - dr / 2, nr)
    L = modes["lmax"]
    if sht is None:
        sht = SHT(modes["nside"], L)
    alm = np.zeros((nr, L + 1, L + 1), complex)
    for (n, l) in pairs(modes):
        x, y, ypp = modes["splines"][(n, l)]
        g = spline_eval(x, y, ypp, rs)
        i0 = _idx0(modes, n, l, 0)
        alm[:, l, :l + 1] += g[:, None] * fnlm[None, i0:i0 + l + 1]
    return sht.synthesis(alm)


def win_rhat_ln_dense(win, rmin, rmax, nr, modes):
    """W[p, l, n] = dr sum_r win[r, p] r^2 g_nl(r) (src/windows.jl:244-257); NaN off-mode."""
    dr = (rmax - rmin) / nr
    rs = np.linspace(rmin + dr / 2, rmax - dr / 2, nr)
    npix = win.shape[1]
    W = np.full((npix, modes["lmax"] + 1, modes["nmax"]), np.nan)
    for (n, l) in pairs(modes):
        x, y, ypp = modes["splines"][(n, l)]
        W[:, l, n - 1] = win.T @ (rs ** 2 * spline_eval(x, y, ypp, rs))
    return W * dr


def win_rhat_ln_separable(phi, mask, rmin, rmax, nr, modes):
    """W_ln[l, n] = dr sum_r r^2 g_nl(r) phi(r) (src/windows.jl:260-270)."""
    dr = (rmax - rmin) / nr
    rs = np.linspace(rmin + dr / 2, rmax - dr / 2, nr)
    W = np.full((modes["lmax"] + 1, modes["nmax"]), np.nan)
    for (n, l) in pairs(modes):
        x, y, ypp = modes["splines"][(n, l)]
        W[l, n - 1] = dr * np.sum(rs ** 2 * spline_eval(x, y, ypp, rs) * phi)
    return mask, W


def integrate_window(win, rmin, rmax, nr):
    """V_eff = dr dOmega sum_r r^2 sum_p W[r, p] (src/windows.jl:219-228)."""
    dr = (rmax - rmin) / nr
    rs = np.linspace(rmin + dr / 2, rmax - dr / 2, nr)
    npix = win.shape[1]
    return dr * (4 * np.pi / npix) * np.sum(win.sum(axis=1) * rs ** 2)


def alm2cl(a1, a2, l):
    """One l of alm2cl (src/SphericalFourierBesselDecompositions.jl:114-129): m = 0
    enters as Re(a1 a2) (no conjugate), m > 0 as 2 Re(a1 conj(a2))."""
    c = (a1[0] * a2[0]).real
    for m in range(1, l + 1):
        c += 2 * (a1[m] * np.conj(a2[m])).real
    return c / (2 * l + 1)


def amln2clnn(anlm1, anlm2, lnn, modesA, modesB=None):
    """C_l(n1, n2) for the columns (l, n1, n2) of lnn (src/...:136-148)."""
    modesB = modesA if modesB is None else modesB
    out = np.full(lnn.shape[1], np.nan)
    for i in range(lnn.shape[1]):
        l, n1, n2 = (int(v) for v in lnn[:, i])
        a = anlm1[_idx0(modesA, n1, l, 0):_idx0(modesA, n1, l, 0) + l + 1]
        b = anlm2[_idx0(modesB, n2, l, 0):_idx0(modesB, n2, l, 0) + l + 1]
        out[i] = alm2cl(a, b, l)
    return out


def winweights2galweights(weights, rbounds, nside, rtp):
    """w_i = weights[bin, pix] (src/cat2anlm.jl:218-238); bin = searchsortedlast(rbounds, r),
    or nr when r == rmax; raises for r out of bounds."""
    rtp = np.asarray(rtp, float)
    nr = weights.shape[0]
    r = rtp[0]
    pix = ang2pix_ring(nside, rtp[1], rtp[2])
    b = np.searchsorted(rbounds, r, side="right")      # 1-based searchsortedlast
    b = np.where(r == rbounds[-1], nr, b)
    if np.any((b < 1) | (b > nr)):
        raise ValueError("r out of bounds")
    return weights[b - 1, pix]


def splitmix64(seed, n):
    """The first n outputs of SplitMix64 (Steele, Lea, Flood 2014) from state
    `seed`: z_i = mix(seed + i * 0x9E3779B97F4A7C15), i = 1..n."""
    with np.errstate(over="ignore"):
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def splitmix64_uniform(seed, n):
    """u_i = (z_i >> 11) * 2^-53 in [0, 1): the library's per-galaxy draws."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def apply_window(rtp, win, rmin, rmax, dr, nside, uniform):
    """Galaxies kept by apply_window (src/windows.jl:169-216), in input order,
    with the per-galaxy draws `uniform` standing in for rand(rng): kept when
    rmin <= r <= rmax, shell ceil((r - rmin)/dr) (0 -> 1) <= nr and
    u <= win[shell, pix] * (1 / maximum(win))."""
    rtp = np.asarray(rtp, float)
    r, th, ph = rtp
    nr = win.shape[0]
    oow = 1.0 / np.max(win)
    keep = np.zeros(r.size, bool)
    idx = np.nonzero((rmin <= r) & (r <= rmax))[0]
    ir = np.ceil((r[idx] - rmin) / dr).astype(np.int64)
    ir[ir == 0] = 1
    ok = ir <= nr
    idx, ir = idx[ok], ir[ok]
    pix = ang2pix_ring(nside, th[idx], ph[idx])
    keep[idx] = uniform[idx] <= win[ir - 1, pix] * oow
    return rtp[:, keep]


def win_lnn(win, rmin, rmax, nr, modes, lnn, niter=3):
    """win_lnn (src/windows.jl:382-392) with calc_intr_gg_fn (:394-422):
    W00 = a_00 of every shell from map2alm to lmax 2 lmax (calc_Wr_lm), then
    sum over the shell midpoints of (g r sqrt(dr) sqrt(f)) (g' r sqrt(dr) sqrt(f)),
    f = W00 / sqrt(4 pi), for every column (l, n, n') of lnn (3 x nlnn)."""
    dr = (rmax - rmin) / nr
    rs = np.linspace(rmin + dr / 2, rmax - dr / 2, nr)
    L2 = 2 * modes["lmax"]
    alm = SHT(modes["nside"], L2).map2alm(np.asarray(win, float), niter=niter)
    f = alm[:, 0, 0].real / np.sqrt(4 * np.pi)
    meas = rs * np.sqrt(dr) * np.sqrt(f)
    out = np.empty(lnn.shape[1])
    for i in range(lnn.shape[1]):
        l, n1, n2 = (int(v) for v in lnn[:, i])
        g1 = spline_eval(*modes["splines"][(n1, l)], rs) * meas
        g2 = spline_eval(*modes["splines"][(n2, l)], rs) * meas
        out[i] = g1 @ g2
    return out


def wigner3j(j1, j2, j3, m1, m2, m3):
    """Wigner 3j symbol from the Racah formula in exact integer arithmetic."""
    import math
    from fractions import Fraction
    if (m1 + m2 + m3 != 0 or not (abs(j1 - j2) <= j3 <= j1 + j2) or abs(m1) > j1 or abs(m2) > j2
            or abs(m3) > j3):
        return 0.0
    f = math.factorial
    pre = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1))
    pre *= f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3)
    s = 0
    for k in range(max(0, j2 - j3 - m1, j1 - j3 + m2), min(j1 + j2 - j3, j1 - m1, j2 + m2) + 1):
        s += Fraction((-1) ** k, f(k) * f(j1 + j2 - j3 - k) * f(j1 - m1 - k) * f(j2 + m2 - k)
                      * f(j3 - j2 + m1 + k) * f(j3 - j1 - m2 + k))
    if s == 0:
        return 0.0
    return (-1) ** (j1 - j2 - m3) * (1 if s > 0 else -1) * math.sqrt(float(s * s * pre))


def calc_wmix(win, rmin, rmax, nr, modes, neg_m=False, niter=3):
    """Window mixing matrix (src/windows.jl:299-366 with calc_wmix_ii :273-296 and
    calc_gaunts_L :451-465), nlmsize x nlmsize complex."""
    from functools import lru_cache
    dr = (rmax - rmin) / nr
    rs = np.linspace(rmin + dr / 2, rmax - dr / 2, nr)
    L2 = 2 * modes["lmax"]
    Wlm = SHT(modes["nside"], L2).map2alm(np.asarray(win, float), niter=niter)     # [s, L, M]
    w3 = lru_cache(maxsize=None)(wigner3j)
    g = {pr: spline_eval(*modes["splines"][pr], rs) * rs * np.sqrt(dr) for pr in pairs(modes)}
    N = nlmsize(modes)
    out = np.full((N, N), np.nan + 1j * np.nan)
    for (n, l) in pairs(modes):
        for (n2, l2) in pairs(modes):
            gg = g[(n, l)] * g[(n2, l2)]
            H = np.einsum("s,sLM->LM", gg, Wlm)
            for am in range(l + 1):
                m = -am if neg_m else am
                for m2 in range(l2 + 1):
                    M = m - m2
                    w = 0j
                    for L in range(abs(l - l2), l + l2 + 1):
                        if abs(M) > L:
                            continue
                        gnt = np.sqrt((2 * L + 1) * (2 * l + 1) * (2 * l2 + 1) / (4 * np.pi)) \
                            * w3(l, l2, L, 0, 0, 0) * w3(L, l, l2, M, -m, m2)
                        w += gnt * H[L, abs(M)]
                    if M < 0:
                        w = (-1) ** M * np.conj(w)
                    out[_idx0(modes, n, l, am), _idx0(modes, n2, l2, m2)] = (-1) ** m * w
    return out
