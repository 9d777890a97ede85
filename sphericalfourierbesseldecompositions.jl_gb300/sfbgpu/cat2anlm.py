"""Catalogue / field -> SFB coefficients on the GPU (host API).

Mirrors the reference's ``Cat2Anlm`` module (``src/cat2anlm.jl:33-34``):
``cat2amln`` (alias ``cat2nlm``), ``field2anlm``, ``anlm2field``,
``win_rhat_ln`` and ``winweights2galweights``, with the same argument meaning.
Every transform runs through the C ABI of ``libsfbgpu.so``; there is no CPU
path, and a missing library or device raises.

Array conventions follow Julia's memory layout: ``rθϕ`` is (3, N), a field is
(nr, npix), a dense window transform is (npix, lmax+1, nmax); coefficient
vectors are complex128 of length ``getnlmsize(amodes)`` in the reference
order.
"""

import numpy as np

from . import _capi as capi
from .healpix import nside2npix
from .modes import getnlmsize
from .windows import SeparableArray

__all__ = ["GPUPlan", "get_plan", "cat2amln", "cat2nlm", "field2anlm", "anlm2field", "win_rhat_ln",
           "map2alm", "ang2pix_ring", "amln2clnn", "anlm2clnn", "winweights2galweights", "apply_window", "win_lnn", "calc_wmix"]

_PRECISION = {"fp64": capi.SFB_FP64, "mixed": capi.SFB_MIXED}
_RADIAL = {"poly": capi.SFB_RADIAL_POLY, "spline": capi.SFB_RADIAL_SPLINE}


class GPUPlan:
    """A device plan for one AnlmModes (tables uploaded once)."""

    def __init__(self, amodes, niter=3, precision="fp64", radial="poly", pieces=0, degree=0, tol=0.0,
                 nside=None):
        self.amodes = amodes
        pairs = amodes.pairs()
        spl = amodes.basisfunctions.spline
        xs = [spl[pr][0] for pr in pairs]
        off = np.zeros(len(pairs) + 1, np.int64)
        off[1:] = np.cumsum([len(x) for x in xs])
        self._x = np.ascontiguousarray(np.concatenate(xs))
        self._y = np.ascontiguousarray(np.concatenate([spl[pr][1] for pr in pairs]))
        self._ypp = np.ascontiguousarray(np.concatenate([spl[pr][2] for pr in pairs]))
        self._off = off
        self._lmax_n = np.ascontiguousarray(amodes.lmax_n, np.int64)
        d = capi.PlanDesc()
        d.nside = int(amodes.nside if nside is None else nside)
        d.lmax = amodes.lmax
        d.nmax = amodes.nmax
        d.lmax_n = self._lmax_n.ctypes.data_as(capi._i64p)
        d.rmin = amodes.rmin
        d.rmax = amodes.rmax
        d.spl_offset = self._off.ctypes.data_as(capi._i64p)
        d.spl_x = self._x.ctypes.data_as(capi._dp)
        d.spl_y = self._y.ctypes.data_as(capi._dp)
        d.spl_ypp = self._ypp.ctypes.data_as(capi._dp)
        d.niter = niter
        d.precision = _PRECISION[precision]
        d.radial_mode = _RADIAL[radial]
        d.radial_pieces = pieces
        d.radial_degree = degree
        d.radial_tol = tol
        h = capi.C.c_void_p()
        capi.check(capi.lib.sfb_plan_create(capi.C.byref(d), capi.C.byref(h)))
        self.handle = h
        self.nside = d.nside
        self.npix = nside2npix(d.nside)
        self.nlmsize = getnlmsize(amodes)

    def info(self):
        i = capi.PlanInfo()
        capi.check(capi.lib.sfb_plan_get_info(self.handle, capi.C.byref(i)))
        return {f: getattr(i, f) for f, _ in capi.PlanInfo._fields_}

    def set_precision(self, precision):
        capi.check(capi.lib.sfb_set_precision(self.handle, _PRECISION[precision]))

    def close(self):
        if getattr(self, "handle", None):
            capi.lib.sfb_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def get_plan(amodes, **opts):
    """Plan cached on the AnlmModes object per option set."""
    cache = amodes.__dict__.setdefault("_gpu_plans", {})
    key = tuple(sorted(opts.items()))
    if key not in cache:
        cache[key] = GPUPlan(amodes, **opts)
    return cache[key]


def _window_struct(win_rhat_ln, amodes, npix, keep):
    w = capi.Window()
    if win_rhat_ln is None:
        w.kind = capi.SFB_WINDOW_ZERO
        return w
    if isinstance(win_rhat_ln, SeparableArray):
        mask = np.ascontiguousarray(win_rhat_ln.arr1, float)
        wln = np.asfortranarray(win_rhat_ln.arr2, float)
        if mask.shape != (npix,) or wln.shape != (amodes.lmax + 1, amodes.nmax):
            raise ValueError("separable win_rhat_ln must be (mask[npix], w_ln[lmax+1, nmax])")
        keep += [mask, wln]
        w.kind = capi.SFB_WINDOW_SEPARABLE
        w.mask = mask.ctypes.data_as(capi._dp)
        w.w_ln = wln.ctypes.data_as(capi._dp)
        return w
    W = np.asfortranarray(win_rhat_ln, float)
    if W.shape != (npix, amodes.lmax + 1, amodes.nmax):
        raise ValueError(f"dense win_rhat_ln must have shape {(npix, amodes.lmax + 1, amodes.nmax)}")
    keep.append(W)
    w.kind = capi.SFB_WINDOW_DENSE
    w.dense = W.ctypes.data_as(capi._dp)
    return w


def cat2amln(rtp, amodes, nbar, win_rhat_ln, weight=None, **plan_opts):
    """a_nlm of a catalogue (reference cat2amln, src/cat2anlm.jl:257-310).

    rtp: (3, N) array of r, theta, phi.  win_rhat_ln: dense (npix, lmax+1, nmax)
    array, ``SeparableArray(mask, w_ln)``, or None for a zero window term.
    weight: (N,) or None (ones).  Extra keyword arguments select the plan
    (precision="fp64"|"mixed", radial="poly"|"spline", niter=3, ...).
    """
    plan = get_plan(amodes, **plan_opts)
    rtp = np.asarray(rtp, float)
    if rtp.ndim != 2 or rtp.shape[0] != 3:
        raise ValueError("rθϕ must be a 3 x N array")
    N = rtp.shape[1]
    gal = np.ascontiguousarray(rtp.T)            # (N, 3): r, theta, phi per galaxy
    w = None
    if weight is not None and len(weight) > 0:
        w = np.ascontiguousarray(weight, float)
        if w.shape != (N,):
            raise ValueError("weight must have one entry per galaxy")
    keep = []
    win = _window_struct(win_rhat_ln, amodes, plan.npix, keep)
    out = np.empty(plan.nlmsize, np.complex128)
    capi.check(capi.lib.sfb_cat2amln(plan.handle, capi.ptr(gal) if N else None, capi.ptr(w), N, float(nbar),
                                     capi.C.byref(win), capi.ptr(out)))
    return out


cat2nlm = cat2amln


def cat2amln_batched(catalogues, amodes, nbars, win_rhat_ln, weights=None, **plan_opts):
    """a_nlm of a batch of mock catalogues sharing the geometry and window:
    ``catalogues`` is a sequence of (3, N_k) arrays, ``nbars`` one n̄ per mock,
    ``weights`` None or a sequence of (N_k,) arrays (None entries for ones).
    Returns (nmocks, nlmsize) complex, row k = cat2amln(catalogues[k], ...)."""
    plan = get_plan(amodes, **plan_opts)
    cats = [np.asarray(c, float) for c in catalogues]
    if any(c.ndim != 2 or c.shape[0] != 3 for c in cats):
        raise ValueError("every catalogue must be a 3 x N array")
    nmocks = len(cats)
    if len(nbars) != nmocks:
        raise ValueError("one nbar per mock")
    sizes = [c.shape[1] for c in cats]
    offsets = np.zeros(nmocks + 1, np.int64)
    offsets[1:] = np.cumsum(sizes)
    gal = np.ascontiguousarray(np.concatenate([c.T for c in cats], axis=0)) if offsets[-1] else np.zeros((0, 3))
    w = None
    if weights is not None:
        w = np.concatenate([np.ones(n) if wk is None else np.asarray(wk, float) for wk, n in zip(weights, sizes)])
        if w.shape != (offsets[-1],):
            raise ValueError("weights must match the catalogues")
        w = np.ascontiguousarray(w)
    nb = np.ascontiguousarray(nbars, float)
    keep = []
    win = _window_struct(win_rhat_ln, amodes, plan.npix, keep)
    out = np.empty((nmocks, plan.nlmsize), np.complex128)
    capi.check(capi.lib.sfb_cat2amln_batched(plan.handle, capi.ptr(gal) if offsets[-1] else None, capi.ptr(w),
                                             capi.ptr(offsets), nmocks, capi.ptr(nb), capi.C.byref(win),
                                             capi.ptr(out)))
    return out


def field2anlm(f_xyz, wmodes, amodes, **plan_opts):
    """SFB coefficients of an (nr, npix) field (reference field2anlm_v2, src/cat2anlm.jl:323-357).
    A float32 field is passed as it is (sfb_field2anlm_typed), anything else as float64."""
    plan = get_plan(amodes, **plan_opts)
    dt = np.float32 if np.asarray(f_xyz).dtype == np.float32 else np.float64
    f = np.asfortranarray(f_xyz, dt)
    if f.shape != (wmodes.nr, plan.npix):
        raise ValueError("field must be nr x npix")
    out = np.empty(plan.nlmsize, np.complex128)
    code = capi.SFB_F32 if dt == np.float32 else capi.SFB_F64
    capi.check(capi.lib.sfb_field2anlm_typed(plan.handle, capi.ptr(f), code, wmodes.nr, wmodes.rmin, wmodes.rmax,
                                             capi.ptr(out)))
    return out


def anlm2field(f_nlm, wmodes, amodes, **plan_opts):
    """(nr, npix) field of SFB coefficients (reference src/cat2anlm.jl:383-422)."""
    plan = get_plan(amodes, **plan_opts)
    a = np.ascontiguousarray(f_nlm, np.complex128)
    if a.shape != (plan.nlmsize,):
        raise ValueError("f_nlm must have getnlmsize(amodes) entries")
    out = np.empty((wmodes.nr, plan.npix), order="F")
    capi.check(capi.lib.sfb_anlm2field(plan.handle, capi.ptr(a), wmodes.nr, wmodes.rmin, wmodes.rmax, capi.ptr(out)))
    return out


def win_rhat_ln(win, wmodes, amodes, **plan_opts):
    """Radial transform of a window (reference src/windows.jl:244-270).

    Dense (nr, npix) -> (npix, lmax+1, nmax); SeparableArray(phi, mask) ->
    SeparableArray(mask, w_ln[lmax+1, nmax]).  Entries with l > lmax_n[n] are NaN.
    """
    plan = get_plan(amodes, **plan_opts)
    if isinstance(win, SeparableArray):
        phi = np.ascontiguousarray(win.arr1, float)
        mask = np.array(win.arr2, float)
        if phi.shape != (wmodes.nr,):
            raise ValueError("separable window must be SeparableArray(phi[nr], mask[npix])")
        out = np.empty((amodes.lmax + 1, amodes.nmax), order="F")
        capi.check(capi.lib.sfb_win_rhat_ln_separable(plan.handle, capi.ptr(phi), wmodes.nr, wmodes.rmin,
                                                       wmodes.rmax, capi.ptr(out)))
        return SeparableArray(mask, out, name1="mask", name2="w_ln")
    W = np.asfortranarray(win, float)
    if W.shape != (wmodes.nr, plan.npix):
        raise ValueError("window must be nr x npix")
    out = np.empty((plan.npix, amodes.lmax + 1, amodes.nmax), order="F")
    capi.check(capi.lib.sfb_win_rhat_ln_dense(plan.handle, capi.ptr(W), wmodes.nr, wmodes.rmin, wmodes.rmax,
                                              capi.ptr(out)))
    return out


def map2alm(maps, amodes, **plan_opts):
    """Batched map2alm with niter refinement: (nmaps, npix) -> (nmaps, lmsize) complex,
    index l(l+1)/2 + m (the transform behind mymap2alm!, src/healpix_helpers.jl:50-56)."""
    plan = get_plan(amodes, **plan_opts)
    m = np.ascontiguousarray(np.atleast_2d(maps), float)
    L = amodes.lmax
    out = np.empty((m.shape[0], (L + 1) * (L + 2) // 2), np.complex128)
    capi.check(capi.lib.sfb_map2alm(plan.handle, capi.ptr(m), m.shape[0], capi.ptr(out)))
    return out


def cat2amln_vjp(rtp, amodes, nbar, abar, **plan_opts):
    """dL/dw for the galaxy weights of cat2amln, given abar = dL/dRe(a) + i dL/dIm(a)
    (FP64 adjoint of the transform; the plan's piecewise-polynomial radial basis)."""
    plan = get_plan(amodes, **plan_opts)
    gal = np.ascontiguousarray(np.asarray(rtp, float).T)
    ab = np.ascontiguousarray(abar, np.complex128)
    if ab.shape != (plan.nlmsize,):
        raise ValueError("abar must have getnlmsize(amodes) entries")
    out = np.empty(gal.shape[0])
    capi.check(capi.lib.sfb_cat2amln_vjp(plan.handle, capi.ptr(gal) if gal.shape[0] else None, gal.shape[0],
                                         float(nbar), capi.ptr(ab), capi.ptr(out)))
    return out


def field2anlm_vjp(abar, wmodes, amodes, dtype=np.float64, **plan_opts):
    """dL/df (nr, npix) for field2anlm, given abar = dL/dRe(a) + i dL/dIm(a);
    dtype float32 writes the gradient in FP32 (the element type of an FP32 field)."""
    plan = get_plan(amodes, **plan_opts)
    ab = np.ascontiguousarray(abar, np.complex128)
    if ab.shape != (plan.nlmsize,):
        raise ValueError("abar must have getnlmsize(amodes) entries")
    dt = np.dtype(dtype)
    if dt not in (np.dtype(np.float32), np.dtype(np.float64)):
        raise ValueError("dtype must be float32 or float64")
    out = np.empty((wmodes.nr, plan.npix), dtype=dt, order="F")
    code = capi.SFB_F32 if dt == np.float32 else capi.SFB_F64
    capi.check(capi.lib.sfb_field2anlm_vjp_typed(plan.handle, capi.ptr(ab), wmodes.nr, wmodes.rmin, wmodes.rmax,
                                                 capi.ptr(out), code))
    return out


def map2alm_adjoint(abar, amodes, **plan_opts):
    """Transpose of map2alm (niter refinement included): (nmaps, lmsize) complex -> (nmaps, npix)."""
    plan = get_plan(amodes, **plan_opts)
    ab = np.ascontiguousarray(np.atleast_2d(abar), np.complex128)
    out = np.empty((ab.shape[0], plan.npix))
    capi.check(capi.lib.sfb_map2alm_adjoint(plan.handle, capi.ptr(ab), ab.shape[0], capi.ptr(out)))
    return out


def ang2pix_ring(nside, theta, phi):
    """0-based RING pixels computed on the GPU (Healpix.jl ang2pixRing minus one)."""
    th = np.ascontiguousarray(theta, float).ravel()
    ph = np.ascontiguousarray(phi, float).ravel()
    out = np.empty(th.shape, np.int64)
    capi.check(capi.lib.sfb_ang2pix_ring(int(nside), capi.ptr(th), capi.ptr(ph), len(th), capi.ptr(out)))
    return out


def amln2clnn(anlm1, anlm2, cmodes=None, **plan_opts):
    """Pseudo-SFB power spectrum C_l(n1, n2) on the GPU
    (reference src/SphericalFourierBesselDecompositions.jl:133-150).

    ``amln2clnn(anlm, cmodes)`` or ``amln2clnn(anlm1, anlm2, cmodes)``; a 2-d
    (nbatch, nlmsize) input gives one spectrum per row (mock batches)."""
    if cmodes is None:
        cmodes, anlm2 = anlm2, None
    plan = get_plan(cmodes.amodesA, **plan_opts)
    a1 = np.ascontiguousarray(np.atleast_2d(anlm1), np.complex128)
    a2 = None if anlm2 is None else np.ascontiguousarray(np.atleast_2d(anlm2), np.complex128)
    if a1.shape[1] != plan.nlmsize or (a2 is not None and a2.shape != a1.shape):
        raise ValueError("coefficient vectors must have getnlmsize(amodes) entries")
    lnn = np.ascontiguousarray(cmodes.lnn.T, np.int64)     # column i at lnn[3i..3i+2]
    out = np.empty((a1.shape[0], lnn.shape[0]))
    capi.check(capi.lib.sfb_amln2clnn(plan.handle, capi.ptr(a1), capi.ptr(a2), a1.shape[0], capi.ptr(lnn),
                                      lnn.shape[0], capi.ptr(out)))
    return out[0] if np.ndim(anlm1) == 1 else out


anlm2clnn = amln2clnn


def winweights2galweights(weights, wmodes, rtp):
    """Per-galaxy weights from a (nr, npix) weight field (reference src/cat2anlm.jl:218-238)."""
    from .windows import get_rbounds
    W = np.asfortranarray(weights, float)
    rb = np.ascontiguousarray(get_rbounds(wmodes), float)
    gal = np.ascontiguousarray(np.asarray(rtp, float).T)
    out = np.empty(gal.shape[0])
    capi.check(capi.lib.sfb_winweights2galweights(wmodes.nside, capi.ptr(W), W.shape[0], capi.ptr(rb),
                                                  capi.ptr(gal), gal.shape[0], capi.ptr(out)))
    return out


def apply_window(rtp, win, wmodes, seed=0, uniform=None):
    """Galaxies of rtp (3, N) kept by the (nr, npix) window (reference
    apply_window, src/windows.jl:169-216), in input order: kept when
    rmin <= r <= rmax and u <= win[shell, pix] / max(win), with u the given
    ``uniform`` draws (one per galaxy, like the reference's rand(rng)) or the
    library's counter-based stream for ``seed``.  Returns (3, nkept)."""
    W = np.asfortranarray(win, float)
    if W.shape != (wmodes.nr, nside2npix(wmodes.nside)):
        raise ValueError("window must be nr x npix")
    gal = np.ascontiguousarray(np.asarray(rtp, float).T)
    n = gal.shape[0]
    u = None
    if uniform is not None:
        u = np.ascontiguousarray(uniform, float)
        if u.shape != (n,):
            raise ValueError("one uniform draw per galaxy")
    out = np.empty((max(n, 1), 3))
    kept = capi.C.c_int64(0)
    capi.check(capi.lib.sfb_apply_window(wmodes.nside, capi.ptr(W), wmodes.nr, wmodes.rmin, wmodes.rmax,
                                         wmodes.dr, capi.ptr(gal) if n else None, n, capi.ptr(u),
                                         int(seed) & 0xFFFFFFFFFFFFFFFF, capi.ptr(out), capi.C.byref(kept)))
    return np.ascontiguousarray(out[:kept.value].T)


def win_lnn(win, wmodes, cmodes, **plan_opts):
    """W_l(n, n') = sum_s r_s^2 dr g_nl(r_s) g_n'l(r_s) W00(r_s) / sqrt(4 pi) for every (l, n, n')
    of cmodes.lnn (reference win_lnn, src/windows.jl:382-392); win is (nr, npix)."""
    plan = get_plan(cmodes.amodesA, **plan_opts)
    W = np.asfortranarray(win, float)
    if W.shape != (wmodes.nr, plan.npix):
        raise ValueError("window must be nr x npix at the plan's nside")
    lnn = np.ascontiguousarray(cmodes.lnn.T, np.int64)
    out = np.empty(lnn.shape[0])
    capi.check(capi.lib.sfb_win_lnn(plan.handle, capi.ptr(W), wmodes.nr, wmodes.rmin, wmodes.rmax, capi.ptr(lnn),
                                    lnn.shape[0], capi.ptr(out)))
    return out


def calc_wmix(win, wmodes, amodes, neg_m=False, **plan_opts):
    """Window mixing matrix W[(n l m), (n' l' m')] (reference calc_wmix, src/windows.jl:299-366) of an
    (nr, npix) window: (nlmsize, nlmsize) complex."""
    plan = get_plan(amodes, **plan_opts)
    W = np.asfortranarray(win, float)
    if W.shape != (wmodes.nr, plan.npix):
        raise ValueError("window must be nr x npix at the plan's nside")
    out = np.empty((plan.nlmsize, plan.nlmsize), np.complex128, order="F")
    capi.check(capi.lib.sfb_calc_wmix(plan.handle, capi.ptr(W), wmodes.nr, wmodes.rmin, wmodes.rmax,
                                      1 if neg_m else 0, capi.C.c_void_p(out.ctypes.data)))
    return out
