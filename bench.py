#!/usr/bin/env python3
"""cat2amln throughput on one GB300: galaxies/s at nside 256, kmax 0.1.

Workload (the reference's nside-256 configuration, seeded synthetic data):
AnlmModes(kmax=0.1, rmin=500, rmax=2500; nside=256), potential boundary
(lmax 238, 7,520 (n,l) pairs, nlmsize 551,664); window = polar cap
theta < 60 deg x Gaussian radial selection (mean 1500, sigma 400) on nr=1000
shells, passed as a separable win_rhat_ln; catalogue = Poisson draw of
nbar*W with E[N] = 1e7, FP64 weights U[0.5, 1.5].

One step = one cat2amln call.  `value` uses device-resident inputs
(sfb_cat2amln_device on the current torch stream, CUDA events around the K
timed steps); `e2e` uses the host-pointer C-ABI call from pinned memory
(H2D + D2H inside the timed region, host wall clock).  Inputs (320 MB) are
larger than the 129 MB L2, so no explicit flush is needed between steps.

--impl reference times the reference algorithm (per-(n,l) spline scatter +
niter=3 map2alm, CPU restatement in oracle/) on the host cores: each step is
a sample of (n,l) pairs run in parallel, extrapolated to all pairs.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "sphericalfourierbesseldecompositions.jl_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "cat2amln galaxies/s at nside256 kmax0.1: mixed vs FP64 GPU, ≤1e-7 rel err"
KMAX, RMIN, RMAX, NSIDE, NR = 0.1, 500.0, 2500.0, 256, 1000
NGAL_MEAN = 10_000_000
CAP_DEG, RMEAN, RSIG = 60.0, 1500.0, 400.0
# per-kernel DRAM bytes of one call of the profile case (ncu, one kernel per capture), one line per kernel:
# stage, kernel, launches, read bytes, write bytes, the unit its traffic scales with, units in the capture
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "dram_traffic_nside256_kmax0.1_profile_case.txt")
WORKLOAD = "cat2amln kmax=0.1 rmin=500 rmax=2500 nside=256 nr=1000 N~Poisson(1e7) cap60 x gauss(1500,400) w~U[0.5,1.5]"


def stage_traffic(stage, units):
    """DRAM bytes (read + write) of one call's kernels of `stage`, scaled from the profile-case ncu
    captures: each kernel's bytes x (units of this run / units of the capture), the unit being maps
    for the map-sized kernels and galaxies for the sort.  (None, []) without a capture of the stage."""
    try:
        with open(TRAFFIC_FILE) as fh:
            lines = fh.read().splitlines()
    except OSError:
        return None, []
    total, parts = 0.0, []
    for ln in lines:
        f = ln.split()
        if not f or f[0].startswith("#") or f[0] != stage:
            continue
        kern, nl, rd, wr, unit, cap = f[1], int(f[2]), float(f[3]), float(f[4]), f[5], float(f[6])
        scale = units[unit] / cap
        total += (rd + wr) * scale
        parts.append(f"{kern} x{nl} ({unit} x{scale:.4g})")
    return (total if parts else None), parts


def make_catalogue(seed=2):
    """Seeded Poisson draw of nbar*W(r, theta) (rejection sampling in r, uniform in the cap)."""
    rng = np.random.default_rng(seed)
    n = int(rng.poisson(NGAL_MEAN))
    f = lambda r: r * r * np.exp(-(r - RMEAN) ** 2 / (2 * RSIG ** 2))
    rpk = (RMEAN + np.sqrt(RMEAN ** 2 + 8 * RSIG ** 2)) / 2
    fmax = f(rpk)
    rs = []
    have = 0
    while have < n:
        r = rng.uniform(RMIN, RMAX, 2 * (n - have) + 1000)
        r = r[rng.random(r.size) * fmax <= f(r)]
        rs.append(r)
        have += r.size
    r = np.concatenate(rs)[:n]
    mu = rng.uniform(np.cos(np.radians(CAP_DEG)), 1.0, n)
    th = np.arccos(mu)
    ph = rng.uniform(0.0, 2 * np.pi, n)
    w = rng.uniform(0.5, 1.5, n)
    return np.ascontiguousarray(np.stack([r, th, ph], axis=1)), w    # (N, 3) = Julia 3xN memory


def mock_sizes(nmocks, seed=7, lo=1_000_000, hi=20_000_000):
    """Uneven mock sizes, uniform integers in [lo, hi] (the batched-mocks configuration)."""
    return np.random.default_rng(seed).integers(lo, hi + 1, nmocks)


def fill_mocks(sizes, gal, w, seed=8):
    """Independent seeded mocks of the bench window written into gal (sum(sizes), 3) and w: r by the
    inverse CDF of r^2 exp(-(r - RMEAN)^2 / 2 RSIG^2) on [RMIN, RMAX] (tabulated at 2^16 equally spaced
    probabilities, linear between them), cos(theta) uniform in the cap, phi uniform, w ~ U[0.5, 1.5].
    Returns the offsets (nmocks + 1)."""
    rg = np.linspace(RMIN, RMAX, 1 << 18)
    pdf = rg * rg * np.exp(-(rg - RMEAN) ** 2 / (2 * RSIG ** 2))
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(rg))])
    cdf /= cdf[-1]
    nq = 1 << 16
    rq = np.interp(np.linspace(0.0, 1.0, nq + 1), cdf, rg)          # r at probabilities j / nq
    off = np.zeros(len(sizes) + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    z0 = np.cos(np.radians(CAP_DEG))
    for k, n in enumerate(sizes):
        rng = np.random.default_rng([seed, k])
        a, b = off[k], off[k + 1]
        q = rng.random(n) * nq
        j = np.minimum(q.astype(np.int64), nq - 1)
        gal[a:b, 0] = rq[j] + (q - j) * (rq[j + 1] - rq[j])
        gal[a:b, 1] = np.arccos(rng.uniform(z0, 1.0, n))
        gal[a:b, 2] = rng.uniform(0.0, 2 * np.pi, n)
        w[a:b] = rng.uniform(0.5, 1.5, n)
    return off


# the reference's CPU-runnable configuration: full sky, r ~ r^2, unit weights
C1 = dict(kmax=0.05, rmin=500.0, rmax=1000.0, nside=32, nr=250, ngal=200_000)
C1_WORKLOAD = "cat2amln kmax=0.05 rmin=500 rmax=1000 nside=32 nr=250 N=2e5 full sky r~r^2 w=1 (C1)"


def c1_catalogue(seed=1):
    """N = 2e5, r = (rmin^3 + u (rmax^3 - rmin^3))^(1/3), cos(theta) ~ U[-1, 1], phi ~ U[0, 2 pi)."""
    rng = np.random.default_rng(seed)
    n, a, b = C1["ngal"], C1["rmin"], C1["rmax"]
    r = np.cbrt(a ** 3 + rng.random(n) * (b ** 3 - a ** 3))
    th = np.arccos(rng.uniform(-1.0, 1.0, n))
    ph = rng.uniform(0.0, 2 * np.pi, n)
    return np.ascontiguousarray(np.stack([r, th, ph], axis=1)), np.ones(n)


def c1_setup(sfbgpu):
    """AnlmModes, catalogue, window (full-sky constant) and nbar = N / V of C1."""
    amodes = sfbgpu.AnlmModes(C1["kmax"], C1["rmin"], C1["rmax"], nside=C1["nside"])
    gal, w = c1_catalogue()
    wm = sfbgpu.ConfigurationSpaceModes(C1["rmin"], C1["rmax"], C1["nr"], C1["nside"])
    phi, mask = np.ones(wm.nr), np.ones(wm.npix)
    nbar = gal.shape[0] / (4 * np.pi / 3 * (C1["rmax"] ** 3 - C1["rmin"] ** 3))
    return amodes, gal, w, wm, phi, mask, nbar


def c1_cpu_full(sfbgpu, workers, runs=3):
    """The reference algorithm on the whole C1 catalogue (every (n,l) pair, no
    extrapolation) on `workers` host processes: median galaxies/s of `runs` calls."""
    from oracle import sfb as osfb
    amodes, gal, w, wm, phi, mask, nbar = c1_setup(sfbgpu)
    md = dict(nmax=amodes.nmax, lmax=amodes.lmax, lmax_n=[int(v) for v in amodes.lmax_n], nside=C1["nside"],
              splines=amodes.basisfunctions.spline, noff=amodes._noff)
    _, wln = osfb.win_rhat_ln_separable(phi, mask, C1["rmin"], C1["rmax"], C1["nr"], md)
    npairs = len(amodes.pairs())
    vals, t_setup = run_reference_sample(amodes, gal, w, nbar, mask, wln, runs, 1, workers, npairs,
                                         nside=C1["nside"])
    v = float(np.median(vals))
    return {"value": v, "unit": "galaxies/s", "cores": workers, "kind": "port", "runs": runs,
            "ms_per_call": gal.shape[0] / v * 1e3, "workload": C1_WORKLOAD,
            "sample": f"the whole C1 call: all {npairs} (n,l) pairs (spline scatter + niter=3 map2alm each) on "
                      f"{workers} processes plus the sort/ang2pix ({t_setup:.2f} s); median of {runs} calls after "
                      f"one warm-up"}


def c1_gpu(sfbgpu, steps=10, warmup=3):
    """C1 through the public host-pointer call (copies included), mixed and FP64,
    with the mixed path's errors against the FP64 one."""
    amodes, gal, w, wm, phi, mask, nbar = c1_setup(sfbgpu)
    rtp = gal.T
    out, res = {"workload": C1_WORKLOAD, "ngal": int(gal.shape[0])}, {}
    for prec in ("mixed", "fp64"):
        win = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, amodes, precision=prec,
                                 radial="poly")
        for _ in range(warmup):
            sfbgpu.cat2amln(rtp, amodes, nbar, win, None, precision=prec, radial="poly")
        t0 = time.perf_counter()
        for _ in range(steps):
            res[prec] = sfbgpu.cat2amln(rtp, amodes, nbar, win, None, precision=prec, radial="poly")
        dt = (time.perf_counter() - t0) / steps
        out[prec] = {"value": gal.shape[0] / dt, "unit": "galaxies/s", "ms_per_call": dt * 1e3,
                     "timing": f"host wall clock over {steps} calls of sfb_cat2amln (host buffers, copies inside)"}
    out["mixed_vs_fp64"] = error_report(res["mixed"], res["fp64"])
    return out


def window_arrays(sfbgpu, amodes):
    wm = sfbgpu.ConfigurationSpaceModes(RMIN, RMAX, NR, NSIDE)
    phi = np.exp(-(wm.r - RMEAN) ** 2 / (2 * RSIG ** 2))
    th, _ = sfbgpu.pix2ang_ring(NSIDE, np.arange(wm.npix))
    mask = (th < np.radians(CAP_DEG)).astype(float)
    return wm, phi, mask


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- reference arm
_W = {}


def _ref_worker_init(shm_names, n, lmax, nside):
    from multiprocessing import shared_memory
    from oracle import sht as osht
    blocks = {}
    for key, name in shm_names.items():
        s = shared_memory.SharedMemory(name=name)
        blocks[key] = s
    _W["shm"] = blocks
    dt = {"r": np.float64, "w": np.float64, "pix": np.int64}
    for key, s in blocks.items():
        _W[key] = np.ndarray((n,), dtype=dt[key], buffer=s.buf)
    _W["sht"] = osht.SHT(nside, lmax)
    _W["nside"] = nside


def _ref_worker_pair(args):
    """One (n,l) iteration of the reference loop (src/cat2anlm.jl:281-306)."""
    (n, l), (x, y, ypp), nbar, mask, wln = args
    from oracle import sfb as osfb
    npix = 12 * _W["nside"] ** 2
    vals = _W["w"] * osfb.spline_eval(x, y, ypp, _W["r"])
    m = np.bincount(_W["pix"], weights=vals, minlength=npix).astype(float)
    m *= 1 / (nbar * 4 * np.pi / npix)
    m = m - mask * wln
    alm = _W["sht"].map2alm(m[None, :], niter=3)
    return alm[0, l, :l + 1]


def run_reference_sample(amodes, gal, w, nbar, mask, wln_arr, steps, warmup, workers, pairs_per_step,
                         nside=NSIDE):
    """Time the CPU reference algorithm on a sample of (n,l) pairs (all of them when
    pairs_per_step is the pair count); returns galaxies/s per step."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    from multiprocessing import shared_memory
    from oracle import healpix as ohp
    N = gal.shape[0]
    # sortout + ang2pix: once per cat2amln call in the reference (src/cat2anlm.jl:259-264)
    t0 = time.perf_counter()
    p = np.argsort(gal[:, 0], kind="stable")
    r = np.ascontiguousarray(gal[p, 0])
    pix = ohp.ang2pix_ring(nside, gal[p, 1], gal[p, 2])
    ws = np.ascontiguousarray(w[p])
    t_setup = time.perf_counter() - t0
    shms = {}
    for key, arr in (("r", r), ("w", ws), ("pix", pix)):
        s = shared_memory.SharedMemory(create=True, size=arr.nbytes)
        np.ndarray(arr.shape, dtype=arr.dtype, buffer=s.buf)[:] = arr
        shms[key] = s
    pairs = amodes.pairs()
    spl = amodes.basisfunctions.spline
    ctx = mp.get_context("spawn")
    vals = []
    try:
        with ProcessPoolExecutor(workers, mp_context=ctx, initializer=_ref_worker_init,
                                 initargs=({k: s.name for k, s in shms.items()}, N, amodes.lmax, nside)) as ex:
            list(ex.map(_ref_worker_pair, [(pairs[0], spl[pairs[0]], nbar, mask, wln_arr[0, 0])] * workers))
            for step in range(warmup + steps):
                idx = np.linspace(0, len(pairs) - 1, pairs_per_step).astype(int)
                idx = (idx + step * 37) % len(pairs)
                args = [(pairs[i], spl[pairs[i]], nbar, mask, wln_arr[pairs[i][1], pairs[i][0] - 1]) for i in idx]
                t0 = time.perf_counter()
                list(ex.map(_ref_worker_pair, args))
                dt = time.perf_counter() - t0
                total = t_setup + dt * len(pairs) / len(idx)
                if step >= warmup:
                    vals.append(N / total)
    finally:
        for s in shms.values():
            s.close()
            s.unlink()
    return vals, t_setup


# ----------------------------------------------------------------------------- GPU arm
def gram_geometry(lmax, niter=3):
    """Aliased rings (nph <= 2 lmax, a prefix of the north rings) and whether the
    mixed path's Gram refinement runs (most rings alias-free, niter > 0)."""
    ral = 0
    while ral < 2 * NSIDE and (4 * (ral + 1) if ral < NSIDE - 1 else 4 * NSIDE) <= 2 * lmax:
        ral += 1
    on = niter > 0 and 4 * ral <= 3 * 2 * NSIDE and os.environ.get("SFBGPU_GRAM_REFINEMENT", "1") != "0"
    return ral, on


def sky_rings(sfbgpu, nside, theta, phi):
    """Ring pairs (north ring i and its mirror 4 nside - i, 0-based pair
    i - 1) that hold galaxies: (pixels on those pairs, number of rings in the
    span from the first to the last such pair).  Outside them every map of the
    mixed path is zero: the ring DFT skips those rows and the first analysis
    pass sums over the span only, so the algorithmic work below is counted
    over the same rings.  Third value: the pixels of the rings that hold
    galaxies, the only ones whose basis-map rows the mixed deposit writes."""
    ns = int(nside)
    npix = 12 * ns * ns
    ncap = 2 * ns * (ns - 1)
    p = np.arange(npix, dtype=np.int64)

    def cap_ring(q):
        i = (1 + np.floor(np.sqrt(1 + 2 * q)).astype(np.int64)) >> 1
        i = np.where(2 * i * (i - 1) > q, i - 1, i)
        return np.where(2 * (i + 1) * i <= q, i + 1, i)

    ring = np.empty(npix, np.int64)
    north, south = p < ncap, p >= npix - ncap
    eq = ~(north | south)
    ring[north] = cap_ring(p[north])
    ring[eq] = (p[eq] - ncap) // (4 * ns) + ns
    ring[south] = 4 * ns - cap_ring(npix - 1 - p[south])
    pair = np.minimum(ring, 4 * ns - ring) - 1
    pix_per_pair = np.bincount(pair, minlength=2 * ns)
    gp = sfbgpu.ang2pix_ring(ns, theta, phi)
    used = np.zeros(2 * ns, bool)
    used[np.unique(pair[gp])] = True
    live_ring = np.zeros(4 * ns - 1, bool)
    live_ring[np.unique(ring[gp]) - 1] = True
    live_pix = int(np.bincount(ring - 1, minlength=4 * ns - 1)[live_ring].sum())
    idx = np.nonzero(used)[0]
    if idx.size == 0:
        return 0, 0, 0
    lo, hi = int(idx[0]), int(idx[-1])
    rings = 2 * (hi - lo + 1) - (1 if hi == 2 * ns - 1 else 0)
    return int(pix_per_pair[used].sum()), rings, live_pix


def stage_work(stage, precision, nm, ngal, nbasis, niter=3, lmax=238, sky=None):
    """Algorithmic work of ONE STEP of a stage as this path computes it:
    (kind, amount).  The N/S ring symmetry and the ten-product slicing are
    implementation choices and do not change the counts.

    leg_analysis / leg_synthesis: 2 (complex) x 2 (multiply-add) flop per
    (ring, (l, m) with m <= l, map).  FP64 path: 1 + niter analysis and niter
    synthesis passes over all 4 nside - 1 rings.  Mixed path (Gram
    refinement): one analysis pass over all rings, then per refinement pass a
    synthesis and an analysis over the 2 ral aliased rings and the Gram
    product, 2 (complex) x 2 flop per (block z, output row, input row, map)
    (counted under leg_synthesis).
    ring_fft: maps read + ring spectra written, nm npix b + nm n_ring (lmax+1)
    2 b bytes (b = 8: FP64, or the mixed path's double-float pairs); the
    mixed path computes it as a tensor-core DFT, whose 4 flop per (pixel, m,
    map) is reported beside.
    sky = sky_rings(...): in the mixed path the DFT flops count the pixels of
    the ring pairs with galaxies and the first analysis pass the rings of
    their span (the rows elsewhere are zero and skipped).
    fold: G read + R written per pass (mixed: the aliased rings only, G FP32
    and R double-float; FP64: F, G read + R written over all rings).
    deposit: 40 B per galaxy (record read + binning update) + the basis maps
    written, 8 B per value (mixed: double-float pairs on the rings holding
    galaxies, sky[2] pixels)."""
    lmsize = (lmax + 1) * (lmax + 2) // 2
    nrn = 2 * NSIDE
    n_ring = 4 * NSIDE - 1
    npix = 12 * NSIDE ** 2
    ncol = 2 * nm
    t = 8                                            # maps, spectra, residuals: FP64 or double-float
    fsz = 2 * (lmax + 1) * nrn * ncol * t
    ral, gram = gram_geometry(lmax, niter)
    gram = gram and precision == "mixed" and nm > 4
    n_al = 2 * ral                                   # aliased rings, both hemispheres
    rows = [((lmax - m - par) // 2 + 1) if m + par <= lmax else 0 for m in range(lmax + 1) for par in (0, 1)]
    gram_flop = 4.0 * nm * sum(r * r for r in rows)
    if stage == "leg_analysis":
        if gram:
            first = sky[1] if (sky and precision == "mixed") else n_ring
            return ("flop", 4.0 * first * lmsize * nm + niter * 4.0 * n_al * lmsize * nm)
        return ("flop", (1 + niter) * 4.0 * n_ring * lmsize * nm)
    if stage == "leg_synthesis":
        if gram:
            return ("flop", niter * (4.0 * n_al * lmsize * nm + gram_flop))
        return ("flop", niter * 4.0 * n_ring * lmsize * nm)
    if stage == "ring_fft":
        return ("byte", float(t) * nm * npix + float(nm) * n_ring * (lmax + 1) * 2 * t)
    if stage == "fold":
        if gram:
            return ("byte", niter * 2.0 * (lmax + 1) * ral * ncol * (4 + 8))   # G (FP32) read, R (pairs) written
        return ("byte", niter * 3.0 * fsz)
    if stage == "deposit":
        mpix = sky[2] if (sky and precision == "mixed") else npix
        return ("byte", 40.0 * ngal + float(t) * nbasis * mpix)
    return ("byte", None)


def roofline_table(stages, precision, nm, ngal, nbasis, peaks, fp64_peak, sky=None):
    """Per stage: algorithmic work of a step / the stage's time in the step.
    Tensor-core stages of the mixed path issue 10 BF16 products per
    algorithmic multiply-add (four-slice error-free splitting); `achieved`
    counts algorithmic flops only, `bf16_issued_frac` the issued ones."""
    out = {}
    for st, v in stages.items():
        ms = v["ms_per_step"]
        kind, amount = stage_work(st, precision, nm, ngal, nbasis, sky=sky)
        if amount is None or ms <= 0:
            continue
        if kind == "flop":
            ach = amount / (ms * 1e-3) / 1e12
            if precision == "mixed":
                # kernels timed inside a ~20 ms step: the sustained (power-capped) bf16 figure
                if "bf16_tflops_sustained" in peaks:
                    peak, src = peaks["bf16_tflops_sustained"], "MEASURED_PEAKS.json bf16_tflops_sustained"
                else:
                    peak, src = 1700.0, "fallback (sustained bf16)"
                bound = "tensor"
            else:
                peak, bound, src = fp64_peak, "fp64", "cuBLAS DGEMM 8192^3 measured in this run"
            out[st] = {"bound": bound, "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                       "per_step": amount, "ms_per_step": ms, "peak_source": src}
            if precision == "mixed":
                out[st]["bf16_issued_frac"] = 10.0 * ach / peak
        else:
            ach = amount / (ms * 1e-3) / 1e9
            peak = peaks.get("hbm_gbs", 6800.0)
            out[st] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                       "per_step": amount, "ms_per_step": ms,
                       "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback"}
            if st == "ring_fft" and precision == "mixed":
                # the mixed ring transform is a tensor-core DFT: its bound is the tensor pipe (fed from
                # shared memory), so it is reported as such, with the HBM bytes beside
                lmax = 238
                dpix = sky[0] if sky else 12 * NSIDE ** 2
                dft = 4.0 * nm * dpix * (lmax + 1)
                tp = peaks.get("bf16_tflops_sustained", 1700.0)
                tach = dft / (ms * 1e-3) / 1e12
                hbm_view = {k: out[st][k] for k in ("achieved", "peak", "unit", "frac", "per_step")}
                out[st] = {"bound": "tensor", "achieved": tach, "peak": tp, "unit": "TFLOP/s", "frac": tach / tp,
                           "per_step": dft, "ms_per_step": ms,
                           "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained" if "bf16_tflops_sustained"
                           in peaks else "fallback (sustained bf16)",
                           "bf16_issued_frac": 10 * tach / tp, "hbm_view": hbm_view,
                           "dft_pixels": dpix, "dft_pixels_frac": dpix / (12 * NSIDE ** 2)}
    return out


def fp64_gemm_peak(torch):
    """Measured FP64 GEMM throughput (cuBLAS DGEMM 8192^3, best of 5) in TFLOP/s."""
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2 * 8192 ** 3 / (best * 1e-3) / 1e12


PER_MODE_FLOOR = 1e-2        # per-mode relative errors over |a_fp64| >= this x max|a_fp64|
MAX_NORM_BAR = 1e-7


def error_report(a, ref, floor=PER_MODE_FLOOR):
    """Errors of the mixed a_nlm against the FP64 ones (complex vectors):
    L2 relative, global max-norm max|da| / max|a|, absolute max / rms, and the
    per-mode relative error |da_i| / |a_i| over the modes whose magnitude is at
    least `floor` times the largest (the relative error of near-zero modes is
    not meaningful)."""
    a = np.asarray(a)
    ref = np.asarray(ref)
    d = np.abs(a - ref)
    mag = np.abs(ref)
    amax = float(mag.max())
    sel = mag >= floor * amax
    rel = d[sel] / mag[sel]
    q = np.quantile(rel, [0.5, 0.99, 0.999]) if rel.size else [float("nan")] * 3
    mx = float(d.max() / amax)
    return {"l2": float(np.linalg.norm(a - ref) / np.linalg.norm(ref)), "max_norm": mx,
            "max_norm_bar": MAX_NORM_BAR, "max_norm_met": bool(mx <= MAX_NORM_BAR),
            "abs_max": float(d.max()), "abs_rms": float(np.sqrt(np.mean(d * d))), "max_abs_a": amax,
            "per_mode": {"floor_frac_of_max": floor, "modes": int(sel.sum()), "of": int(d.size),
                         "max": float(rel.max()) if rel.size else None, "median": float(q[0]),
                         "p99": float(q[1]), "p999": float(q[2])},
            "definitions": "l2 = ||da||_2/||a||_2; max_norm = max|da|/max|a|; per_mode = |da_i|/|a_i| over "
                           "|a_i| >= floor x max|a|"}


def aggregate_replicas(ms, ngal, world, device=None):
    """Replica runs (one independent catalogue per rank): the job's step time is
    the slowest rank's, and its throughput counts every rank's galaxies.
    Returns (ms_max, ngal_total, galaxies/s); collective over the initialised
    process group when world > 1 (NCCL on the GPUs, gloo in the CPU tests)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        n = torch.tensor([float(ngal)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(n, op=dist.ReduceOp.SUM)
        ms, ngal = float(t.item()), int(round(n.item()))
    return ms, ngal, ngal / (ms * 1e-3)


def batched_mocks_bench(nmocks, repeats, capi, torch, plan, mask, wln, veff, nlmsize):
    """Batched mocks: M independent seeded catalogues of the bench window, sizes uniform in [1e6, 2e7],
    concatenated in pinned host memory and transformed by one sfb_cat2amln_batched call (host buffers,
    the catalogue copies and result copies inside the timed call).  Prints one JSON line: galaxies/s over
    the timed calls, the per-mock time, and the largest relative difference between a mock's row and the
    single-catalogue call on the same mock (first and last mock).  Returns the record."""
    sizes = mock_sizes(nmocks)
    ntot = int(sizes.sum())
    h_gal = torch.empty((ntot, 3), dtype=torch.float64).pin_memory()
    h_w = torch.empty(ntot, dtype=torch.float64).pin_memory()
    t0 = time.perf_counter()
    off = fill_mocks(sizes, h_gal.numpy(), h_w.numpy())
    t_gen = time.perf_counter() - t0
    nbars = np.ascontiguousarray(sizes / veff, dtype=np.float64)
    h_mask = torch.from_numpy(mask).pin_memory()
    h_wln = torch.from_numpy(np.ascontiguousarray(wln.T)).pin_memory()
    out = torch.empty((len(sizes), 2 * nlmsize), dtype=torch.float64).pin_memory()
    hwin = capi.Window()
    hwin.kind = capi.SFB_WINDOW_SEPARABLE
    hwin.mask = capi.C.cast(h_mask.data_ptr(), capi._dp)
    hwin.w_ln = capi.C.cast(h_wln.data_ptr(), capi._dp)

    def call():
        capi.check(capi.lib.sfb_cat2amln_batched(plan.handle, capi.C.c_void_p(h_gal.data_ptr()),
                                                 capi.C.c_void_p(h_w.data_ptr()), capi.C.c_void_p(off.ctypes.data),
                                                 len(sizes), capi.C.c_void_p(nbars.ctypes.data),
                                                 capi.C.byref(hwin), capi.C.c_void_p(out.data_ptr())))

    call()
    torch.cuda.synchronize()
    ts = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        call()
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    res = out.numpy()
    diffs = []
    for k in (0, len(sizes) - 1):
        a, b = int(off[k]), int(off[k + 1])
        single = np.empty(2 * nlmsize)
        capi.check(capi.lib.sfb_cat2amln(plan.handle, capi.C.c_void_p(h_gal[a:b].data_ptr()),
                                         capi.C.c_void_p(h_w[a:b].data_ptr()), b - a, float(nbars[k]),
                                         capi.C.byref(hwin), capi.C.c_void_p(single.ctypes.data)))
        diffs.append(float(np.max(np.abs(res[k] - single)) / np.max(np.abs(single))))
    line = {"metric": "batched cat2amln galaxies/s (mixed)", "value": ntot / t, "unit": "galaxies/s",
            "higher_is_better": True, "mocks": int(len(sizes)), "galaxies": ntot,
            "sizes": {"min": int(sizes.min()), "max": int(sizes.max()), "mean": float(sizes.mean())},
            "s_per_batch": t, "ms_per_mock": t / len(sizes) * 1e3, "repeats": repeats,
            "timing": "host wall clock of one sfb_cat2amln_batched call (median of the repeats after one "
                      "warm-up): pinned host catalogues, their copies and the a_nlm copies inside",
            "h2d_bytes_per_batch": int(32 * ntot), "d2h_bytes_per_batch": int(16 * nlmsize * len(sizes)),
            "rows_vs_single_calls_max_rel_diff": max(diffs), "generation_s": t_gen,
            "config": {"workload": f"{len(sizes)} independent seeded mocks of the bench window (cap 60 x "
                                   "gauss(1500,400), w~U[0.5,1.5]), sizes uniform in [1e6, 2e7], kmax=0.1 "
                                   "nside=256, mixed precision", "data": "synthetic"}}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-fp64-leg", action="store_true", help="skip timing the FP64 path beside the mixed one")
    ap.add_argument("--ngal", type=int, default=0, help="override the catalogue size (testing)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c1", action="store_true", help="skip the C1 (nside 32) GPU timings")
    ap.add_argument("--cpu-workers", type=int, default=0)
    ap.add_argument("--cpu-pairs", type=int, default=0)
    ap.add_argument("--profile-case", action="store_true",
                    help="small case for ncu captures: same geometry, 2 radial pieces x degree 15 (34 maps), "
                         "1e6 galaxies, no e2e / CPU baseline")
    ap.add_argument("--batched-mocks", type=int, default=0,
                    help="time sfb_cat2amln_batched on this many seeded mocks of the bench window with sizes "
                         "uniform in [1e6, 2e7] (pinned host buffers), instead of the single-catalogue bench")
    ap.add_argument("--batched-repeats", type=int, default=4, help="timed batched calls (after one warm-up)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 8-mock batched extra of the default run")
    ap.add_argument("--full-basis", action="store_true",
                    help="with --profile-case: the bench's own radial basis (328 maps) with the profile case's "
                         "galaxy count, for per-kernel DRAM traffic captures")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    plan_extra = {}
    if args.profile_case:
        args.ngal = args.ngal or 1_000_000
        args.no_cpu_baseline = True
        args.no_c1 = True
        plan_extra = {} if args.full_basis else {"pieces": 2, "degree": 15}

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    global NGAL_MEAN
    if args.ngal:
        NGAL_MEAN = args.ngal

    import sfbgpu
    cores = os.cpu_count() or 1
    workers = args.cpu_workers or max(1, min(16, cores))

    if args.impl == "reference":
        if rank != 0:
            return
        amodes = sfbgpu.AnlmModes(KMAX, RMIN, RMAX, nside=NSIDE)
        gal, w = make_catalogue()
        wm, phi, mask = window_arrays(sfbgpu, amodes)
        from oracle import sfb as osfb
        md = dict(nmax=amodes.nmax, lmax=amodes.lmax, lmax_n=[int(v) for v in amodes.lmax_n], nside=NSIDE,
                  splines=amodes.basisfunctions.spline, noff=amodes._noff)
        _, wln = osfb.win_rhat_ln_separable(phi, mask, RMIN, RMAX, NR, md)
        veff = sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
        nbar = gal.shape[0] / veff
        ppst = args.cpu_pairs or workers
        vals, t_setup = run_reference_sample(amodes, gal, w, nbar, mask, wln, args.steps, args.warmup, workers, ppst)
        v = float(np.median(vals))
        line = {"metric": METRIC, "value": v, "unit": "galaxies/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": gal.shape[0] / v * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": WORKLOAD, "ngal": int(gal.shape[0]), "npairs": len(amodes.pairs()),
                           "l2": "inputs larger than L2 (CPU run)"},
                "cpu_baseline": {"value": v, "unit": "galaxies/s", "cores": workers, "kind": "port",
                                 "sample": f"{ppst} of {len(amodes.pairs())} (n,l) pairs per step (spline scatter "
                                           f"+ niter=3 map2alm each) on {workers} processes, extrapolated by pair "
                                           f"count, plus the once-per-call sort/ang2pix ({t_setup:.2f} s)",
                                 "c1_full": c1_cpu_full(sfbgpu, workers)},
                "e2e": {"value": v, "unit": "galaxies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    import torch.distributed as dist
    from sfbgpu import _capi as capi
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    amodes = sfbgpu.AnlmModes(KMAX, RMIN, RMAX, nside=NSIDE)
    plan = sfbgpu.get_plan(amodes, precision=args.precision, radial="poly", **plan_extra)
    info = plan.info()
    gal, w = make_catalogue(seed=2 + rank)
    N = gal.shape[0]
    wm, phi, mask = window_arrays(sfbgpu, amodes)
    winsep = sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, amodes,
                                precision=args.precision, radial="poly", **plan_extra)
    wln = np.asfortranarray(winsep.w_ln)
    veff = sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    nbar = N / veff
    nlmsize = plan.nlmsize

    dev = torch.device("cuda", local)
    d_gal = torch.from_numpy(gal).to(dev)
    d_w = torch.from_numpy(w).to(dev)
    d_mask = torch.from_numpy(mask).to(dev)
    d_wln = torch.from_numpy(np.ascontiguousarray(wln.T)).to(dev)    # element (l, n) at l + (lmax+1)(n-1)
    d_out = torch.empty(2 * nlmsize, dtype=torch.float64, device=dev)
    win = capi.Window()
    win.kind = capi.SFB_WINDOW_SEPARABLE
    win.mask = capi.C.cast(d_mask.data_ptr(), capi._dp)
    win.w_ln = capi.C.cast(d_wln.data_ptr(), capi._dp)
    stream = torch.cuda.current_stream(dev)
    if args.batched_mocks:
        if rank == 0:
            print(json.dumps(batched_mocks_bench(args.batched_mocks, args.batched_repeats, capi, torch, plan, mask,
                                                 wln, veff, nlmsize)), flush=True)
        return

    def step():
        capi.check(capi.lib.sfb_cat2amln_device(plan.handle, capi.C.c_void_p(d_gal.data_ptr()),
                                                capi.C.c_void_p(d_w.data_ptr()), N, float(nbar),
                                                capi.C.byref(win), capi.C.c_void_p(d_out.data_ptr()),
                                                capi.C.c_void_p(stream.cuda_stream)))

    for _ in range(args.warmup):
        step()
    capi.check(capi.lib.sfb_set_profiling(plan.handle, 1))
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = capi.lib.sfb_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    launches = capi.lib.sfb_launch_count() - l0
    ms, n_job, value = aggregate_replicas(e0.elapsed_time(e1) / args.steps, N, world, dev)
    stage_ms = (capi.C.c_double * 7)()
    stage_n = (capi.C.c_int64 * 7)()
    capi.check(capi.lib.sfb_get_stage_times(plan.handle, stage_ms, stage_n))
    capi.check(capi.lib.sfb_set_profiling(plan.handle, 0))
    stages = {nm: {"ms_per_step": stage_ms[i] / args.steps, "launches_per_step": stage_n[i] / args.steps}
              for i, nm in enumerate(capi.STAGES)}

    if args.profile_case:
        if rank == 0:
            print(json.dumps({"profile_case": True, "ms_per_step": ms, "stages": stages}), flush=True)
        return
    # end to end: host-pointer C-ABI call from pinned memory
    h_gal = torch.from_numpy(gal).pin_memory()
    h_w = torch.from_numpy(w).pin_memory()
    h_mask = torch.from_numpy(mask).pin_memory()
    h_wln = torch.from_numpy(np.ascontiguousarray(wln.T)).pin_memory()
    h_out = torch.empty(2 * nlmsize, dtype=torch.float64).pin_memory()
    hwin = capi.Window()
    hwin.kind = capi.SFB_WINDOW_SEPARABLE
    hwin.mask = capi.C.cast(h_mask.data_ptr(), capi._dp)
    hwin.w_ln = capi.C.cast(h_wln.data_ptr(), capi._dp)

    def host_step():
        capi.check(capi.lib.sfb_cat2amln(plan.handle, capi.C.c_void_p(h_gal.data_ptr()),
                                         capi.C.c_void_p(h_w.data_ptr()), N, float(nbar), capi.C.byref(hwin),
                                         capi.C.c_void_p(h_out.data_ptr())))

    host_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    _, _, e2e_value = aggregate_replicas(e2e_s * 1e3, N, world, dev)
    h2d = 8 * (3 * N + N + mask.size + wln.size)
    d2h = 16 * nlmsize
    res_dev = d_out.cpu().numpy()
    same = float(np.max(np.abs(h_out.numpy() - res_dev)) / max(np.max(np.abs(res_dev)), 1e-300))

    # the metric compares the mixed path with the FP64 GPU path on the same catalogue
    vs64 = None
    if args.precision == "mixed" and not args.no_fp64_leg:
        wln64 = np.asfortranarray(sfbgpu.win_rhat_ln(sfbgpu.SeparableArray(phi, mask, "phi", "mask"), wm, amodes,
                                                     precision="fp64", radial="poly", **plan_extra).w_ln)
        d_wln64 = torch.from_numpy(np.ascontiguousarray(wln64.T)).to(dev)
        win64 = capi.Window()
        win64.kind = capi.SFB_WINDOW_SEPARABLE
        win64.mask = capi.C.cast(d_mask.data_ptr(), capi._dp)
        win64.w_ln = capi.C.cast(d_wln64.data_ptr(), capi._dp)

        def time_fp64(plan64, d_res, steps):
            def step64():
                capi.check(capi.lib.sfb_cat2amln_device(plan64.handle, capi.C.c_void_p(d_gal.data_ptr()),
                                                        capi.C.c_void_p(d_w.data_ptr()), N, float(nbar),
                                                        capi.C.byref(win64), capi.C.c_void_p(d_res.data_ptr()),
                                                        capi.C.c_void_p(stream.cuda_stream)))
            for _ in range(args.warmup):
                step64()
            torch.cuda.synchronize()
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            for _ in range(steps):
                step64()
            f1.record(stream)
            torch.cuda.synchronize()
            return aggregate_replicas(f0.elapsed_time(f1) / steps, N, world, dev)

        # (1) the same algorithm as the mixed path (Gram refinement, first pass over the rings with data)
        plan64 = sfbgpu.get_plan(amodes, precision="fp64", radial="poly", **plan_extra)
        d_out64 = torch.empty_like(d_out)
        ms64, _, value64 = time_fp64(plan64, d_out64, args.steps)
        # (2) the FP64 path with full synthesis / fold / analysis refinement passes over every ring
        os.environ["SFBGPU_GRAM_REFINEMENT"] = "0"
        try:
            plan64f = sfbgpu.GPUPlan(amodes, precision="fp64", radial="poly", **plan_extra)
        finally:
            os.environ.pop("SFBGPU_GRAM_REFINEMENT", None)
        d_out64f = torch.empty_like(d_out)
        ms64f, _, value64f = time_fp64(plan64f, d_out64f, min(args.steps, 5))
        plan64f.close()
        step()
        torch.cuda.synchronize()
        a_mix, a_64, a_64f = (x.cpu().numpy().view(np.complex128) for x in (d_out, d_out64, d_out64f))
        vs64 = {"fp64_value": value64, "fp64_ms_per_step": ms64, "speedup": ms64 / ms,
                "fp64_algorithm": "same as the mixed path: Gram refinement of the alias-free rings, first "
                                  "analysis pass over the ring pairs with data",
                "errors": error_report(a_mix, a_64),
                "rel_err": float(np.linalg.norm(a_mix - a_64) / np.linalg.norm(a_64)),
                "rel_err_definition": "||a_mixed - a_fp64||_2 / ||a_fp64||_2 over the a_nlm vector",
                "fp64_full_passes": {"value": value64f, "ms_per_step": ms64f, "speedup": ms64f / ms,
                                     "steps": min(args.steps, 5),
                                     "algorithm": "FP64 with full synthesis / fold / analysis refinement "
                                                  "passes over all rings (no Gram refinement, no ring span)",
                                     "rel_diff_vs_fp64": float(np.linalg.norm(a_64f - a_64) /
                                                               np.linalg.norm(a_64))}}

    # roofline of every stage; the headline is the dominant one
    nm = info["nbasis"] + 1
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    fp64_peak = fp64_gemm_peak(torch) if args.precision == "fp64" else None
    sky = sky_rings(sfbgpu, NSIDE, gal[:, 1], gal[:, 2]) if args.precision == "mixed" else None
    table = roofline_table(stages, args.precision, nm, N, info["nbasis"], peaks, fp64_peak, sky)
    if args.precision == "mixed":
        for k in table:
            traffic, parts = stage_traffic(k, {"maps": nm, "galaxies": N})
            table[k]["traffic"] = traffic
            if traffic is not None:
                table[k]["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per call, one kernel "
                                              "per capture, on the profile cases (transforms: the bench basis with "
                                              "1e6 galaxies; deposit: 35 maps with 1e7 galaxies), scaled to this run "
                                              "by maps or galaxies: " + ", ".join(parts))
    dom = max(table, key=lambda k: stages[k]["ms_per_step"])
    roof = dict(table[dom])
    roof["kernel_stage"] = dom
    roof.setdefault("traffic", None)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import sfb as osfb
        md = dict(nmax=amodes.nmax, lmax=amodes.lmax, lmax_n=[int(v) for v in amodes.lmax_n], nside=NSIDE,
                  splines=amodes.basisfunctions.spline, noff=amodes._noff)
        ppst = args.cpu_pairs or workers
        vals, t_setup = run_reference_sample(amodes, gal, w, nbar, mask, wln, 1, 0, workers, ppst)
        cpu = {"value": float(vals[0]), "unit": "galaxies/s", "cores": workers, "kind": "port",
               "sample": f"{ppst} of {len(amodes.pairs())} (n,l) pairs (spline scatter + niter=3 map2alm each) on "
                         f"{workers} processes, extrapolated by pair count, plus the once-per-call sort/ang2pix "
                         f"({t_setup:.2f} s)",
               "c1_full": c1_cpu_full(sfbgpu, workers)}
    c1 = c1_gpu(sfbgpu) if (rank == 0 and world == 1 and not args.no_c1) else None
    # batched mocks beside the single-catalogue numbers: 8 uneven mocks (~8e7 galaxies) through
    # sfb_cat2amln_batched; a failure here is reported in the record, not raised
    batched = None
    if rank == 0 and world == 1 and args.precision == "mixed" and not args.no_batched:
        try:
            batched = batched_mocks_bench(8, 2, capi, torch, plan, mask, wln, veff, nlmsize)
            batched.pop("metric", None)
            batched.pop("higher_is_better", None)
        except Exception as exc:          # noqa: BLE001 - recorded, the headline stands without it
            batched = {"error": f"{type(exc).__name__}: {exc}"[:300]}
    if c1 and cpu:
        c1["mixed"]["vs_cpu_c1_full"] = c1["mixed"]["value"] / cpu["c1_full"]["value"]

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "galaxies/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "mixed",
                "data": "synthetic",
                "config": {"workload": WORKLOAD, "ngal": N, "precision": args.precision, "radial": "poly",
                           "radial_pieces": info["radial_pieces"], "radial_degree": info["radial_degree"],
                           "radial_error": info["radial_error"], "nbasis": info["nbasis"],
                           "l2": "inputs (320 MB) and maps larger than L2; no flush",
                           "parallelism": "replicas" if world > 1 else "single"},
                "roofline": roof, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": "galaxies/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h), "host_vs_device_result_rel_diff": same},
                "mixed_vs_fp64": vs64, "c1": c1, "batched_mocks": batched,
                "stages": stages, "stage_roofline": table, "clocks": clk, "gpu_launches": int(launches)}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
