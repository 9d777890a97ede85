"""The benchmark configurations against the oracle's reference algorithm
(src/cat2anlm.jl:257-310 restated in oracle/sfb.py).

C1 (the reference's CPU-runnable case: kmax 0.05, r in [500, 1000], nside 32,
nr 250, 2e5 galaxies r ~ r^2 on the full sky, unit weights, n = N/V, full-sky
constant window), every coefficient:
* FP64 spline mode vs oracle: 1e-11 (the same algorithm in FP64);
* FP64 piecewise-Legendre radial basis vs oracle: 2e-7 (the basis replaces the
  per-galaxy cubic spline; its projection error is near the spline's own);
* mixed vs FP64 (same radial basis): 1e-7, L2 and max-norm (the precision bar
  of the mixed path), with per-mode errors recorded (config 3);
* mixed vs oracle: 2e-7.
All errors are max|x - ref| / max|ref| unless stated.

C2 geometry (kmax 0.1, r in [500, 2500], nside 256, lmax 238, 7,520 (n,l)
pairs) on a 1e6-galaxy draw of the benchmark window: the GPU FP64 path with
its 13 x 24 radial basis against the oracle on 32 (n,l) pairs spread over the
pair list, 2e-7 (relative to the largest coefficient of those pairs).
"""

import importlib.util
import os

import numpy as np
import pytest

import sfbgpu
from helpers import modes_dict, record, rel_err
from oracle import sfb as osfb

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_cfg", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def bench():
    return _bench()


@pytest.fixture(scope="module")
def c1(bench):
    amodes, gal, w, wm, phi, mask, nbar = bench.c1_setup(sfbgpu)
    md = modes_dict(amodes)
    C = bench.C1
    _, wln = osfb.win_rhat_ln_separable(phi, mask, C["rmin"], C["rmax"], C["nr"], md)
    rtp = gal.T
    ref = osfb.cat2amln(rtp, md, nbar, ("separable", mask, wln), None)
    win = sfbgpu.SeparableArray(mask, wln, "mask", "w_ln")
    return amodes, rtp, nbar, win, ref


def _per_mode(x, ref, floor=1e-2):
    d, mag = np.abs(x - ref), np.abs(ref)
    sel = mag >= floor * mag.max()
    rel = d[sel] / mag[sel]
    return {"per_mode_floor": floor, "per_mode_max": float(rel.max()), "per_mode_p999": float(np.quantile(rel, 0.999)),
            "abs_max": float(d.max()), "abs_rms": float(np.sqrt(np.mean(d * d)))}


def test_c1_fp64_vs_reference_algorithm(c1):
    amodes, rtp, nbar, win, ref = c1
    spl = sfbgpu.cat2amln(rtp, amodes, nbar, win, None, precision="fp64", radial="spline")
    e_s = rel_err(spl, ref)
    poly = sfbgpu.cat2amln(rtp, amodes, nbar, win, None, precision="fp64", radial="poly")
    e_p = rel_err(poly, ref)
    record("c1_fp64_spline_vs_oracle", e_s)
    record("c1_fp64_poly_vs_oracle", e_p, **_per_mode(poly, ref))
    assert e_s < 1e-11
    assert e_p < 2e-7


def test_c1_mixed_per_mode(c1):
    """Config 3: the mixed path on the C1 catalogue, global and per-mode errors
    against the FP64 path of the same radial basis and against the oracle."""
    amodes, rtp, nbar, win, ref = c1
    f64 = sfbgpu.cat2amln(rtp, amodes, nbar, win, None, precision="fp64", radial="poly")
    mix = sfbgpu.cat2amln(rtp, amodes, nbar, win, None, precision="mixed", radial="poly")
    e2 = float(np.linalg.norm(mix - f64) / np.linalg.norm(f64))
    emax = rel_err(mix, f64)
    e_ref = rel_err(mix, ref)
    record("c1_mixed_vs_fp64", e2, maxnorm=emax, **_per_mode(mix, f64))
    record("c1_mixed_vs_oracle", e_ref, **_per_mode(mix, ref))
    assert e2 < 1e-7 and emax < 1e-7
    assert e_ref < 2e-7


def test_c2_pair_subset_vs_reference_algorithm(bench):
    """The C2 radial basis (13 pieces x degree 24) end to end against the
    per-galaxy spline algorithm, on 32 (n,l) pairs spread over the pair list."""
    amodes = sfbgpu.AnlmModes(bench.KMAX, bench.RMIN, bench.RMAX, nside=bench.NSIDE)
    bench.NGAL_MEAN = 1_000_000
    gal, w = bench.make_catalogue(seed=5)
    wm, phi, mask = bench.window_arrays(sfbgpu, amodes)
    md = modes_dict(amodes)
    _, wln = osfb.win_rhat_ln_separable(phi, mask, bench.RMIN, bench.RMAX, bench.NR, md)
    nbar = gal.shape[0] / sfbgpu.integrate_window(sfbgpu.SeparableArray(phi, mask), wm)
    rtp = gal.T
    pairs = amodes.pairs()
    sub = [pairs[i] for i in np.linspace(0, len(pairs) - 1, 32).astype(int)]
    ref = osfb.cat2amln(rtp, md, nbar, ("separable", mask, wln), w, pair_subset=sub)
    win = sfbgpu.SeparableArray(mask, wln, "mask", "w_ln")
    gpu = sfbgpu.cat2amln(rtp, amodes, nbar, win, w, precision="fp64", radial="poly")
    idx = np.concatenate([md["noff"][n - 1] + l * (l + 1) // 2 + np.arange(l + 1) for n, l in sub])
    e = rel_err(gpu[idx], ref[idx])
    info = sfbgpu.get_plan(amodes, precision="fp64", radial="poly").info()
    record("c2_pair_subset_fp64_poly_vs_oracle", e, pairs=len(sub), coefficients=int(idx.size),
           radial_error=info["radial_error"])
    assert e < 2e-7
