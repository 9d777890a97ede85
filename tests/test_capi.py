"""The C ABI library: loads, exports every declared symbol, struct layouts
match the header, argument checks and the no-device failure (CPU only)."""

import os
import re
import subprocess
import tempfile

import ctypes as C
import numpy as np
import pytest

from sfbgpu import _capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sfb_gpu.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|int64_t)\s+\*?(sfb_\w+)\s*\(", txt, re.M)))


def test_every_declared_symbol_is_exported():
    names = declared()
    assert len(names) >= 12
    for n in names:
        assert hasattr(capi.lib, n), n
    assert set(names) <= {p[0] for p in capi._PROTOS}


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(f'''#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
#define P(s, f) printf("%s.%s %zu\\n", #s, #f, offsetof(s, f));
int main(void) {{
  printf("sfb_plan_desc %zu\\nsfb_window %zu\\nsfb_plan_info %zu\\n", sizeof(sfb_plan_desc), sizeof(sfb_window), sizeof(sfb_plan_info));
  P(sfb_plan_desc, spl_offset) P(sfb_plan_desc, niter) P(sfb_plan_desc, radial_tol)
  P(sfb_window, mask) P(sfb_window, dense) P(sfb_plan_info, radial_error) P(sfb_plan_info, device_bytes)
  return 0; }}''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n") if l)
    assert int(out["sfb_plan_desc"]) == C.sizeof(capi.PlanDesc)
    assert int(out["sfb_window"]) == C.sizeof(capi.Window)
    assert int(out["sfb_plan_info"]) == C.sizeof(capi.PlanInfo)
    assert int(out["sfb_plan_desc.radial_tol"]) == capi.PlanDesc.radial_tol.offset
    assert int(out["sfb_plan_desc.niter"]) == capi.PlanDesc.niter.offset
    assert int(out["sfb_window.dense"]) == capi.Window.dense.offset
    assert int(out["sfb_plan_info.device_bytes"]) == capi.PlanInfo.device_bytes.offset


def _desc(nside=4, lmax=3):
    lmax_n = np.array([lmax], np.int64)
    x = np.linspace(500, 1000, 20)
    xs = np.concatenate([x] * (lmax + 1))
    off = np.arange(lmax + 2, dtype=np.int64) * 20
    keep = [lmax_n, xs, off]
    d = capi.PlanDesc(nside=nside, lmax=lmax, nmax=1, lmax_n=lmax_n.ctypes.data_as(capi._i64p), rmin=500.0,
                      rmax=1000.0, spl_offset=off.ctypes.data_as(capi._i64p), spl_x=xs.ctypes.data_as(capi._dp),
                      spl_y=xs.ctypes.data_as(capi._dp), spl_ypp=xs.ctypes.data_as(capi._dp), niter=3)
    return d, keep


def test_argument_checks_before_device():
    h = C.c_void_p()
    assert capi.lib.sfb_plan_create(None, C.byref(h)) == capi.SFB_EINVAL
    d, keep = _desc(nside=4, lmax=17)          # lmax > 4*nside (src/healpix_helpers.jl:51-54)
    assert capi.lib.sfb_plan_create(C.byref(d), C.byref(h)) == capi.SFB_ERANGE
    assert "4*nside" in capi.last_error()
    d, keep = _desc()
    d.rmin = 2000.0
    assert capi.lib.sfb_plan_create(C.byref(d), C.byref(h)) == capi.SFB_EINVAL
    d, keep = _desc()
    d.precision = 9
    assert capi.lib.sfb_plan_create(C.byref(d), C.byref(h)) == capi.SFB_EINVAL
    assert capi.lib.sfb_cat2amln(None, None, None, 0, 1.0, None, None) == capi.SFB_EINVAL
    assert capi.lib.sfb_ang2pix_ring(0, None, None, 1, None) == capi.SFB_EINVAL


def test_no_device_fails_loudly_or_plan_works():
    d, keep = _desc()
    h = C.c_void_p()
    st = capi.lib.sfb_plan_create(C.byref(d), C.byref(h))
    if st == capi.SFB_OK:          # a GPU is present
        capi.lib.sfb_plan_destroy(h)
    else:
        assert st == capi.SFB_ECUDA
        assert "CUDA" in capi.last_error()


def test_last_error_truncates():
    capi.lib.sfb_plan_create(None, None)
    buf = C.create_string_buffer(8)
    assert capi.lib.sfb_last_error(buf, 8) == capi.SFB_OK
    assert len(buf.value) <= 7
