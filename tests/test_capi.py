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


def _julia_ccalls():
    """(symbol, return type, argument types) of every ccall in the Julia binding."""
    src = open(os.path.join(ROOT, "sphericalfourierbesseldecompositions.jl_gb300", "julia", "SFBGPU.jl")).read()
    out = []
    for m in re.finditer(r"ccall\(\(:(\w+),\s*libsfb\),\s*(\w+),\s*\(", src):
        i, depth, args, cur = m.end(), 1, [], ""
        while depth:
            ch = src[i]
            if ch in "({":
                depth += 1
            elif ch in ")}":
                depth -= 1
            if depth == 1 and ch == ",":
                args.append(cur.strip())
                cur = ""
            elif depth:
                cur += ch
            i += 1
        if cur.strip():
            args.append(cur.strip())
        out.append((m.group(1), m.group(2), args))
    return out


def _header_params():
    """Parameter lists of the header's functions, each parameter classified as 'ptr' or its C type."""
    hdr = open(os.path.join(ROOT, "include", "sfb_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    hdr = re.sub(r"//[^\n]*", "", hdr)
    decls = {}
    for m in re.finditer(r"\b(int|void|int64_t)\s+(sfb_\w+)\s*\(([^)]*)\)\s*;", hdr):
        params = [p.strip() for p in m.group(3).split(",") if p.strip() and p.strip() != "void"]
        kinds = []
        for p in params:
            if "*" in p:
                kinds.append("ptr")
            else:
                kinds.append(" ".join(p.replace("const ", "").split()[:-1]))
        decls[m.group(2)] = (m.group(1), kinds)
    return decls


JULIA_TO_C = {"Int64": "int64_t", "Float64": "double", "Int32": "int32_t", "Cint": "int", "UInt64": "uint64_t",
              "Csize_t": "size_t"}


def test_julia_binding_matches_header():
    """Every ccall of the Julia binding names a function the header declares, with as many arguments, each
    of the matching kind (pointers as Ptr/Ref, integers and doubles by width), and the same return type."""
    decls = _header_params()
    calls = _julia_ccalls()
    assert len(calls) >= 14
    for name, ret, args in calls:
        assert name in decls, name
        cret, kinds = decls[name]
        assert {"Cint": "int", "Cvoid": "void", "Int64": "int64_t"}[ret] == cret, name
        assert len(args) == len(kinds), (name, args, kinds)
        for a, k in zip(args, kinds):
            jk = "ptr" if a.startswith(("Ptr{", "Ref{")) else JULIA_TO_C[a]
            assert jk == k, (name, a, k)
