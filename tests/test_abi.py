"""The C ABI library loads and exports every symbol include/pencilfft_gb300.h
declares (no compute call; CPU only)."""
import ctypes
import os
import re

import pencilffts_gb300 as P
from pencilffts_gb300 import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(REPO, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(REPO, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(pfgb_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_symbols_exported():
    L = P.load_library()
    names = declared_symbols()
    assert "pfgb_forward" in names and "pfgb_plan_create" in names
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/ but not exported"
    # the ctypes table covers every declared entry point
    assert names <= set(_lib.SIGNATURES), names - set(_lib.SIGNATURES)


def test_struct_layouts_match_header():
    # pfgb_plan_desc: int32 + 8 int64 + 4*8 int32 + 3 int32 + 4 int64 + 2 int32
    assert ctypes.sizeof(_lib.PlanDesc) == 4 + 4 + 64 + 4 * 32 + 12 + 4 + 32 + 8
    assert ctypes.alignment(_lib.PlanDesc) == 8


def test_version_and_error_buffer():
    L = P.load_library()
    assert b"sm_103a" in L.pfgb_version()
    buf = ctypes.create_string_buffer(8)
    L.pfgb_last_error(buf, len(buf))  # callable without a device


def test_null_arguments_rejected_without_device():
    L = P.load_library()
    assert L.pfgb_plan_create(None, None) == _lib.ERR_ARGUMENT
    assert L.pfgb_forward(None, None, None, None) == _lib.ERR_ARGUMENT
    assert L.pfgb_plan_destroy(None) == _lib.OK


def _julia_struct(name):
    """Fields (name, ctypes type) of an isbits struct of the Julia binding."""
    src = open(os.path.join(REPO, "pencilffts.jl_gb300", "julia", "PencilFFTsGB300.jl")).read()
    m = re.search(r"^struct %s\n(.*?)^end" % name, src, flags=re.S | re.M)
    assert m, name
    scalar = {"Int32": ctypes.c_int32, "Int64": ctypes.c_int64, "Float64": ctypes.c_double,
              "Ptr{Cvoid}": ctypes.c_void_p}
    consts = {"MAX_DIMS": _lib.MAX_DIMS, "MAX_EXTRA": 4}
    out = []
    for line in m.group(1).strip().splitlines():
        fname, ftype = [t.strip() for t in line.split("::")]
        t = re.fullmatch(r"NTuple\{(\w+),(\w+)\}", ftype)
        out.append((fname, scalar[t.group(2)] * consts[t.group(1)] if t else scalar[ftype]))
    return out


def test_julia_structs_mirror_the_header():
    """The Julia binding's PlanDesc, PlanInfo and BatchOp have the C structs' fields, in
    order and with the same types (Julia lays isbits structs out with C
    alignment), so ccall passes them by reference unchanged."""
    for jname, cstruct in (("PlanDesc", _lib.PlanDesc), ("PlanInfo", _lib.PlanInfo), ("BatchOp", _lib.BatchOp)):
        jf = _julia_struct(jname)
        cf = cstruct._fields_
        assert [n for n, _ in jf] == [n for n, _ in cf], jname
        for (n, jt), (_, ct) in zip(jf, cf):
            assert ctypes.sizeof(jt) == ctypes.sizeof(ct) and getattr(jt, "_type_", jt) == getattr(ct, "_type_", ct), (jname, n)
    # offsets the binding relies on, e.g. scale_factor of pfgb_plan_info
    assert _lib.PlanInfo.scale_factor.offset == 184


def test_struct_offsets_match_a_c_compiler(tmp_path):
    """Every struct of the header, compiled by the host C compiler: size and
    field offsets equal those of the ctypes mirrors."""
    import shutil
    import subprocess
    import pytest
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"pfgb_plan_desc": _lib.PlanDesc, "pfgb_plan_info": _lib.PlanInfo,
               "pfgb_pass_timing": _lib.PassTiming, "pfgb_batch_op": _lib.BatchOp,
               "pfgb_batch_info": _lib.BatchInfo}
    lines = ['#include <stdio.h>', '#include "pencilfft_gb300.h"', "int main(void) {"]
    for cname, ct in mirrors.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in ct._fields_:  # (a trailing underscore avoids a Python keyword)
            lines.append(f'  printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0].rstrip("_")}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for cname, ct in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(ct), cname
        for f in ct._fields_:
            assert got[(cname, f[0])] == getattr(ct, f[0]).offset, (cname, f[0])
