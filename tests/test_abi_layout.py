"""The C structs of the boundary (include/nmgpu.h, include/nmmodel.h) against
their mirrors: the ctypes structures of the Python bindings and the bind(C)
derived types of include/nmgpu_mod.f90.  A C program compiled here prints
every field's offset and size; the ctypes layout must match it, and the
Fortran types, laid out by the C rules that bind(C) follows, must list the
same fields in the same order at the same offsets."""
import os
import re
import subprocess

import pytest

from normalmodes_gb300 import model as M
from normalmodes_gb300 import nmgpu as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")

STRUCTS = {
    "nm_csr": G.NmCsr, "nm_opts": G.NmOpts, "nm_solve_opts": G.NmSolveOpts, "nm_result": G.NmResult,
    "nm_elem_model": G.NmElemModel, "nm_slice": G.NmSlice, "nm_csr_fill": G.NmCsrFill, "nm_kpm_opts": G.NmKpmOpts, "nm_info": G.NmInfo,
    "nmm_ball_opts": M.BallOpts, "nmm_info_t": M.Info,
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    d = tmp_path_factory.mktemp("abi")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "nmgpu.h"', '#include "nmmodel.h"',
             "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} . %zu %zu\\n", (size_t)0, sizeof({cname}));')
        for f in py._fields_:
            name = f[0]
            lines.append(f'  printf("{cname} {name} %zu %zu\\n", offsetof({cname}, {name}), '
                         f"sizeof((({cname}*)0)->{name}));")
    lines += ["  return 0;", "}"]
    src = d / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "abi"
    subprocess.run(["gcc", "-std=c11", "-I", INC, str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    lay = {}
    for ln in out.splitlines():
        s, f, off, size = ln.split()
        lay.setdefault(s, {})[f] = (int(off), int(size))
    return lay


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_ctypes_mirrors_match_c(c_layout, cname):
    py = STRUCTS[cname]
    import ctypes
    assert ctypes.sizeof(py) == c_layout[cname]["."][1], cname
    for f in py._fields_:
        desc = getattr(py, f[0])
        assert (desc.offset, desc.size) == c_layout[cname][f[0]], (cname, f[0])
    # every C member is mirrored (sizes add up with the padding the offsets imply)
    assert len(py._fields_) == len(c_layout[cname]) - 1


_FKIND = {"integer(c_int)": (4, 4), "real(c_double)": (8, 8), "integer(c_long_long)": (8, 8),
          "type(c_ptr)": (8, 8), "type(c_funptr)": (8, 8), "integer(c_size_t)": (8, 8)}


def _fortran_types():
    text = open(os.path.join(INC, "nmgpu_mod.f90")).read()
    out = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", text, re.S):
        fields = []
        for ln in m.group(2).splitlines():
            ln = ln.split("!")[0].strip()
            if not ln:
                continue
            kind, names = [x.strip() for x in ln.split("::")]
            for nm in re.findall(r"(\w+)(?:\((\d+)\))?", names):
                fields.append((nm[0], kind, int(nm[1]) if nm[1] else 1))
        out[m.group(1)] = fields
    return out


def test_fortran_module_matches_c(c_layout):
    ftypes = _fortran_types()
    assert {"nm_csr", "nm_opts", "nm_solve_opts", "nm_result", "nm_slice", "nm_kpm_opts"} <= set(ftypes)
    for tname, fields in ftypes.items():
        c = c_layout[tname]
        off = 0
        align_max = 1
        for name, kind, count in fields:
            size, align = _FKIND[kind.lower()]
            off = (off + align - 1) // align * align
            assert name in c, (tname, name)
            assert c[name] == (off, size * count), (tname, name, c[name], (off, size * count))
            off += size * count
            align_max = max(align_max, align)
        total = (off + align_max - 1) // align_max * align_max
        assert total == c["."][1], tname
        assert len(fields) == len(c) - 1, tname
