"""The Fortran iso_c_binding shim printed in INTEGRATION.md against the C header.

No Fortran compiler exists here, so the shim itself is never compiled.  These tests read its
source out of INTEGRATION.md and check what a compiler would otherwise catch only at run
time:
- every `type, bind(C)` derived type has the components of the C struct of the same name in
  include/msmgb.h, in the same order, with interoperable kinds, and the offsets and size the
  Fortran declaration order implies (the C layout rules a bind(C) type follows: natural
  alignment of c_int 4, c_double 8, c_ptr 8, arrays of their element) equal offsetof/sizeof
  of the real header compiled by gcc;
- every interface body names a function the header declares, with the same number of
  arguments, and passes by value exactly the arguments the C prototype takes by value
  (pointers otherwise).
"""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "msmgb.h")
DOC = os.path.join(ROOT, "INTEGRATION.md")

KINDS = {"integer(c_int)": ("int", 4), "real(c_double)": ("double", 8), "type(c_ptr)": ("ptr", 8)}


def fortran_source():
    text = open(DOC).read()
    m = re.search(r"```fortran\n(.*?)```", text, re.S)
    assert m, "no fortran block in INTEGRATION.md"
    # join continuation lines
    return re.sub(r"&\s*\n\s*", " ", m.group(1))


def fortran_types(src):
    """{type name: [(component, kind, count)]} in declaration order."""
    out = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", src, re.S):
        comps = []
        for line in m.group(2).splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, names = (s.strip() for s in line.split("::"))
            assert kind in KINDS, kind
            for nm in re.findall(r"\w+(?:\(\d+\))?", names):
                cnt = int(re.search(r"\((\d+)\)", nm).group(1)) if "(" in nm else 1
                comps.append((nm.split("(")[0], KINDS[kind][0], cnt))
        out[m.group(1)] = comps
    return out


def c_layout_of(comps):
    """Offsets and size of a bind(C) type under the C rules (LP64)."""
    off, offs, align = 0, [], 1
    for _, kind, cnt in comps:
        sz = 4 if kind == "int" else 8
        off = (off + sz - 1) // sz * sz
        offs.append(off)
        off += sz * cnt
        align = max(align, sz)
    return offs, (off + align - 1) // align * align


def c_struct_fields(name):
    """(field, kind, count) of `typedef struct { ... } name;` in the header, in order."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r";", text)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "const double *potr, *fpotr" / "double lo[3]" / "int n"
        base = re.match(r"^(?:const\s+)?(?:unsigned\s+)?(\w+)", decl).group(1)
        body = re.sub(r"^(const\s+)?(unsigned\s+)?\w+\s*", "", decl)
        for part in body.split(","):
            cnt = re.search(r"\[(\d+)\]", part)
            kind = "ptr" if "*" in part else {"int": "int", "double": "double"}[base]
            fields.append((re.sub(r"[\s*]|\[\d+\]", "", part), kind, int(cnt.group(1)) if cnt else 1))
    return fields


def c_prototypes():
    """{function: [(is_pointer, text)]} of the header's entry points."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:int|void|int64_t|const char)\s*\*?\s*(msmgb_\w+)\s*\(([^)]*)\)\s*;", text):
        args = [a.strip() for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(1)] = [("*" in a or "[" in a, a) for a in args]
    return out


def fortran_interfaces(src):
    """{bound C name: [(dummy, by_value)]}"""
    out = {}
    for m in re.finditer(r"function (\w+)\(([^)]*)\)\s*bind\(C, name=\"(\w+)\"\)(.*?)end function", src, re.S):
        dummies = [d.strip() for d in m.group(2).split(",") if d.strip()]
        body = m.group(4)
        byval = set()
        for decl in re.split(r";|\n", body):
            if "::" not in decl:
                continue
            attrs, names = decl.split("::", 1)
            if "value" in attrs:
                byval.update(re.findall(r"\w+", re.sub(r"\(.*?\)", "", names.split("!")[0])))
        out[m.group(3)] = [(d, d in byval) for d in dummies]
    return out


@pytest.fixture(scope="module")
def c_offsets():
    """offsetof / sizeof of every struct the Fortran block declares, from the real header."""
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    types = fortran_types(fortran_source())
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "msmgb.h"', "int main(void) {"]
    for t, comps in types.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (t, t))
        for nm, _, _ in comps:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (t, nm, t, nm))
    lines += ["return 0; }"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "lay.c"), os.path.join(d, "lay")
        open(src, "w").write("\n".join(lines))
        subprocess.run([gcc, "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True,
                       capture_output=True)
        outp = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in outp.splitlines():
        t, f, v = line.split()
        res[(t, f)] = int(v)
    return res


def test_bind_c_types_match_header_layout(c_offsets):
    types = fortran_types(fortran_source())
    assert set(types) == {"msmgb_params", "msmgb_forcetable", "msmgb_box"}
    for t, comps in types.items():
        assert comps == c_struct_fields(t), t      # names, kinds and array lengths
        offs, size = c_layout_of(comps)
        for (nm, _, _), off in zip(comps, offs):
            assert c_offsets[(t, nm)] == off, (t, nm, c_offsets[(t, nm)], off)
        assert c_offsets[(t, "size")] == size, (t, size)


def test_interfaces_match_prototypes():
    protos = c_prototypes()
    ifaces = fortran_interfaces(fortran_source())
    assert len(ifaces) >= 15
    for name, dummies in ifaces.items():
        assert name in protos, name
        cargs = protos[name]
        assert len(dummies) == len(cargs), (name, dummies, cargs)
        for (d, byval), (isptr, ctext) in zip(dummies, cargs):
            # a c_ptr passed by value is a C pointer (the context handle)
            if byval and ctext.startswith("msmgb_ctx"):
                continue
            assert byval == (not isptr), (name, d, ctext)
