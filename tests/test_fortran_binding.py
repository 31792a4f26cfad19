"""The Fortran binding a maintainer adds to the reference (fortran/omx_gpu_mod.f90) against the
C-ABI it binds (include/omx_gpu.h), without a Fortran compiler: every bind(C) derived type has
the size and field offsets of its C struct (measured by a gcc-compiled probe of the header), and
every bound function exists in the header with the same number and kinds of arguments."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "omx_gpu.h")
FMOD = os.path.join(ROOT, "one-mxll-to-rule-them-all_gb300", "fortran", "omx_gpu_mod.f90")
FTYPE = os.path.join(ROOT, "one-mxll-to-rule-them-all_gb300", "fortran", "mxll_3D_gpu_mod.f90")

# C size of the iso_c_binding kinds used in the module
KIND_SIZE = {"integer(c_int)": 4, "real(c_double)": 8, "character(kind=c_char)": 1, "integer(c_int32_t)": 4,
             "integer(c_long_long)": 8}


def _strip(src):
    """Fortran source without comments, continuation lines joined."""
    out = []
    for line in src.splitlines():
        line = line.split("!")[0].rstrip()
        if out and out[-1].endswith("&"):
            out[-1] = out[-1][:-1] + " " + line.strip()
        else:
            out.append(line)
    return [l for l in out if l.strip()]


def fortran_types(src):
    """{type name: [(field, kind, count)]} of the bind(C) derived types."""
    types, cur = {}, None
    for line in _strip(src):
        s = line.strip()
        m = re.match(r"type\s*,\s*bind\(C\)\s*::\s*(\w+)", s, re.I)
        if m:
            cur = m.group(1)
            types[cur] = []
            continue
        if cur and re.match(r"end\s+type", s, re.I):
            cur = None
            continue
        if cur:
            kind, names = [x.strip() for x in s.split("::")]
            for part in re.findall(r"(\w+)(?:\((\d+)\))?", names):
                types[cur].append((part[0], kind, int(part[1]) if part[1] else 1))
    return types


def c_layout(types):
    """offsetof / sizeof of the same structs and fields, from a gcc-compiled probe."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "%s"' % HEADER, "int main(void) {"]
    for t, fields in types.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (t, t))
        for f, _, _ in fields:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (t, f, t, f))
    lines.append("return 0; }")
    return "\n".join(lines)


def test_derived_types_match_c_structs(tmp_path):
    types = fortran_types(open(FMOD).read())
    assert set(types) == {"omx_grid_desc", "omx_medium", "omx_source_desc", "omx_plane_source_desc",
                          "omx_qgroup_desc"}
    src = tmp_path / "probe.c"
    src.write_text(c_layout(types))
    exe = tmp_path / "probe"
    r = subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.splitlines())
    for t, fields in types.items():
        # bind(C) types follow the companion C processor's layout rules: natural alignment
        off, align = 0, 1
        for f, kind, count in fields:
            size = KIND_SIZE[kind]
            off = (off + size - 1) // size * size
            assert int(got["%s.%s" % (t, f)]) == off, (t, f)
            off += size * count
            align = max(align, size)
        assert int(got["%s size" % t]) == (off + align - 1) // align * align, t


def _c_prototypes():
    text = re.sub(r"/\*.*?\*/", " ", open(HEADER).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|long long|const char \*)\s*\**\s*(omx_\w+)\s*\(([^;{]*?)\)\s*;", text):
        args = [a.strip() for a in m.group(2).split(",")] if m.group(2).strip() not in ("", "void") else []
        protos[m.group(1)] = args
    return protos


def _c_kind(arg):
    a = re.sub(r"\bconst\b", "", arg)
    a = re.sub(r"\w+\s*\[\d*\]$", "*", a)            # int grid_Ndims[3] -> pointer
    stars = a.count("*")
    base = a.replace("*", " ").split()[0]
    if base in ("omx_ctx", "omx_batch", "omx_closure", "omx_fdop", "void"):
        return "handle" + "*" * (stars - 1) if stars else "handle"
    if base.startswith("omx_"):
        return "struct*"
    name = {"int": "int", "int32_t": "int", "double": "double", "float": "float", "char": "char"}.get(base, base)
    if base == "long":
        name = "ll"
    return name + ("*" if stars else "")


def fortran_interfaces(src):
    """{bound C name: [argument kind]} from the interface block."""
    lines = _strip(src)
    out, i = {}, 0
    while i < len(lines):
        s = lines[i].strip()
        m = re.match(r".*function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", s, re.I)
        if not m:
            i += 1
            continue
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        decl = {}
        i += 1
        while not re.match(r"end\s+function", lines[i].strip(), re.I):
            d = lines[i].strip()
            if "::" in d:
                spec, names = [x.strip() for x in d.split("::")]
                for nm in re.findall(r"(\w+)(\(\*\))?", names):
                    decl[nm[0].lower()] = (spec.lower(), bool(nm[1]))
            i += 1
        kinds = []
        for a in args:
            spec, arr = decl[a.lower()]
            value = "value" in spec
            if spec.startswith("type(c_ptr)"):
                kinds.append("handle" if value else "handle*")
            elif spec.startswith("type("):
                kinds.append("struct*")
            else:
                base = {"integer(c_int)": "int", "integer(c_int32_t)": "int", "real(c_double)": "double",
                        "integer(c_long_long)": "ll"}[spec.split(",")[0].strip()]
                kinds.append(base if value and not arr else base + "*")
        out[m.group(3)] = kinds
    return out


def test_bound_functions_match_prototypes():
    protos = _c_prototypes()
    ifaces = fortran_interfaces(open(FMOD).read())
    assert len(ifaces) >= 20
    for name, kinds in ifaces.items():
        assert name in protos, name
        ck = [_c_kind(a) for a in protos[name]]
        assert ck == kinds, (name, ck, kinds)


def test_gpu_type_calls_are_declared():
    """Every library call the TMxll_3D_gpu type makes is an interface of omx_gpu_mod."""
    ifaces = fortran_interfaces(open(FMOD).read())
    calls = set(re.findall(r"\b(omx_\w+)\s*\(", open(FTYPE).read())) - {"omx_check", "omx_gpu_mod"}
    assert calls and calls <= set(ifaces), calls - set(ifaces)


@pytest.mark.parametrize("path", [FMOD, FTYPE])
def test_fortran_files_say_uncompiled(path):
    assert "Uncompiled" in open(path).read()
