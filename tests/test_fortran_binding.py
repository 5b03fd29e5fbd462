"""The Fortran binding (eqdyna_gb300/fortran/eqd_gpu_mod.f90) against the C header, on CPU.

No Fortran compiler is needed: both sources are parsed as text.  Every bind(C) derived type must
list the fields of its C struct in the same order with the interoperable kind of the same C type
(double -> real(c_double), int32_t -> integer(c_int32_t), int64_t -> integer(c_int64_t), any
pointer -> type(c_ptr), fixed arrays with the same extent), every bind(C) interface must name an
entry point the header declares with the same number of arguments, and eqd_fill_from_globalvar
must set every field of the two structs it fills.
"""
import os
import re

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "eqdyna_gb300.h")
MODULE = os.path.join(ROOT, "eqdyna_gb300", "fortran", "eqd_gpu_mod.f90")

C_KIND = {"double": "c_double", "float": "c_float", "int32_t": "c_int32_t", "int64_t": "c_int64_t",
          "uint64_t": "c_int64_t", "int": "c_int"}


def _strip_c_comments(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def c_structs():
    text = _strip_c_comments(open(HEADER).read())
    out = {}
    for name, body in re.findall(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*\1\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(?:const\s+)?(\w+)\s+(.*)", decl)
            base, rest = m.group(1), m.group(2)
            for item in rest.split(","):
                item = item.strip()
                ptr = item.startswith("*")
                item = item.lstrip("*").strip()
                am = re.match(r"(\w+)\s*(?:\[(\d+)\])?$", item)
                fname, ext = am.group(1), int(am.group(2) or 1)
                fields.append((fname.lower(), "c_ptr" if ptr else C_KIND[base], ext))
        out[name] = fields
    return out


def c_functions():
    text = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\**\s*(eqd_\w+)\s*\(([^)]*)\)\s*;", text, flags=re.M | re.S):
        args = [a for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(1)] = len(args)
    return out


def _fortran_lines():
    src = open(MODULE).read()
    src = re.sub(r"![^\n]*", "", src)
    src = re.sub(r"&\s*\n\s*", " ", src)  # continuation lines
    return [ln.strip() for ln in src.splitlines() if ln.strip()]


def fortran_types():
    out, cur = {}, None
    for ln in _fortran_lines():
        m = re.match(r"type\s*,\s*bind\s*\(\s*C\s*\)\s*::\s*(\w+)", ln, flags=re.I)
        if m:
            cur = m.group(1)
            out[cur] = []
            continue
        if cur and re.match(r"end\s+type", ln, flags=re.I):
            cur = None
            continue
        if cur:
            m = re.match(r"(real|integer|type)\s*\(\s*(\w+)\s*\)\s*::\s*(.*)", ln, flags=re.I)
            assert m, ln
            kind = m.group(2).lower()
            for item in re.findall(r"(\w+)\s*(?:\(\s*(\d+)\s*\))?", m.group(3)):
                out[cur].append((item[0].lower(), kind, int(item[1] or 1)))
    return out


def fortran_interfaces():
    out = {}
    for ln in _fortran_lines():
        m = re.match(r".*function\s+(\w+)\s*\(([^)]*)\)\s*bind\s*\(\s*C\s*,\s*name\s*=\s*\"(\w+)\"", ln, flags=re.I)
        if m:
            args = [a for a in m.group(2).split(",") if a.strip()]
            out[m.group(3)] = len(args)
    return out


def test_every_fortran_type_matches_its_c_struct():
    cs, fs = c_structs(), fortran_types()
    assert {"eqd_scalars", "eqd_host_arrays", "eqd_options", "eqd_elem_device_view"} <= set(fs)
    for name, ffields in fs.items():
        assert name in cs, f"{name} has no C struct"
        assert ffields == cs[name], (name, [(a, b) for a, b in zip(ffields, cs[name]) if a != b][:3],
                                     len(ffields), len(cs[name]))


def test_every_fortran_interface_names_a_header_entry_with_its_arity():
    cf, fi = c_functions(), fortran_interfaces()
    assert {"eqd_gpu_init", "eqd_gpu_step", "eqd_gpu_fetch", "eqd_gpu_finalize",
            "eqd_gpu_elem_forces_noalloc"} <= set(fi)
    for name, n in fi.items():
        assert name in cf, name
        assert cf[name] == n, (name, n, cf[name])


def test_fill_from_globalvar_sets_every_field():
    src = "\n".join(_fortran_lines())
    body = re.search(r"subroutine\s+eqd_fill_from_globalvar(.*?)end\s+subroutine", src, flags=re.S | re.I).group(1)
    cs = c_structs()
    for var, struct in (("s", "eqd_scalars"), ("a", "eqd_host_arrays")):
        set_fields = {f.lower() for f in re.findall(rf"\b{var}%(\w+)\s*=", body)}
        missing = [f for f, _, _ in cs[struct] if f not in set_fields]
        assert not missing, (struct, missing)
