"""Consistency of the Fortran iso_c_binding module
(ns-lsm-single-phase_gb300/fortran/lsm_iso_c.F90) with the C headers: every
bound name is declared in include/*.h, and the bind(C) derived types list
the C structs' fields in the same order with matching kinds.  (No Fortran
compiler is available here; this checks the text.)"""
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(REPO, "ns-lsm-single-phase_gb300", "fortran", "lsm_iso_c.F90")
HEADERS = [os.path.join(REPO, "include", h) for h in ("lsm_c.h", "lsm_batch.h")]


def _c_text():
    return "\n".join(open(h).read() for h in HEADERS)


def _c_struct(name):
    txt = re.sub(r"/\*.*?\*/", "", _c_text(), flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\}" % name, txt, re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(int|double)\s+(.*)", decl)
        kind = "c_int" if m.group(1) == "int" else "c_double"
        for v in m.group(2).split(","):
            v = v.strip()
            n = re.match(r"(\w+)(\[(\d+)\])?", v)
            out.append((n.group(1), kind, int(n.group(3) or 1)))
    return out


def _f_type(name):
    txt = open(F90).read()
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type" % name, txt, re.S).group(1)
    out = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        m = re.match(r"(integer|real)\((c_int|c_double)\) :: (.*)", line)
        for v in m.group(3).split(","):
            v = v.strip()
            n = re.match(r"(\w+)(\((\d+)\))?", v)
            out.append((n.group(1), m.group(2), int(n.group(3) or 1)))
    return out


def test_bound_names_are_declared():
    names = re.findall(r'bind\(C, name="(\w+)"\)', open(F90).read())
    assert names
    txt = _c_text()
    for n in names:
        assert re.search(r"\b%s\s*\(" % n, txt), n


def test_struct_layouts_match():
    for c, f in (("lsm_grid", "lsm_grid"), ("lsm_params", "lsm_params"),
                 ("lsm_batch_instance", "lsm_batch_instance"), ("lsm_batch_config", "lsm_batch_config"),
                 ("lsm_geom_info", "lsm_geom_info")):
        assert [(a.lower(), k, n) for a, k, n in _c_struct(c)] == [(a.lower(), k, n) for a, k, n in _f_type(f)], c
