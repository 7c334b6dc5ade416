"""The Fortran interface module (fortran/m_afivo_gb300.f90) cannot be
compiled here (no Fortran compiler), so its text is checked against the C
header: every bind(C) name is a function the header declares, and every
constant has the header's value."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header():
    return open(os.path.join(ROOT, "include", "afivo_gb300.h")).read()


def _header_constants(h):
    out = {}
    for body in re.findall(r"enum\s*\{([^}]*)\}", h):
        for name, val in re.findall(r"(AFV_\w+)\s*=\s*(-?\d+)", body):
            out[name] = int(val)
    return out


def test_bind_names_are_declared():
    h = _header()
    f = open(os.path.join(ROOT, "fortran", "m_afivo_gb300.f90")).read()
    names = [n for n in re.findall(r'bind\(C,\s*name="(\w+)"\)', f) if n.startswith("afv_")]
    assert len(names) > 10
    for n in names:
        assert re.search(r"\b%s\s*\(" % n, h), n


def test_constants_match_header():
    consts = _header_constants(_header())
    f = open(os.path.join(ROOT, "fortran", "m_afivo_gb300.f90")).read()
    found = 0
    for line in f.splitlines():
        if "parameter ::" not in line:
            continue
        for name, val in re.findall(r"(AFV_\w+)\s*=\s*(-?\d+)", line.split("::", 1)[1]):
            assert consts[name] == int(val), name
            found += 1
    assert found >= 20


def test_python_constants_match_header():
    import afivo_gb300 as a
    for name, val in _header_constants(_header()).items():
        if hasattr(a, name):
            assert getattr(a, name) == val, name
