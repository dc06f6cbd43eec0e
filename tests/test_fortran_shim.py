"""The Fortran side of the drop-in (include/geoflac_gb300.f90, the bind(C)
mirror of the C header, and include/geoflac_gb300_shim.f90, the bodies of
the reference's routines), checked as text on CPU (no Fortran compiler
here): the derived types lay out like gf_params / gf_clock / gf_layout
(field names, order, offsets and total sizes under C's alignment rules,
against the ctypes mirrors whose sizes the library itself reports), every
bound entry point exists in the library, and the shim fills every
parameter and array and defines the reference's routine names."""
import ctypes as C
import os
import re

import pytest

from geoflac_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
IFACE = os.path.join(ROOT, "include", "geoflac_gb300.f90")
SHIM = os.path.join(ROOT, "include", "geoflac_gb300_shim.f90")
HEADER = os.path.join(ROOT, "include", "geoflac_gb300.h")


def _source(path):
    """Fortran text with comments removed and continuation lines joined."""
    out = []
    for line in open(path):
        line = line.split("!")[0].rstrip()
        if out and out[-1].endswith("&"):
            out[-1] = out[-1][:-1] + " " + line.strip()
        else:
            out.append(line)
    return [x for x in out if x.strip()]


def _parameters(lines):
    vals = {}
    for ln in lines:
        m = re.match(r"\s*integer(?:\(c_int\))?\s*,\s*parameter\s*::\s*(.*)", ln, re.I)
        if m:
            for item in m.group(1).split(","):
                if "=" in item:
                    k, v = item.split("=")
                    try:
                        vals[k.strip().lower()] = int(v)
                    except ValueError:
                        pass
    return vals


KINDS = {"integer(c_int)": (4, 4), "real(c_double)": (8, 8), "character(kind=c_char)": (1, 1),
         "type(c_ptr)": (8, 8)}


def _components(lines, tname, params):
    """[(name, size, align)] of `type, bind(C) :: tname` in declaration order."""
    comps, inside = [], False
    for ln in lines:
        s = ln.strip()
        if re.match(rf"type\s*,\s*bind\(c\)\s*::\s*{tname}\b", s, re.I):
            inside = True
            continue
        if inside and re.match(r"end\s+type", s, re.I):
            return comps
        if not inside:
            continue
        kind, decl = [x.strip() for x in s.split("::")]
        size, align = KINDS[kind.lower().replace(" ", "")]
        # split the declarations at top-level commas
        depth, cur, items = 0, "", []
        for ch in decl:
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            if ch == "," and depth == 0:
                items.append(cur)
                cur = ""
            else:
                cur += ch
        items.append(cur)
        for it in items:
            m = re.match(r"\s*(\w+)\s*(?:\((.*)\))?\s*$", it)
            count = 1
            if m.group(2):
                for dim in m.group(2).split(","):
                    dim = dim.strip().lower()
                    count *= params[dim] if dim in params else int(dim)
            comps.append((m.group(1), size * count, align))
    raise AssertionError(f"type {tname} not found")


def _c_layout(comps):
    off, out, amax = 0, [], 1
    for name, size, align in comps:
        off = (off + align - 1) // align * align
        out.append((name.lower(), off, size))
        off += size
        amax = max(amax, align)
    return out, (off + amax - 1) // amax * amax


@pytest.mark.parametrize("tname,cls,which", [("gf_params_t", capi.GfParams, 0), ("gf_clock_t", capi.GfClock, 1),
                                             ("gf_layout_t", capi.GfLayout, 2)])
def test_derived_types_mirror_the_c_structs(tname, cls, which):
    lines = _source(IFACE)
    comps = _components(lines, tname, _parameters(lines))
    layout, size = _c_layout(comps)
    expect = [(name.lower(), getattr(cls, name).offset, getattr(cls, name).size) for name, _ in cls._fields_]
    assert layout == expect
    assert size == C.sizeof(cls) == capi.load_library().gf_struct_size(which)


def test_bound_entry_points_exist_in_the_library():
    lib = capi.load_library()
    header = open(HEADER).read()
    names = re.findall(r"bind\(C,\s*name='(\w+)'\)", open(IFACE).read())
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
        assert re.search(rf"\b{n}\(", header), n


def test_shim_fills_every_parameter_and_array():
    lines = _source(IFACE)
    params = _parameters(lines)
    text = open(SHIM).read()
    for tname, var in (("gf_params_t", "gfp"), ("gf_layout_t", "gfl")):
        for name, _, _ in _components(lines, tname, params):
            assert re.search(rf"\b{var}%{name}\b", text, re.I), f"{var}%{name} is never set"
    # the clock goes both ways around every call
    for name in ("nloop", "nsrate", "nmarkers", "time", "dt", "dtavg", "dt_elastic", "dt_maxwell", "frac"):
        assert re.search(rf"gfk%{name}\s*=\s*{name}\b", text), name
        assert re.search(rf"\b{name}\s*=\s*gfk%{name}\b", text), name


def test_shim_replaces_the_reference_routines():
    text = open(SHIM).read()
    defined = set(m.lower() for m in re.findall(r"^subroutine\s+(\w+)", text, re.M | re.I))
    for r in ("fl_therm", "change_phase", "fl_rheol", "fl_node", "fl_move", "rmasses", "dt_mass", "init_visc",
              "itest_mesh", "remesh", "bar2euler", "lpeuler2bar", "marker2elem"):
        assert r in defined, r
    for helper in ("gf_push_clock", "gf_pull_clock", "gf_shim_init", "gf_shim_sync_host", "gf_shim_sync_device"):
        assert re.search(rf"subroutine\s+{helper}\b", text), helper
    # the reference's stop codes come back as stops
    for code in (22, 40, 41, 133, 134, 999):
        assert re.search(rf"case \({code}\)\s*\n\s*stop {code}\b", text), code
