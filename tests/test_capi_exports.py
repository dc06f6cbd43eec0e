"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute call: these run without a GPU)."""
import ctypes
import glob
import os
import re

from geoflac_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(gf_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("gf_read_params", "gf_setflac_host", "gf_create", "gf_fl_therm", "gf_fl_rheol", "gf_fl_node",
              "gf_fl_move", "gf_rmasses", "gf_dt_mass", "gf_change_phase", "gf_marker2elem", "gf_step"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = capi.load_library()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_mirrors_match_abi():
    lib = capi.load_library()
    assert lib.gf_struct_size(0) == ctypes.sizeof(capi.GfParams)
    assert lib.gf_struct_size(1) == ctypes.sizeof(capi.GfClock)
    assert lib.gf_struct_size(2) == ctypes.sizeof(capi.GfLayout)


def test_strerror_maps_reference_stop_codes():
    lib = capi.load_library()
    assert b"22" in lib.gf_strerror(22)
    assert b"40" in lib.gf_strerror(40)
