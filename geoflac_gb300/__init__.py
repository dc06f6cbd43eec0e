"""GB300-native explicit FLAC time step (GeoFLAC's fl_therm / fl_rheol /
fl_node / fl_move / rmasses / dt_mass / change_phase) behind a C-ABI.

Importing the package never falls back to CPU compute: the step runs only
through ``libgeoflac_gb300.so`` (see ``geoflac_gb300.build``).
"""
from .capi import GfError, HostState, load_library, read_params  # noqa: F401
from .flac import Flac, clone, new_state  # noqa: F401

__all__ = ["Flac", "GfError", "HostState", "load_library", "read_params", "new_state", "clone"]
