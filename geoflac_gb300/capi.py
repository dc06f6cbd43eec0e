"""ctypes binding of the C-ABI in include/geoflac_gb300.h.

The structures below mirror gf_params / gf_clock / gf_layout field by field.
``load_library()`` loads the in-tree ``libgeoflac_gb300.so`` and raises if it
is missing: there is no CPU fallback for the step.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgeoflac_gb300.so")

MAXZONE, MAXBC, MAXZONE_AGE, MAXZONE_LAYER, MAXPH, MAXINH = 10, 20, 32, 10, 20, 100
MAX_MARKERS_PER_ELEM = 32
SEC_YEAR = 3.1558e7

MODE_FP64, MODE_MIXED = 0, 1

F_CORD, F_VEL, F_TEMP, F_STRESS, F_AREA, F_STRAIN, F_APS, F_VISN = (1 << k for k in range(8))
F_MASS, F_PHASE, F_RATE, F_BC, F_MARKERS = (1 << k for k in range(8, 13))
F_ALL = 0xFFFFFFFF

ERR = {0: "ok", -1: "CUDA error", -2: "bad argument", -3: "cannot open file",
       -4: "malformed .inp file", -5: "unsupported", -6: "timeout", -7: "out of memory",
       -8: "non-finite value", -9: "input larger than a fixed device scratch"}

_d = C.c_double
_i = C.c_int


def _arr(t, n):
    return t * n


class GfBatchConfig(C.Structure):
    _fields_ = [("threads", _i), ("items_per_thread", _i), ("ctas_per_sm", _i), ("graph_steps", _i)]


class GfParams(C.Structure):
    _fields_ = [
        ("nx", _i), ("nz", _i),
        ("x0", _d), ("z0", _d), ("rxbo", _d), ("rzbo", _d),
        ("ircoord", _i), ("coordfile", C.c_char * 200),
        ("nzonx", _i), ("nzony", _i),
        ("nelz_x", _arr(_i, MAXZONE)), ("nelz_y", _arr(_i, MAXZONE)),
        ("sizez_x", _arr(_d, MAXZONE)), ("sizez_y", _arr(_d, MAXZONE)),
        ("nystressbc", _i), ("nydrsides", _i), ("nofbc", _i),
        ("nofside", _arr(_i, MAXBC)), ("nbc1", _arr(_i, MAXBC)), ("nbc2", _arr(_i, MAXBC)),
        ("nbc", _arr(_i, MAXBC)),
        ("bca", _arr(_d, MAXBC)), ("bcb", _arr(_d, MAXBC)), ("bcc", _arr(_d, MAXBC)),
        ("bcd", _arr(_d, MAXBC)), ("bce", _arr(_d, MAXBC)), ("bcf", _arr(_d, MAXBC)),
        ("bcg", _arr(_d, MAXBC)), ("bch", _arr(_d, MAXBC)), ("bci", _arr(_d, MAXBC)),
        ("nyhydro", _i), ("iphsub", _i),
        ("pisos", _d), ("drosub", _d), ("damp_vis", _d), ("g", _d),
        ("i_prestress", _i), ("itherm", _i), ("istress_therm", _i), ("ishearh", _i),
        ("itemp_bc", _i), ("irtemp", _i),
        ("extra_pres", _d), ("t_top", _d), ("t_bot", _d), ("hs", _d), ("hr", _d), ("bot_bc", _d),
        ("tempfile", C.c_char * 200),
        ("nzone_age", _i),
        ("ictherm", _arr(_i, MAXZONE_AGE)), ("ixtb1", _arr(_i, MAXZONE_AGE)),
        ("ixtb2", _arr(_i, MAXZONE_AGE)), ("nph_layer", _arr(_i, MAXZONE_AGE)),
        ("iph_col_trans", _arr(_i, MAXZONE_AGE)),
        ("iph_col", _arr(_arr(_i, MAXZONE_LAYER), MAXZONE_AGE)),
        ("age_1", _arr(_d, MAXZONE_AGE)), ("tp1", _arr(_d, MAXZONE_AGE)), ("tp2", _arr(_d, MAXZONE_AGE)),
        ("hc", _arr(_arr(_d, MAXZONE_LAYER), MAXZONE_AGE)),
        ("nphase", _i), ("irheol", _arr(_i, MAXPH)),
    ] + [(n, _arr(_d, MAXPH)) for n in (
        "visc", "den", "alfa", "beta", "pln", "acoef", "eactiv", "vactiv", "rl", "rm",
        "plstrain1", "plstrain2", "fric1", "fric2", "cohesion1", "cohesion2", "dilat1", "dilat2",
        "conduct", "cp", "ts", "tl", "tk", "erodibility")] + [
        ("irphase", _i), ("phasefile", C.c_char * 200),
        ("inhom", _i),
        ("ix1", _arr(_i, MAXINH)), ("ix2", _arr(_i, MAXINH)), ("iy1", _arr(_i, MAXINH)),
        ("iy2", _arr(_i, MAXINH)), ("inphase", _arr(_i, MAXINH)), ("igeom", _arr(_i, MAXINH)),
        ("xinitaps", _arr(_d, MAXINH)),
        ("ten_off", _d), ("tau_heal", _d), ("v_min", _d), ("v_max", _d), ("efoldc", _d),
        ("ivis_shape", _i),
        ("itype_melting", _i), ("nelem_serp", _i), ("nelem_dike", _i),
        ("prod_magma", _d), ("prod_magma2", _d), ("rho_magma", _d), ("angle_mzone", _d),
        ("fmagma_max", _d), ("ratio_mantle_mzone", _d), ("ratio_crust_mzone", _d),
        ("latent_heat_magma", _d), ("lambda_freeze", _d), ("lambda_freeze_tdep", _d),
        ("weaken_ratio_plastic", _d), ("weaken_ratio_viscous", _d),
        ("ny_rem", _i), ("mode_rem", _i), ("ntest_rem", _i),
        ("angle_rem", _d), ("dx_rem", _d), ("topo_kappa", _d), ("fac_kappa", _d),
        ("idt_scale", _i), ("i_rey", _i), ("ifreq_rmasses", _i), ("ifreq_imasses", _i),
        ("ifreq_visc", _i), ("ifreq_avgsr", _i),
        ("dt_scale", _d), ("strain_inert", _d), ("xReyn", _d), ("frac", _d), ("fracm", _d), ("demf", _d),
        ("movegrid", _i), ("ndim", _i), ("mix_strain", _i), ("mix_stress", _i),
        ("time_max", _d), ("dtout_screen", _d), ("dtout_file", _d), ("dtsave_file", _d),
        ("io_flags", _arr(_i, 19)), ("lastout", _i), ("lastsave", _i),
        ("dxmin", _d), ("dzmin", _d), ("vbc", _d), ("Amin", _d),
        ("ivis_present", _i), ("incoming_left", _i), ("incoming_right", _i), ("nopbmax", _i),
        ("markers_per_side", _i), ("eclogite_rule", _i), ("therm_sweeps", _i),
    ]


class GfClock(C.Structure):
    _fields_ = [("nloop", _i), ("nsrate", _i), ("nmarkers", _i), ("need_remeshing", _i),
                ("time", _d), ("dt", _d), ("dtavg", _d),
                ("dt_elastic", _d), ("dt_maxwell", _d), ("dtmax_therm", _d),
                ("frac", _d), ("vel_max", _d), ("dlmin", _d),
                ("therm_sweeps", _i), ("therm_unconverged", _i)]


_P = C.POINTER
_pd, _pi, _pi8 = _P(_d), _P(_i), _P(C.c_int8)

LAYOUT_FIELDS = [
    ("cord", _pd), ("vel", _pd), ("temp", _pd), ("temp0", _pd), ("amass", _pd), ("rmass", _pd),
    ("bc", _pd), ("ncod", _pi),
    ("stress0", _pd), ("area", _pd), ("dvol", _pd), ("strain", _pd), ("se2sr", _pd),
    ("aps", _pd), ("visn", _pd), ("e2sr", _pd), ("source", _pd), ("shrheat", _pd), ("sshrheat", _pd),
    ("fmagma", _pd), ("fmagma2", _pd), ("dike_released", _pd),
    ("iphase", _pi), ("phase_ratio", _pd), ("jmoho", _pi), ("dhacc_correction", _pd),
    ("mark_a1", _pd), ("mark_a2", _pd), ("mark_age", _pd),
    ("mark_dead", _pi8), ("mark_phase", _pi8), ("mark_ntriag", _pi),
    ("mark_id_elem", _pi), ("nmark_elem", _pi),
    ("dhacc", _pd), ("extr_acc", _pd), ("dtopo", _pd),
    ("xoriginal", _pd), ("zoriginal", _pd), ("q_init", _pd), ("vel_flex_old", _pd),
    ("fmelt", _pd), ("fmelt2", _pd), ("dike_backlog", _pd), ("dike_marker_vol", _pd),
    ("mor_marker_vol", _pd), ("extrusion", _pd),
]


class GfLayout(C.Structure):
    _fields_ = [("nx", _i), ("nz", _i), ("nphase", _i), ("max_markers", _i)] + LAYOUT_FIELDS


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library.  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m geoflac_gb300.build` "
            "(the FLAC step has no CPU fallback)")
    lib = C.CDLL(path)
    P, K, Lp = C.POINTER(GfParams), C.POINTER(GfClock), C.POINTER(GfLayout)
    vp = C.c_void_p
    sig = {
        "gf_read_params": (_i, [C.c_char_p, P]),
        "gf_layout_sizes": (_i, [P, _P(C.c_size_t), _P(C.c_size_t), _P(C.c_size_t)]),
        "gf_setflac_host": (_i, [P, K, Lp]),
        "gf_create": (_i, [_P(vp), P, Lp, _i]),
        "gf_destroy": (None, [vp]),
        "gf_upload": (_i, [vp, C.c_uint]),
        "gf_download": (_i, [vp, C.c_uint]),
        "gf_set_clock": (_i, [vp, K]),
        "gf_get_clock": (_i, [vp, K]),
        "gf_set_params": (_i, [vp, P]),
        "gf_get_params": (_i, [vp, P]),
        "gf_outflac": (_i, [vp, C.c_char_p, _i]), "gf_outmarker": (_i, [vp, C.c_char_p, _i]),
        "gf_saveflac": (_i, [vp, C.c_char_p]), "gf_rsflac": (_i, [vp, C.c_char_p]),
        "gf_finish_setflac": (_i, [vp]),
        "gf_fl_therm": (_i, [vp]), "gf_change_phase": (_i, [vp]), "gf_fl_rheol": (_i, [vp]),
        "gf_fl_node": (_i, [vp]), "gf_fl_move": (_i, [vp]), "gf_rmasses": (_i, [vp]),
        "gf_dt_mass": (_i, [vp]), "gf_init_visc": (_i, [vp]), "gf_marker2elem": (_i, [vp]),
        "gf_flac": (_i, [vp]), "gf_step": (_i, [vp, _i]),
        "gf_itest_mesh": (_i, [vp, _P(_d)]), "gf_remesh": (_i, [vp]),
        "gf_status": (_i, [vp]), "gf_launch_count": (C.c_longlong, [vp]),
        "gf_strerror": (C.c_char_p, [_i]),
        "gf_struct_size": (C.c_size_t, [_i]),
        "gf_set_sync": (_i, [vp, _i]),
        "gf_stream": (vp, [vp]),
        "gf_batch_create": (_i, [_P(vp), _P(vp), _i]),
        "gf_batch_destroy": (None, [vp]),
        "gf_batch_set_config": (_i, [vp, _P(GfBatchConfig)]),
        "gf_batch_get_config": (_i, [vp, _P(GfBatchConfig)]),
        "gf_batch_tune": (_i, [vp, _i, _P(GfBatchConfig), _P(_d)]),
        "gf_batch_step": (_i, [vp, _i]),
        "gf_batch_stream": (vp, [vp]),
        "gf_batch_elements": (C.c_longlong, [vp]),
        "gf_batch_grid": (_i, [vp]),
        "gf_batch_sample": (_i, [vp, vp, _i, _i, _i]),
        "gf_batch_inject": (_i, [vp, vp, _i, _i]),
        "gf_batch_force_residual": (_i, [vp, _P(_d)]),
        "gf_batch_backup": (_i, [vp]),
        "gf_batch_restore": (_i, [vp, _P(_i), _i]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    for k, cls in enumerate((GfParams, GfClock, GfLayout)):
        n = lib.gf_struct_size(k)
        if n != C.sizeof(cls):
            raise RuntimeError(f"ABI mismatch for {cls.__name__}: C {n} vs ctypes {C.sizeof(cls)}")
    _lib = lib
    return lib


class GfError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = code
        msg = ERR.get(code)
        if msg is None and _lib is not None:
            msg = _lib.gf_strerror(code).decode()
        super().__init__(f"{where}: status {code} ({msg})")


def check(code: int, where: str = "") -> int:
    if code != 0:
        raise GfError(code, where)
    return code


def read_params(path: str, markers_per_side: int = 3, eclogite_rule: int = 0,
                therm_sweeps: int = 0) -> GfParams:
    lib = load_library()
    p = GfParams()
    p.markers_per_side = markers_per_side
    p.eclogite_rule = eclogite_rule
    p.therm_sweeps = therm_sweeps
    check(lib.gf_read_params(path.encode(), C.byref(p)), f"gf_read_params({path})")
    return p


class HostState:
    """Host arrays of one model in the reference's layout (Fortran order,
    0-based indices: ``cord[j, i, k]`` is the reference's cord(j+1,i+1,k+1))."""

    NODE2 = ("cord", "vel", "bc")
    NODE1 = ("temp", "temp0", "amass", "rmass")
    ELEM1 = ("aps", "visn", "e2sr", "source", "shrheat", "sshrheat", "fmagma", "fmagma2",
             "dike_released", "fmelt", "fmelt2", "dike_backlog", "dike_marker_vol", "mor_marker_vol")

    def __init__(self, p: GfParams):
        nx, nz, nph = p.nx, p.nz, p.nphase
        self.nx, self.nz, self.nphase = nx, nz, nph
        self.max_markers = nx * nz * MAX_MARKERS_PER_ELEM
        f8 = dict(dtype=np.float64, order="F")
        self.arrays = {}
        A = self.arrays
        for n in self.NODE2:
            A[n] = np.zeros((nz, nx, 2), **f8)
        for n in self.NODE1:
            A[n] = np.zeros((nz, nx), **f8)
        A["ncod"] = np.zeros((nz, nx, 2), dtype=np.int32, order="F")
        A["stress0"] = np.zeros((nz - 1, nx - 1, 4, 4), **f8)
        A["area"] = np.zeros((nz - 1, nx - 1, 4), **f8)
        A["dvol"] = np.zeros((nz - 1, nx - 1, 4), **f8)
        A["strain"] = np.zeros((nz - 1, nx - 1, 3), **f8)
        A["se2sr"] = np.zeros((nz - 1, nx - 1, 3), **f8)
        for n in self.ELEM1:
            A[n] = np.zeros((nz - 1, nx - 1), **f8)
        A["iphase"] = np.zeros((nz - 1, nx - 1), dtype=np.int32, order="F")
        A["phase_ratio"] = np.zeros((nph, nz - 1, nx - 1), **f8)
        A["jmoho"] = np.zeros(nx, dtype=np.int32)
        A["dhacc_correction"] = np.zeros(nx, dtype=np.float64)
        for k in ("dhacc", "extr_acc", "dtopo", "q_init", "vel_flex_old", "extrusion"):
            A[k] = np.zeros(nx, dtype=np.float64)
        # xoriginal, zoriginal as the two planes of one (nz, nx, 2) array
        A["orig"] = np.zeros((nz, nx, 2), **f8)
        A["xoriginal"] = A["orig"][:, :, 0]
        A["zoriginal"] = A["orig"][:, :, 1]
        M = self.max_markers
        A["mark_a1"] = np.zeros(M)
        A["mark_a2"] = np.zeros(M)
        A["mark_age"] = np.zeros(M)
        A["mark_dead"] = np.zeros(M, dtype=np.int8)
        A["mark_phase"] = np.zeros(M, dtype=np.int8)
        A["mark_ntriag"] = np.zeros(M, dtype=np.int32)
        A["mark_id_elem"] = np.zeros((MAX_MARKERS_PER_ELEM, nz - 1, nx - 1), dtype=np.int32, order="F")
        A["nmark_elem"] = np.zeros((nz - 1, nx - 1), dtype=np.int32, order="F")
        self.layout = GfLayout()
        self.layout.nx, self.layout.nz, self.layout.nphase, self.layout.max_markers = nx, nz, nph, M
        for name, typ in LAYOUT_FIELDS:
            setattr(self.layout, name, A[name].ctypes.data_as(typ))

    def __getitem__(self, k):
        return self.arrays[k]

    def rehome(self, names, make):
        """Move arrays to memory from ``make(nbytes) -> writable buffer``
        (e.g. pinned host memory), keeping contents and layout.  Call it
        before a device context is created on this state."""
        for name in names:
            old = self.arrays[name]
            buf = make(old.nbytes)
            new = np.ndarray(old.shape, dtype=old.dtype, buffer=buf, order="F")
            new[...] = old
            self.arrays[name] = new
            typ = dict(LAYOUT_FIELDS)[name]
            setattr(self.layout, name, new.ctypes.data_as(typ))
        self._keep = getattr(self, "_keep", []) + [make]

    def copy_from(self, other: "HostState"):
        for k, v in other.arrays.items():
            if k not in ("xoriginal", "zoriginal"):  # views of "orig"
                self.arrays[k][...] = v

    def snapshot(self):
        return {k: v.copy() for k, v in self.arrays.items()}


def setflac_host(p: GfParams, state: HostState) -> GfClock:
    lib = load_library()
    clk = GfClock()
    check(lib.gf_setflac_host(C.byref(p), C.byref(clk), C.byref(state.layout)), "gf_setflac_host")
    return clk
