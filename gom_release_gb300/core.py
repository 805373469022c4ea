"""ctypes binding of the C ABI in include/gom_core.h.

``GomCore`` drives a context of any library that exports the ABI.  The product library is
``libgomcore.so`` (CUDA, sm_103a); ``load_core()`` fails loudly when it is missing or when no
GPU is visible -- there is no CPU fallback on the product path.  The CPU restatement used as
the test checker lives under ``oracle/`` and is loaded only by the tests, ``smoke()`` and the
CPU-baseline leg of ``bench.py`` through ``GomCore(lib_path=...)``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CORE_SO = PKG / "_build" / "libgomcore.so"

# gom_field enum of include/gom_core.h (tests check this table against the header)
FIELDS = [
    "eta_cell", "eta_cell_new", "eta_node", "wetdry_node",
    "un_face", "vn_face", "un_face_new", "vn_face_new", "un_elm", "vn_elm",
    "wn_cell", "wn_cell_new", "u_node", "v_node", "w_node", "u_face_level", "v_face_level",
    "dz_cell", "dz_cell_new", "dzhalf_cell", "dzhalf_cell_new",
    "dz_face", "dz_face_new", "dzhalf_face", "dzhalf_face_new",
    "dz_node", "dz_node_new", "dzhalf_node", "dzhalf_node_new",
    "top_layer_cell", "top_layer_face", "top_layer_node",
    "ainvg1", "ainvg2", "ainvdz1", "ainvdz2", "kh", "av", "kv",
    "salt_cell", "salt_cell_new", "temp_cell", "temp_cell_new", "salt_node", "temp_node",
    "salt_face", "temp_face", "rho_cell", "rho_node", "rho_face", "num_sub_elm",
    "cdb", "gamma_b", "qu_boundary", "elm_foot", "elm_near_edge",
    "wind_stress_normal", "wind_stress_tangnt", "gamma_t", "air_p", "eta_at_ob_old", "eta_at_ob_new",
    "q_add", "phi_sw", "phi_sz",
]

_CELL_FIELDS = {"eta_cell", "eta_cell_new", "wn_cell", "wn_cell_new", "dz_cell", "dz_cell_new", "dzhalf_cell",
                "dzhalf_cell_new", "top_layer_cell", "kv", "salt_cell", "salt_cell_new", "temp_cell",
                "temp_cell_new", "rho_cell", "phi_sw", "phi_sz"}
_NODE_FIELDS = {"eta_node", "wetdry_node", "u_node", "v_node", "w_node", "dz_node", "dz_node_new", "dzhalf_node",
                "dzhalf_node_new", "top_layer_node", "salt_node", "temp_node", "rho_node", "num_sub_elm"}


def field_kind(name: str) -> str:
    """Entity a field is indexed by: 'cell', 'face', 'node', 'qb' (river cells) or 'ob'."""
    if name == "qu_boundary":
        return "qb"
    if name in ("eta_at_ob_old", "eta_at_ob_new"):
        return "ob"
    if name == "air_p":
        return "node"
    if name in _CELL_FIELDS:
        return "cell"
    if name in _NODE_FIELDS:
        return "node"
    return "face"
FIELD_ID = {name: i + 1 for i, name in enumerate(FIELDS)}

ERR_NAMES = {0: "GOM_OK", 1: "GOM_E_ARG", 2: "GOM_E_CUDA", 3: "GOM_E_NOT_SPD", 4: "GOM_E_ZERO_PIVOT",
             5: "GOM_E_ELM", 6: "GOM_E_DRY", 7: "GOM_E_LAYER", 8: "GOM_E_DENSITY", 9: "GOM_E_PCG_MAXIT",
             10: "GOM_E_TIMEOUT", 11: "GOM_E_NOMEM"}

# gom_status.site of a mesh gom_geometry_build rejects (GOM_GEO_* of include/gom_core.h)
GOM_GEO = {"CONCAVE": 1, "AREA": 2, "MAX_NB": 3, "HANGING": 4, "SURROUNDING": 5, "FACE_COUNT": 6,
           "FACE_LENGTH": 7, "BALL": 8, "VORONOI": 9, "CENTRES": 10, "BOUNDARY": 11, "VERTICAL": 12}

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)


class GomDims(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_nodes", C.c_int32),
                ("n_layers", C.c_int32), ("max_nb", C.c_int32), ("n_ob", C.c_int32),
                ("n_qb", C.c_int32), ("n_runs", C.c_int32)]


_PARAM_D = ["gravity", "rho_o", "msl", "dt", "theta", "adv_onoff_depth", "von_karman", "cd_const",
            "dry_depth", "smagorinsky", "ah_0", "kh_0", "error_tolerance", "delta_z_min",
            "denominator_min_for_matrix"]
_PARAM_I = ["advection_flag", "elm_backtrace_flag", "elm_sub_iter", "elm_min_iter", "elm_max_iter",
            "bf_flag", "baroclinic_flag", "ana_density", "max_iteration_pcg", "transport_flag",
            "trans_sub_iter", "h_flux_limiter", "v_flux_limiter", "is_salt", "is_temp", "heat_option",
            "test_barrier_phantom_blocks", "precision", "turbulence_flag", "transport_solver"]
_PARAM_PP = ["pp_h1", "pp_h2", "pp_vdmax1", "pp_vdmax2", "pp_vdmin1", "pp_vdmin2", "pp_tdmin"]


class GomParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in _PARAM_D] + [(n, C.c_int32) for n in _PARAM_I] + \
               [(n, C.c_double) for n in _PARAM_PP]


_GEOM = [
    ("x_node", _D), ("y_node", _D), ("h_node", _D), ("adj_cells_at_node", _I), ("adj_cellnum_at_node", _I),
    ("node_count_each_element", _I), ("adj_nodes_at_node", _I), ("adj_nodenum_at_node", _I),
    ("bottom_layer_at_node", _I), ("initial_wetdry_node", _I),
    ("x_cell", _D), ("y_cell", _D), ("h_cell", _D), ("area", _D), ("tri_or_quad", _I),
    ("nodenum_at_cell", _I), ("facenum_at_cell", _I), ("adj_cellnum_at_cell", _I), ("sign_in_outflow", _I),
    ("bottom_layer_at_element", _I), ("ob_element_flag", _I), ("qb_element_flag", _I),
    ("x_face", _D), ("y_face", _D), ("h_face", _D), ("face_length", _D), ("delta_j", _D),
    ("cos_theta", _D), ("sin_theta", _D), ("cos_theta2", _D), ("sin_theta2", _D),
    ("adj_cellnum_at_face", _I), ("nodenum_at_face", _I), ("bottom_layer_at_face", _I),
    ("boundary_type_of_face", _I), ("isflowside3", _I), ("coriolis_factor", _D), ("manning", _D),
    ("bf_height", _D), ("ob_cell_id", _I), ("qb_cell", _I), ("qb_face", _I), ("z_level", _D), ("delta_z", _D),
    ("run_cell_start", _I), ("run_face_start", _I), ("run_node_start", _I), ("run_ob_start", _I),
]


class GomGeom(C.Structure):
    _fields_ = _GEOM


class GomForcing(C.Structure):
    _fields_ = [("elapsed_time", C.c_double), ("spinup_tide", C.c_double), ("spinup_baroclinic", C.c_double),
                ("reserved", C.c_double), ("eta_at_ob_old", _D), ("eta_at_ob_new", _D), ("q_add", _D),
                ("wind_stress_normal", _D), ("wind_stress_tangnt", _D), ("gamma_t", _D), ("air_p", _D),
                ("con_at_ob", _D), ("con_at_qb", _D), ("phi_sw", _D), ("phi_sz", _D)]


class GomStorm(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x0", "y0", "heading", "speed", "rmax", "dp", "b", "coriolis",
                                           "tide_amplitude", "tide_period", "tide_phase", "spinup", "t0")]


class GomSeries(C.Structure):
    _fields_ = [("n_series", C.c_int32), ("reserved", C.c_int32), ("start", _I), ("time", _D), ("value", _D)]


class GomBoundarySeries(C.Structure):
    _fields_ = [("julian_day", C.c_double), ("tide_spinup_period", C.c_double),
                ("baroclinic_spinup_period", C.c_double), ("step", C.c_int32), ("reference_diff_days", C.c_int32),
                ("tide_spinup", C.c_int32), ("baroclinic_spinup", C.c_int32), ("q_interp_method", C.c_int32),
                ("n_harmonic", C.c_int32)] + \
        [(n, _I) for n in ("ob_eta_type", "ob_harmonic_id", "ob_eta_id", "ob_salt_id", "ob_temp_id", "qb_q_id",
                           "qb_salt_id", "qb_temp_id")] + [("qb_portion", _D), ("harmonic_start", _I)] + \
        [(n, _D) for n in ("amplitude", "period_h", "nodal", "eq_arg", "phase", "phase_shift")] + \
        [(n, GomSeries) for n in ("eta", "q", "salt", "temp")] + \
        [(n, C.c_int32) for n in ("wind_flag", "wind_formular", "wind_spinup", "n_wind")] + \
        [("wind_spinup_period", C.c_double), ("rho_a", C.c_double), ("wind_station_node", _I)] + \
        [(n, GomSeries) for n in ("wind_u", "wind_v")] + \
        [("hurricane_flag", C.c_int32), ("hurricane_read_interval", C.c_int32), ("hurricane_start_jday", C.c_double),
         ("hurricane_end_jday", C.c_double), ("hurricane_frames", _D), ("hurricane_interp_method", C.c_int32),
         ("reserved_hurricane", C.c_int32), ("hurricane_track", C.c_double * 6)] + \
        [(n, C.c_int32) for n in ("heat_flag", "sol_swr", "n_air", "reserved_heat")] + \
        [(n, C.c_double) for n in ("fwz_a", "fwz_b", "fwz_c", "wind_height", "light_extinction", "sol_absorb",
                                   "sed_water_exchange", "t_sed", "sed_temp_coeff")] + \
        [("air_time", _D), ("air_values", _D), ("year", C.c_int32), ("month", C.c_int32), ("lon", C.c_double),
         ("lat", C.c_double)]


class GomMesh(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("n_nodes", "n_cells", "max_nb", "voronoi", "n_layers", "n_ob", "n_qb",
                                          "reserved")] + \
        [("x_node", _D), ("y_node", _D), ("h_node", _D), ("tri_or_quad", _I), ("nodenum_at_cell", _I),
         ("z_level", _D), ("msl", C.c_double), ("ob_nodes", _I), ("qb_nodes", _I)]


# outputs of gom_geometry_build, in gom_mesh_geometry order: (name, ctype, per, width)
# per: "node", "cell", "face", "ob", "qb"; width: values per entity ("nb" = max_nb, "nb1" = max_nb + 1)
MESH_GEOMETRY_OUT = [
    ("adj_cells_at_node", _I, "node", 1), ("adj_cellnum_at_node", _I, "node", "nb"),
    ("node_count_each_element", _I, "node", "nb"), ("adj_nodes_at_node", _I, "node", 1),
    ("adj_nodenum_at_node", _I, "node", "nb1"), ("bottom_layer_at_node", _I, "node", 1),
    ("initial_wetdry_node", _I, "node", 1),
    ("x_cell", _D, "cell", 1), ("y_cell", _D, "cell", 1), ("h_cell", _D, "cell", 1), ("area", _D, "cell", 1),
    ("facenum_at_cell", _I, "cell", 4), ("adj_cellnum_at_cell", _I, "cell", 4), ("sign_in_outflow", _I, "cell", 4),
    ("bottom_layer_at_element", _I, "cell", 1), ("ob_element_flag", _I, "cell", 1), ("qb_element_flag", _I, "cell", 1),
    ("x_face", _D, "face", 1), ("y_face", _D, "face", 1), ("h_face", _D, "face", 1), ("face_length", _D, "face", 1),
    ("delta_j", _D, "face", 1), ("cos_theta", _D, "face", 1), ("sin_theta", _D, "face", 1),
    ("cos_theta2", _D, "face", 1), ("sin_theta2", _D, "face", 1), ("adj_cellnum_at_face", _I, "face", 2),
    ("nodenum_at_face", _I, "face", 2), ("bottom_layer_at_face", _I, "face", 1),
    ("boundary_type_of_face", _I, "face", 1), ("isflowside3", _I, "face", 1),
    ("ob_cell_id", _I, "ob", 1), ("ob_face_id", _I, "ob", 1), ("qb_cell", _I, "qb", 1), ("qb_face", _I, "qb", 1),
]


class GomMeshGeometry(C.Structure):
    _fields_ = [("face_capacity", C.c_int32), ("n_faces", C.c_int32)] + [(n, t) for n, t, _, _ in MESH_GEOMETRY_OUT]


class GomStatus(C.Structure):
    _fields_ = [("code", C.c_int32), ("site", C.c_int32), ("entity", C.c_int32), ("layer", C.c_int32),
                ("value", C.c_double), ("entity_kind", C.c_int32), ("run", C.c_int32)]


class GomError(RuntimeError):
    def __init__(self, code: int, where: str, status: GomStatus | None = None, message: str = ""):
        self.code = code
        self.status = status
        s = f"{where}: {ERR_NAMES.get(code, code)}"
        if status is not None and status.code:
            s += f" (site={status.site} entity={status.entity} layer={status.layer} value={status.value:g})"
        if message:
            s += f" [{message}]"
        super().__init__(s)


ABI_VERSION = 4      # GOM_ABI_VERSION of include/gom_core.h

_STEPS = ["bottom_friction", "boundary_velocity", "advection", "momentum", "velocities", "layers",
          "node_velocity", "transport", "density", "turbulence", "swap"]


def _bind(lib: C.CDLL) -> C.CDLL:
    vp = C.c_void_p
    lib.gom_abi_version.restype = C.c_int
    lib.gom_errstr.restype = C.c_char_p
    lib.gom_errstr.argtypes = [C.c_int]
    lib.gom_last_message.restype = C.c_char_p
    lib.gom_last_message.argtypes = [vp]
    lib.gom_field_info.argtypes = [C.POINTER(GomDims), C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    lib.gom_create.argtypes = [C.POINTER(GomDims), C.POINTER(GomParams), C.POINTER(GomGeom), C.POINTER(vp)]
    lib.gom_destroy.argtypes = [vp]
    lib.gom_destroy.restype = None
    lib.gom_set_field.argtypes = [vp, C.c_int, vp, C.c_int64]
    lib.gom_get_field.argtypes = [vp, C.c_int, vp, C.c_int64]
    lib.gom_set_forcing.argtypes = [vp, C.POINTER(GomForcing)]
    for s in _STEPS:
        getattr(lib, f"gom_step_{s}").argtypes = [vp]
    lib.gom_step_free_surface.argtypes = [vp, C.POINTER(C.c_int32)]
    lib.gom_step_all.argtypes = [vp, C.POINTER(C.c_int32)]
    lib.gom_step_launch.argtypes = [vp]
    lib.gom_step_wait.argtypes = [vp, C.POINTER(C.c_int32)]
    lib.gom_conservation.argtypes = [vp, _D, _D]
    lib.gom_set_stations.argtypes = [vp, C.c_int32, C.c_int32, _I, _I]
    lib.gom_station_series.argtypes = [vp, _D]
    lib.gom_set_storms.argtypes = [vp, C.c_int32, C.POINTER(GomStorm), C.c_double]
    lib.gom_set_boundary_series.argtypes = [vp, C.POINTER(GomBoundarySeries)]
    lib.gom_push_hurricane_frame.argtypes = [vp, _D]
    lib.gom_push_hurricane_center.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    lib.gom_geometry_build.argtypes = [C.POINTER(GomMesh), C.POINTER(GomMeshGeometry), C.POINTER(GomStatus)]
    lib.gom_cold_start.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
    lib.gom_autotune.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32)]
    lib.gom_tuning_variants.argtypes = [C.POINTER(C.c_int32)]
    lib.gom_set_tuning.argtypes = [vp, C.POINTER(C.c_int32)]
    lib.gom_copy_run.argtypes = [vp, C.c_int32, vp, C.c_int32]
    lib.gom_profile_kernel.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_double)]
    lib.gom_device_bytes.argtypes = [vp]
    lib.gom_device_bytes.restype = C.c_int64
    lib.gom_snapshot_begin.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_void_p)]
    lib.gom_snapshot_ready.argtypes = [vp]
    lib.gom_snapshot_wait.argtypes = [vp]
    lib.gom_host_alloc.argtypes = [C.c_int64, C.POINTER(C.c_void_p)]
    lib.gom_host_free.argtypes = [C.c_void_p]
    lib.gom_host_free.restype = None
    lib.gom_get_status.argtypes = [vp, C.POINTER(GomStatus), C.c_int]
    lib.gom_synchronize.argtypes = [vp]
    lib.gom_pcg_iterations_total.argtypes = [vp]
    lib.gom_pcg_iterations_total.restype = C.c_int64
    lib.gom_stream.argtypes = [vp]
    lib.gom_stream.restype = vp
    lib.gom_measure_fp64_peak.argtypes = [_D]
    lib.gom_measure_fp64_issue.argtypes = [C.c_int32, _D]
    lib.gom_selftest_compares.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    return lib


def measure_fp64_peak(lib: C.CDLL) -> float:
    """FP64 FMA throughput of the current GPU (GFLOP/s), measured by the library."""
    v = C.c_double()
    rc = lib.gom_measure_fp64_peak(C.byref(v))
    if rc != 0:
        raise GomError(rc, "gom_measure_fp64_peak")
    return v.value


def measure_fp64_issue(lib: C.CDLL, active_lanes: int = 32) -> float:
    """FP64 warp instructions per second with `active_lanes` lanes of every warp working,
    measured by the library."""
    v = C.c_double()
    rc = lib.gom_measure_fp64_issue(int(active_lanes), C.byref(v))
    if rc != 0:
        raise GomError(rc, "gom_measure_fp64_issue")
    return v.value


def selftest_compares(lib: C.CDLL) -> tuple[int, int]:
    """(comparisons checked, mismatches) of the library's bit-pattern comparison self-test."""
    checked, bad = C.c_int64(), C.c_int64()
    rc = lib.gom_selftest_compares(C.byref(checked), C.byref(bad))
    if rc != 0:
        raise GomError(rc, "gom_selftest_compares")
    return checked.value, bad.value


def load_library(path: str | os.PathLike) -> C.CDLL:
    path = Path(path)
    if not path.exists():
        raise FileNotFoundError(f"{path} is not built")
    lib = _bind(C.CDLL(str(path), mode=C.RTLD_LOCAL))
    v = lib.gom_abi_version()
    if v != ABI_VERSION:
        raise RuntimeError(f"{path}: ABI version {v}, expected {ABI_VERSION}")
    return lib


def load_core() -> C.CDLL:
    """The CUDA library.  Raises if it is not built or no GPU is usable."""
    if not CORE_SO.exists():
        raise RuntimeError(f"CUDA extension missing: {CORE_SO} (run __graft_entry__.build())")
    return load_library(CORE_SO)


def _ptr(a: np.ndarray | None, kind):
    if a is None:
        return C.cast(None, kind)
    return a.ctypes.data_as(kind)


def _dbl(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _int(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class GomCore:
    """One context of a library exporting the GOM core ABI, created from a ``Deck``."""

    def __init__(self, deck, lib: C.CDLL | None = None, lib_path: str | os.PathLike | None = None):
        if lib is None:
            lib = load_library(lib_path) if lib_path is not None else load_core()
        self.lib = lib
        self.deck = deck
        d = deck
        p = d.params
        runs = getattr(d, "runs", None)
        self.dims = GomDims(d.n_cells, d.n_faces, d.n_nodes, d.n_layers, d.max_nb, d.n_ob, d.n_qb,
                            len(runs["run_cell_start"]) - 1 if runs else 0)
        self.params = GomParams(*[getattr(p, n) for n in _PARAM_D], *[int(getattr(p, n, 1 if n == "transport_solver" else 0))
                                                                      for n in _PARAM_I],
                                *[getattr(p, n) for n in _PARAM_PP])
        g = d.geo
        keep = {}
        for name, kind in _GEOM:
            if name == "ob_cell_id":
                arr = d.ob_cell_id
            elif name in ("qb_cell", "qb_face"):
                arr = getattr(d, name)
            elif name == "z_level":
                arr = d.z_level
            elif name == "delta_z":
                arr = d.delta_z
            elif name.startswith("run_"):
                if not runs:
                    keep[name] = None
                    continue
                arr = runs[name]
            else:
                arr = g[name]
            keep[name] = _dbl(arr) if kind is _D else _int(arr)
        self._geom_keep = keep
        self.geom = GomGeom(**{n: _ptr(keep[n], k) for n, k in _GEOM})
        ctx = C.c_void_p()
        rc = lib.gom_create(C.byref(self.dims), C.byref(self.params), C.byref(self.geom), C.byref(ctx))
        if rc != 0:
            raise GomError(rc, "gom_create")
        self.ctx = ctx
        self._forcing_keep = {}

    # ------------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "ctx", None):
            self.lib.gom_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ fields
    def field_info(self, name: str) -> tuple[int, int]:
        n = C.c_int64()
        eb = C.c_int32()
        rc = self.lib.gom_field_info(C.byref(self.dims), FIELD_ID[name], C.byref(n), C.byref(eb))
        if rc:
            raise GomError(rc, f"gom_field_info({name})")
        return n.value, eb.value

    def set_field(self, name: str, arr: np.ndarray):
        n, eb = self.field_info(name)
        a = _int(arr) if eb == 4 else _dbl(arr)
        if a.size != n:
            raise ValueError(f"{name}: {a.size} elements, expected {n}")
        self._check(self.lib.gom_set_field(self.ctx, FIELD_ID[name], a.ctypes.data, n), f"set_field({name})")

    def get_field(self, name: str) -> np.ndarray:
        n, eb = self.field_info(name)
        a = np.empty(n, dtype=np.int32 if eb == 4 else np.float64)
        self._check(self.lib.gom_get_field(self.ctx, FIELD_ID[name], a.ctypes.data, n), f"get_field({name})")
        return a

    def load_state(self, state: dict):
        for name, arr in state.items():
            self.set_field(name, arr)

    def state(self, names=None) -> dict:
        return {n: self.get_field(n) for n in (names or FIELDS)}

    # ------------------------------------------------------------------ forcing / steps
    def set_forcing(self, f: dict):
        keep = {}

        def arr(name):
            if name not in f or f[name] is None:
                return C.cast(None, _D)
            a = _dbl(np.asarray(f[name]).transpose(2, 1, 0).ravel()
                     if name in ("con_at_ob", "con_at_qb") else f[name])
            keep[name] = a
            return a.ctypes.data_as(_D)

        s = GomForcing(f.get("elapsed_time", 0.0), f.get("spinup_tide", 1.0), f.get("spinup_baroclinic", 1.0), 0.0,
                       arr("eta_at_ob_old"), arr("eta_at_ob_new"), arr("q_add"), arr("wind_stress_normal"),
                       arr("wind_stress_tangnt"), arr("gamma_t"), arr("air_p"), arr("con_at_ob"),
                       arr("con_at_qb"), arr("phi_sw"), arr("phi_sz"))
        self._forcing_keep = keep
        self._check(self.lib.gom_set_forcing(self.ctx, C.byref(s)), "set_forcing")

    def step(self, name: str):
        if name == "free_surface":
            it = C.c_int32()
            self._check(self.lib.gom_step_free_surface(self.ctx, C.byref(it)), "step_free_surface")
            return it.value
        self._check(getattr(self.lib, f"gom_step_{name}")(self.ctx), f"step_{name}")
        return None

    def step_all(self) -> int:
        it = C.c_int32()
        self._check(self.lib.gom_step_all(self.ctx, C.byref(it)), "step_all")
        return it.value

    def step_launch(self):
        self._check(self.lib.gom_step_launch(self.ctx), "step_launch")

    def step_wait(self) -> int:
        it = C.c_int32()
        self._check(self.lib.gom_step_wait(self.ctx, C.byref(it)), "step_wait")
        return it.value

    def synchronize(self):
        self._check(self.lib.gom_synchronize(self.ctx), "synchronize")

    def cold_start(self, salt: float, temp: float, av_0: float, kv_0: float):
        """Initial state built on the device (then ``step("density")`` as prepare does)."""
        self._check(self.lib.gom_cold_start(self.ctx, salt, temp, av_0, kv_0), "cold_start")

    def autotune(self, reps: int = 3) -> list[int]:
        """Pick the fastest compiled variant of each tunable launch on the current state."""
        out = (C.c_int32 * 4)()
        self._check(self.lib.gom_autotune(self.ctx, reps, out), "autotune")
        return list(out)

    def tuning_variants(self) -> list[int]:
        """Number of compiled variants of each tunable launch."""
        out = (C.c_int32 * 4)()
        self._check(self.lib.gom_tuning_variants(out), "tuning_variants")
        return list(out)

    def set_tuning(self, choice) -> None:
        """Select the variant of each tunable launch (-1 keeps the current one)."""
        arr = (C.c_int32 * 4)(*choice)
        self._check(self.lib.gom_set_tuning(self.ctx, arr), "set_tuning")

    KERNEL_ELM_WALK, KERNEL_MOMENTUM, KERNEL_TRANSPORT_SOLVE = 1, 2, 3

    def profile_kernel(self, which: int, reps: int = 5) -> float:
        """Mean milliseconds per launch of one kernel of the step, on the current state."""
        ms = C.c_double()
        self._check(self.lib.gom_profile_kernel(self.ctx, which, reps, C.byref(ms)), "profile_kernel")
        return ms.value

    def copy_run(self, dst_run: int, src: "GomCore", src_run: int):
        """Copy one run's state from another context (packed contexts being repacked)."""
        self._check(self.lib.gom_copy_run(self.ctx, dst_run, src.ctx, src_run), "copy_run")

    def device_bytes(self) -> int:
        return int(self.lib.gom_device_bytes(self.ctx))

    # ------------------------------------------------------------------ asynchronous snapshots
    def snapshot_begin(self, names, buffers) -> None:
        """Enqueue a copy of the named fields into the given arrays (pinned for overlap) after the
        work enqueued so far; read them only after snapshot_wait / snapshot_ready."""
        ids = (C.c_int32 * len(names))(*[FIELD_ID[n] for n in names])
        ptrs = (C.c_void_p * len(names))(*[b.ctypes.data for b in buffers])
        self._check(self.lib.gom_snapshot_begin(self.ctx, len(names), ids, ptrs), "snapshot_begin")

    def snapshot_ready(self) -> bool:
        rc = self.lib.gom_snapshot_ready(self.ctx)
        if rc < 0:
            self._check(rc, "snapshot_ready")
        return rc == 1

    def snapshot_wait(self) -> None:
        self._check(self.lib.gom_snapshot_wait(self.ctx), "snapshot_wait")

    def set_storms(self, storms, elapsed_time: float = 0.0):
        """Device-side storm forcing, one storm per run (objects with gom_storm's fields)."""
        arr = (GomStorm * len(storms))(*[GomStorm(*[float(getattr(s, n, 0.0)) for n, _ in GomStorm._fields_])
                                         for s in storms])
        self._check(self.lib.gom_set_storms(self.ctx, len(storms), arr, float(elapsed_time)), "set_storms")

    def set_boundary_series(self, bs) -> None:
        """Hold a ``series.BoundarySeries`` on the device: every later ``step_all`` /
        ``step_launch`` advances the clock and forms the boundary forcing from it first."""
        keep = []

        def ints(a):
            a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
            keep.append(a)
            return a.ctypes.data_as(_I)

        def dbls(a):
            a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
            keep.append(a)
            return a.ctypes.data_as(_D)

        sets = {}
        for kind in ("eta", "q", "salt", "temp", "wind_u", "wind_v"):
            start, t, v = bs.flat(kind)
            sets[kind] = GomSeries(len(start) - 1, 0, ints(start), dbls(t), dbls(v))
        wind = getattr(bs, "wind", None) or {}
        hur = getattr(bs, "hurricane", None) or {}
        frames = hur.get("frames")
        heat = getattr(bs, "heat", None) or {}
        air_t = np.asarray(heat.get("air_time", []), np.float64)
        air_v = np.asarray(heat.get("air_values", np.zeros((5, 0))), np.float64).reshape(5, -1)
        n_air = int(air_t.size)
        hs, amp, per, nod, eq, ph, shift = bs.flat_harmonics()
        arg = GomBoundarySeries(
            julian_day=float(bs.julian_day), tide_spinup_period=float(bs.tide_spinup_period),
            baroclinic_spinup_period=float(bs.baroclinic_spinup_period), step=int(bs.step),
            reference_diff_days=int(bs.reference_diff_days), tide_spinup=int(bs.tide_spinup),
            baroclinic_spinup=int(bs.baroclinic_spinup), q_interp_method=int(bs.q_interp_method),
            n_harmonic=len(hs) - 1, ob_eta_type=ints(bs.ob_eta_type), ob_harmonic_id=ints(bs.ob_harmonic_id),
            ob_eta_id=ints(bs.ob_eta_id), ob_salt_id=ints(bs.ob_salt_id), ob_temp_id=ints(bs.ob_temp_id),
            qb_q_id=ints(bs.qb_q_id), qb_salt_id=ints(bs.qb_salt_id), qb_temp_id=ints(bs.qb_temp_id),
            qb_portion=dbls(bs.qb_portion), harmonic_start=ints(hs), amplitude=dbls(amp), period_h=dbls(per),
            nodal=dbls(nod), eq_arg=dbls(eq), phase=dbls(ph), phase_shift=dbls(shift),
            wind_flag=int(wind.get("flag", 0)), wind_formular=int(wind.get("formular", 1)),
            wind_spinup=int(wind.get("spinup", 0)), n_wind=len(bs.series.get("wind_u", [])),
            wind_spinup_period=float(wind.get("spinup_period", 0.0)), rho_a=float(wind.get("rho_a", 1.2)),
            wind_station_node=ints(wind.get("station_node", [])),
            hurricane_flag=int(hur.get("flag", 0)), hurricane_read_interval=int(hur.get("read_interval", 1)),
            hurricane_start_jday=float(hur.get("start_jday", 0.0)), hurricane_end_jday=float(hur.get("end_jday", 0.0)),
            hurricane_frames=dbls(np.asarray(frames, np.float64).reshape(3, 3, -1).ravel())
            if frames is not None else None, hurricane_interp_method=int(hur.get("interp_method", 1)),
            hurricane_track=(C.c_double * 6)(*[float(v) for v in hur.get("track", [0.0] * 6)]),
            heat_flag=int(heat.get("flag", 0)), sol_swr=int(heat.get("sol_swr", 2)), n_air=n_air,
            fwz_a=float(heat.get("fwz_a", 9.2)), fwz_b=float(heat.get("fwz_b", 0.46)),
            fwz_c=float(heat.get("fwz_c", 2.0)), wind_height=float(heat.get("wind_height", 2.0)),
            light_extinction=float(heat.get("light_extinction", 0.45)), sol_absorb=float(heat.get("sol_absorb", 0.45)),
            sed_water_exchange=float(heat.get("sed_water_exchange", 0.3)), t_sed=float(heat.get("t_sed", 11.5)),
            sed_temp_coeff=float(heat.get("sed_temp_coeff", 0.0)),
            air_time=dbls(air_t) if n_air else None, air_values=dbls(air_v) if n_air else None,
            year=int(heat.get("year", 2001)), month=int(heat.get("month", 1)), lon=float(heat.get("lon", 0.0)),
            lat=float(heat.get("lat", 0.0)), **sets)
        self._check(self.lib.gom_set_boundary_series(self.ctx, C.byref(arg)), "set_boundary_series")

    def push_hurricane_frame(self, frame) -> None:
        """The next hurricane_ser.inp record, shape (3, n_nodes): wind_u, wind_v, air_p (Pa); the
        device takes it at the next read step of the boundary series' hurricane frames."""
        a = np.ascontiguousarray(np.asarray(frame, np.float64).reshape(3, -1))
        if a.shape[1] != self.deck.n_nodes:
            raise ValueError("a hurricane record has one (u, v, p) per node")
        self._check(self.lib.gom_push_hurricane_frame(self.ctx, a.ctypes.data_as(_D)), "push_hurricane_frame")

    def push_hurricane_center(self, x: float, y: float, julian_day: float) -> None:
        """Method 2: the next hurricane_center record (x, y, julian day), taken with the next
        frame at the next read step."""
        self._check(self.lib.gom_push_hurricane_center(self.ctx, float(x), float(y), float(julian_day)),
                    "push_hurricane_center")

    def conservation(self) -> tuple[float, float]:
        v = C.c_double()
        s = C.c_double()
        self._check(self.lib.gom_conservation(self.ctx, C.byref(v), C.byref(s)), "conservation")
        return v.value, s.value

    # ------------------------------------------------------------------ station time series
    def set_stations(self, hloc: int, station_cell=None, station_node=None) -> None:
        """Register the time-series stations (1-based ids): hloc 1 at cells, 2 at nodes."""
        ids = station_cell if hloc == 1 else station_node
        arr = np.ascontiguousarray(np.asarray(ids if ids is not None else [], dtype=np.int32))
        cells = arr.ctypes.data_as(_I) if hloc == 1 else None
        nodes = arr.ctypes.data_as(_I) if hloc == 2 else None
        self._check(self.lib.gom_set_stations(self.ctx, hloc, len(arr), cells, nodes), "set_stations")
        self._n_stations = len(arr)

    def station_series(self) -> np.ndarray:
        """(n_stations, 7 + 4 L) records: eta, H, ubar, u(1:L), vbar, v(1:L), sbar, salt(1:L),
        tbar, temp(1:L), air pressure (write_tser_out_files.f90 values)."""
        n = getattr(self, "_n_stations", 0)
        out = np.zeros((n, 7 + 4 * self.dims.n_layers), dtype=np.float64)
        self._check(self.lib.gom_station_series(self.ctx, out.ctypes.data_as(_D)), "station_series")
        return out

    def status(self, clear: bool = False) -> GomStatus:
        st = GomStatus()
        self.lib.gom_get_status(self.ctx, C.byref(st), 1 if clear else 0)
        return st

    def stream_handle(self) -> int:
        return int(self.lib.gom_stream(self.ctx) or 0)

    def pcg_iterations_total(self) -> int:
        return int(self.lib.gom_pcg_iterations_total(self.ctx))

    def _check(self, rc: int, where: str):
        if rc != 0:
            msg = self.lib.gom_last_message(self.ctx) if getattr(self, "ctx", None) else b""
            raise GomError(rc, where, self.status(), (msg or b"").decode(errors="replace"))


# ------------------------------------------------------------------ time loop (main.f90:53-304)
TIME_LOOP = ["bottom_friction", "boundary_velocity", "advection", "momentum", "free_surface",
             "velocities", "layers", "node_velocity", "transport", "density", "turbulence", "swap"]


def geometry_build(lib: C.CDLL, raw, max_nb: int, voronoi: int, z_level, msl: float, ob_pairs=(), q_pairs=()):
    """gom_geometry_build of a library (the CUDA library, or the oracle in tests): the start-up
    geometry of a mesh (``mesh.RawMesh``) with its vertical grid and boundary node pairs.
    Returns a dict of arrays shaped as ``mesh.build_geometry`` and ``deck._finish_levels`` hold
    them (n_faces rows for face arrays); raises GomError with the failing check's status."""
    x, y, h = (np.ascontiguousarray(a, dtype=np.float64) for a in (raw.x, raw.y, raw.h))
    tq = np.ascontiguousarray(raw.tri_or_quad, dtype=np.int32)
    cells = np.ascontiguousarray(raw.cells, dtype=np.int32).reshape(-1, 4)
    zl = np.ascontiguousarray(z_level, dtype=np.float64)
    ob = np.ascontiguousarray(np.asarray(ob_pairs, dtype=np.int32).reshape(-1, 2))
    qb = np.ascontiguousarray(np.asarray(q_pairs, dtype=np.int32).reshape(-1, 2))
    nn, nc, L = len(x), len(tq), len(zl) - 1
    m = GomMesh(nn, nc, int(max_nb), int(voronoi), L, len(ob), len(qb), 0,
                x.ctypes.data_as(_D), y.ctypes.data_as(_D), h.ctypes.data_as(_D), tq.ctypes.data_as(_I),
                cells.ctypes.data_as(_I), zl.ctypes.data_as(_D), float(msl), ob.ctypes.data_as(_I),
                qb.ctypes.data_as(_I))
    cap = int(tq.sum())
    count = {"node": nn, "cell": nc, "face": cap, "ob": len(ob), "qb": len(qb)}
    arrays = {}
    out = GomMeshGeometry(face_capacity=cap)
    for name, t, per, width in MESH_GEOMETRY_OUT:
        w = {"nb": max_nb, "nb1": max_nb + 1}.get(width, width)
        a = np.zeros((count[per], w) if w != 1 else count[per], dtype=np.int32 if t is _I else np.float64)
        arrays[name] = a
        setattr(out, name, a.ctypes.data_as(t))
    st = GomStatus()
    rc = lib.gom_geometry_build(C.byref(m), C.byref(out), C.byref(st))
    if rc != 0:
        raise GomError(rc, "gom_geometry_build", st if st.code else None)
    nf = out.n_faces
    for name, _, per, _ in MESH_GEOMETRY_OUT:
        if per == "face":
            arrays[name] = arrays[name][:nf].copy()
    arrays["n_faces"] = nf
    return arrays


def prepare(core: GomCore, state: dict):
    """prepare_gom.f90: upload the cold-start state and compute the initial density."""
    core.load_state(state)
    core.step("density")
