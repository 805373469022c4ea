"""Output snapshots and the reference's output file formats.

``Snapshot`` takes copies of state fields through ``gom_snapshot_begin`` into pinned host buffers:
the copy is ordered after the step that produced the state, and the transfer overlaps the steps
that follow; ``wait()`` hands the arrays over.  The writers reproduce the reference's files from
such a snapshot:

* ``write_restart``: the unformatted sequential file of write_restart.f90:7-74 (gfortran record
  layout: a 4-byte little-endian length before and after each record), named
  ``<id_restart_out><it as I7.7>.out``;
* ``write_dump3d``: one time slice of the node dump of write_dump3D.f90:4-42, text
  (``IS3D_dump_binary = 0``, one ``F15.5`` time line, then per node ``1 + 6 L + 3`` values in
  ``E15.5E4``) or unformatted (``IS3D_dump_binary = 1``);
* ``tser_header`` / ``tser_row``: the station time-series files of open_tser_outfiles_tec.f90,
  open_tser_outfiles_vtk.f90, open_tser_outfiles_sub.f90:28-58 (headers) and
  write_tser_out_files.f90:30-330 (one row per output step), from the station records of
  ``GomCore.station_series`` (``gom_station_series``: the values are gathered on the GPU, so an
  output step moves a few kB instead of whole fields).

Arrays keep the library's layout (layer fastest per entity, ``gom_get_field`` sizes).
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from .core import FIELD_ID, GomCore

RESTART_FIELDS = ("eta_cell", "eta_cell_new", "eta_node", "un_face", "vn_face", "u_node", "v_node", "wn_cell",
                  "w_node", "salt_cell", "temp_cell", "rho_cell", "salt_node", "temp_node", "rho_node",
                  "salt_face", "temp_face", "rho_face")
DUMP3D_FIELDS = ("eta_node", "u_node", "v_node", "w_node", "salt_node", "temp_node", "rho_node")


class Snapshot:
    """Pinned host buffers for a fixed list of fields and the asynchronous copy into them."""

    def __init__(self, core: GomCore, names):
        self.core = core
        self.names = tuple(names)
        self._mem = []
        self.buffers = []
        for n in self.names:
            count, eb = core.field_info(n)
            p = C.c_void_p()
            core._check(core.lib.gom_host_alloc(max(1, count * eb), C.byref(p)), "host_alloc")
            self._mem.append(p)
            ctype = C.c_int32 if eb == 4 else C.c_double
            arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(ctype)), shape=(count,))
            self.buffers.append(arr)
        self.pending = False

    def begin(self):
        """Enqueue the copy after the work enqueued so far on the context."""
        self.core.snapshot_begin(self.names, self.buffers)
        self.pending = True

    def ready(self) -> bool:
        return not self.pending or self.core.snapshot_ready()

    def wait(self) -> dict:
        """Block until the copy has landed; returns name -> array views of the pinned buffers
        (valid until the next begin)."""
        if self.pending:
            self.core.snapshot_wait()
            self.pending = False
        return dict(zip(self.names, self.buffers))

    def close(self):
        if self.pending:
            self.core.snapshot_wait()
            self.pending = False
        for p in self._mem:
            self.core.lib.gom_host_free(p)
        self._mem = []
        self.buffers = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------- file formats
def _records(rows: np.ndarray) -> bytes:
    """gfortran unformatted sequential records, one per row of a 2-D float64 array."""
    n, w = rows.shape
    rec = np.empty(n, dtype=[("a", "<i4"), ("d", "<f8", (w,)), ("b", "<i4")])
    rec["a"] = 8 * w
    rec["b"] = 8 * w
    rec["d"] = rows
    return rec.tobytes()


def restart_file_name(id_restart_out: str, it: int) -> str:
    return f"{id_restart_out}{it:07d}.out"


def write_restart(path: str | os.PathLike, st: dict, n_layers: int) -> None:
    """write_restart.f90:21-73 from a state snapshot (RESTART_FIELDS)."""
    L = n_layers

    def cols(name, lo):
        a = np.asarray(st[name], dtype=np.float64)
        return a.reshape(-1, L - lo + 1)

    parts = [
        np.stack([st["eta_cell"], st["eta_cell_new"]], axis=1),
        np.asarray(st["eta_node"], dtype=np.float64)[:, None],
        np.hstack([cols("un_face", 1), cols("vn_face", 1)]),
        np.hstack([cols("u_node", 0), cols("v_node", 0)]),
        cols("wn_cell", 0),
        cols("w_node", 0),
        np.hstack([cols("salt_cell", 1), cols("temp_cell", 1), cols("rho_cell", 1)]),
        np.hstack([cols("salt_node", 1), cols("temp_node", 1), cols("rho_node", 1)]),
        np.hstack([cols("salt_face", 1), cols("temp_face", 1), cols("rho_face", 1)]),
    ]
    with open(path, "wb") as fh:
        for rows in parts:
            fh.write(_records(np.ascontiguousarray(rows, dtype=np.float64)))


def read_restart(path: str | os.PathLike, n_cells: int, n_faces: int, n_nodes: int, n_layers: int) -> dict:
    """Inverse of write_restart (for restart input and for checking files)."""
    L = n_layers
    data = np.fromfile(path, dtype=np.uint8)
    pos = 0
    out = {}

    def take(n, w):
        nonlocal pos
        rec = np.frombuffer(data, dtype=[("a", "<i4"), ("d", "<f8", (w,)), ("b", "<i4")], count=n, offset=pos)
        if n and (np.any(rec["a"] != 8 * w) or np.any(rec["b"] != 8 * w)):
            raise ValueError("record length mismatch")
        pos += n * (8 * w + 8)
        return rec["d"].reshape(n, w)

    r = take(n_cells, 2)
    out["eta_cell"], out["eta_cell_new"] = r[:, 0].copy(), r[:, 1].copy()
    out["eta_node"] = take(n_nodes, 1)[:, 0].copy()
    r = take(n_faces, 2 * L)
    out["un_face"], out["vn_face"] = r[:, :L].ravel(), r[:, L:].ravel()
    r = take(n_nodes, 2 * (L + 1))
    out["u_node"], out["v_node"] = r[:, :L + 1].ravel(), r[:, L + 1:].ravel()
    out["wn_cell"] = take(n_cells, L + 1).ravel()
    out["w_node"] = take(n_nodes, L + 1).ravel()
    for kind, n in (("cell", n_cells), ("node", n_nodes), ("face", n_faces)):
        r = take(n, 3 * L)
        out[f"salt_{kind}"], out[f"temp_{kind}"], out[f"rho_{kind}"] = (r[:, :L].ravel(), r[:, L:2 * L].ravel(),
                                                                        r[:, 2 * L:].ravel())
    if pos != data.size:
        raise ValueError("trailing bytes in restart file")
    return out


def _fortran_e(v: float, d: int = 5, e: int = 4, w: int = 15) -> str:
    """Fortran Ew.dEe with the default scale factor: 0.ddddd mantissa."""
    if v == 0.0 or not math.isfinite(v):
        s = (("-" if math.copysign(1.0, v) < 0 else "") + "0." + "0" * d + "E+" + "0" * e) if v == 0.0 else str(v)
        return s.rjust(w)
    a = abs(v)
    ex = math.floor(math.log10(a)) + 1
    m = round(a / 10.0 ** ex * 10 ** d)
    if m >= 10 ** d:
        m //= 10
        ex += 1
    elif m < 10 ** (d - 1):
        m *= 10
        ex -= 1
    s = ("-" if v < 0 else "") + "0." + f"{m:0{d}d}" + ("E+" if ex >= 0 else "E-") + f"{abs(ex):0{e}d}"
    return s.rjust(w)


def dump3d_rows(st: dict, n_layers: int) -> np.ndarray:
    """Per node: eta_node, u(0:L), v(0:L), w(0:L), S(1:L), T(1:L), rho(1:L)."""
    L = n_layers
    nn = np.asarray(st["eta_node"]).size
    return np.hstack([np.asarray(st["eta_node"], dtype=np.float64)[:, None],
                      np.asarray(st["u_node"]).reshape(nn, L + 1), np.asarray(st["v_node"]).reshape(nn, L + 1),
                      np.asarray(st["w_node"]).reshape(nn, L + 1), np.asarray(st["salt_node"]).reshape(nn, L),
                      np.asarray(st["temp_node"]).reshape(nn, L), np.asarray(st["rho_node"]).reshape(nn, L)])


def write_dump3d(fh, time_value: float, st: dict, n_layers: int, binary: bool = False) -> None:
    """One time slice of write_dump3D.f90:13-41 appended to an open file (text or binary mode):
    time_value is julian_day * IS3D_dump_time_conv."""
    rows = dump3d_rows(st, n_layers)
    if binary:
        fh.write(_records(np.array([[time_value]], dtype=np.float64)))
        fh.write(_records(rows))
        return
    fh.write(f"{time_value:15.5f}\n")
    for r in rows:
        fh.write("".join(_fortran_e(float(x)) for x in r) + "\n")


# ---------------------------------------------------------------------------- station time series
# file stems of mod_file_definition.f90:129-142 (.dat Tecplot, .txt Paraview) and titles of
# open_tser_outfiles_tec.f90:24-38, by tser_list order
TSER_KINDS = ("eta", "H", "u", "v", "salt", "temp", "airp")
TSER_FILES = {"eta": "eta_tser_from_msl", "H": "H_tser", "u": "u_tser", "v": "v_tser", "salt": "salt_tser",
              "temp": "temp_tser", "airp": "airp_tser"}
_TSER_TITLES = {"eta": "Water elevation time series from msl", "H": "Total water depth (H) time series",
                "u": "Velocity 2d u time series", "v": "Velocity 2d v time series", "salt": "Salinity time series",
                "temp": "Temperature time series", "airp": "Air pressure time series"}
# tser_time -> unit label and tser_time_conv (open_tser_out_files.f90:21-29)
TSER_TIME = {1: ("sec", 86400.0), 2: ("min", 1440.0), 3: ("hr", 24.0), 4: ("day", 1.0)}


def tser_time_value(julian_day: float, tser_time: int) -> float:
    """The first column of every row: julian_day * tser_time_conv."""
    return julian_day * TSER_TIME[tser_time][1]


def tser_header(kind: str, hloc: int, tser_time: int, names, n_layers: int, fmt: str = "tec") -> str:
    """Header lines of one time-series file (fmt "tec" for the .dat file, "vtk" for .txt).

    eta and H name one column per station; the layered kinds name the depth mean and each layer
    as ``<station>_(kk)``, kk = 00..L.  (The reference opens no air-pressure file: its rows go to
    the unit's default file, so only eta..temp have headers there.)"""
    out = []
    if fmt == "tec":
        out.append('Title = "' + _TSER_TITLES[kind] + (' at cell"' if hloc == 1 else ' at node"') + "\n")
        first = 'Variables = "Elapsed Time [' + TSER_TIME[tser_time][0] + ']"'
    else:
        first = '"Elapsed Time [' + TSER_TIME[tser_time][0] + ']"'
    if kind in ("eta", "H"):
        cols = "".join(', "' + str(n).strip() + '"' for n in names)
    else:
        cols = "".join(', "' + str(n).strip() + "_(" + f"{k:02d}" + ')"' for n in names for k in range(n_layers + 1))
    out.append(first + cols + "\n")
    return "".join(out)


def tser_values(kind: str, records: np.ndarray, n_layers: int) -> np.ndarray:
    """The values one row of ``kind`` writes, per station, from (n_stations, 7 + 4 L) records."""
    L = n_layers
    r = np.asarray(records, dtype=np.float64).reshape(-1, 7 + 4 * L)
    start = {"eta": 0, "H": 1, "u": 2, "v": 3 + L, "salt": 4 + 2 * L, "temp": 5 + 3 * L, "airp": 6 + 4 * L}[kind]
    width = L + 1 if kind in ("u", "v", "salt", "temp") else 1
    return r[:, start:start + width]


def tser_row(kind: str, time_value: float, records: np.ndarray, n_layers: int) -> str:
    """One line of write_tser_out_files.f90: E15.5E4 time, then ',' and E15.5E4 per value
    (format1 for eta, H, air pressure; format2, mean then layers 1..L per station, otherwise)."""
    vals = tser_values(kind, records, n_layers).ravel()
    return _fortran_e(float(time_value)) + "".join("," + _fortran_e(float(x)) for x in vals) + "\n"
