"""GOM's own input decks: node.inp, cell.inp, main.inp and the boundary series files.

GOM's Fortran start-up reads these (read_node_inp.f90, read_cell_inp.f90, read_main_inp.f90 with
its card state machine, read_eta_ser.f90, read_q_ser.f90, read_salt_ser.f90, read_temp_ser.f90)
and its time loop turns the series into per-step forcing (setup_spinup.f90,
compute_boundary_eta.f90, calculate_Q.f90 and the series interpolation of
solve_transport_equation_v19.f90:229-397).  This module restates both on the host so that a
reference deck drives the C ABI exactly as GOM's driver would:

* ``read_deck(directory)``   parses a deck into plain arrays and card values (``DeckData``);
* ``deck_from_data(data)``   builds the ``Deck`` (mesh, geometry, vertical grid, parameters,
                             boundaries, initial tracers) that ``GomCore`` takes;
* ``SeriesForcing``          the per-step host forcing from the deck's series.

Supported as the hot path needs them: coordinate_system 1 (metres), ana_depth 0, voronoi 0 or 1,
open-boundary elevation types 1 (harmonic) and 2 (time series), river discharge series with
linear (1) or second-order Lagrange (2) interpolation, salinity / temperature series at open and
river boundaries, tide and baroclinic spin-up.  Cards the core does not read (output, checks,
withdraw/return, source/sink, tide potential, wind and hurricane data) are parsed but not used.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .deck import PI, Deck, HostForcing, Params, _finish_levels, f32
from .mesh import RawMesh


# ----------------------------------------------------------------------------- text readers
def _records(path: Path) -> list[list[str]]:
    """Data records of a GOM input file: skip_header_lines.f90 drops leading lines whose first
    column holds '!', 'C' or 'c'; list-directed reads then take whitespace-separated values from
    each record and ignore what follows them (trailing comments)."""
    out: list[list[str]] = []
    started = False
    for line in Path(path).read_text().splitlines():
        if not started:
            if not line.strip() or line[:1] in ("!", "C", "c"):
                continue
            started = True
        if not line.strip():
            continue
        tok = line.replace("\t", " ").split("!")[0].split()
        if tok:
            out.append(tok)
    return out


def read_node_inp(path) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """read_node_inp.f90:47-63 (coordinate_system 1): node count, then `id x y depth` records."""
    rec = _records(path)
    n = int(rec[0][0])
    a = np.array([[float(v) for v in r[1:4]] for r in rec[1:n + 1]])
    return a[:, 0].copy(), a[:, 1].copy(), a[:, 2].copy()


def read_cell_inp(path) -> tuple[np.ndarray, np.ndarray]:
    """read_cell_inp.f90:37-65: cell count, then `id 3|4 n1 .. n3|n4` records (CCW nodes)."""
    rec = _records(path)
    n = int(rec[0][0])
    tq = np.zeros(n, np.int32)
    cells = np.zeros((n, 4), np.int32)
    for i, r in enumerate(rec[1:n + 1]):
        k = int(r[1])
        tq[i] = k
        cells[i, :k] = [int(v) for v in r[2:2 + k]]
    return tq, cells


def _series_file(path, n_series: int, shape: int, with_method: bool = False):
    """read_eta_ser.f90 / read_q_ser.f90 / read_salt_ser.f90 / read_temp_ser.f90: shape 1 holds
    the series one after another, each with its header; shape 2 one header and a column per
    series.  Times become (t + time_adjust) * time_conv, values (v + adjust) * unit_conv.
    Returns (times, values, interp_method) with times / values lists of arrays per series."""
    rec = _records(path)
    times, values = [], []
    method = 1
    pos = 0
    if shape == 1:
        for _ in range(n_series):
            h = rec[pos]
            pos += 1
            cnt, tconv, tadj, uconv, uadj = int(h[1]), float(h[2]), float(h[3]), float(h[4]), float(h[5])
            if with_method and len(h) > 6:
                method = int(h[6])
            t = np.array([(float(r[0]) + tadj) * tconv for r in rec[pos:pos + cnt]])
            v = np.array([(float(r[1]) + uadj) * uconv for r in rec[pos:pos + cnt]])
            pos += cnt
            times.append(t)
            values.append(v)
    else:
        h = rec[0]
        cnt, tconv, tadj, uconv, uadj = int(h[1]), float(h[2]), float(h[3]), float(h[4]), float(h[5])
        rows = rec[1:1 + cnt]
        for s in range(n_series):
            times.append(np.array([(float(r[0]) + tadj) * tconv for r in rows]))
            values.append(np.array([(float(r[1 + s]) + uadj) * uconv for r in rows]))
    return times, values, method


def parse_main_inp(path) -> dict[str, list[list[str]]]:
    """main.inp as read_main_inp.f90 reads it: each card's header lines begin with its id in
    the first column (C01, C5_02, C20_1, ...); the data records that follow belong to that card.
    Returns card id -> list of records (tokens, trailing comments removed)."""
    cards: dict[str, list[list[str]]] = {}
    cur = None
    for line in Path(path).read_text().splitlines():
        if not line.strip() or line[:1] == "!":
            continue
        if line[:1] in ("C", "c"):
            cur = line.split()[0].upper()
            cards.setdefault(cur, [])
            continue
        tok = line.replace("\t", " ").split("!")[0].split()
        if tok and cur is not None:
            cards[cur].append(tok)
    return cards


# ----------------------------------------------------------------------------- deck data
@dataclass
class DeckData:
    """Everything the core and its host forcing take from a reference deck, as plain values."""

    name: str
    x: np.ndarray
    y: np.ndarray
    h: np.ndarray
    tri_or_quad: np.ndarray
    cells: np.ndarray
    cards: dict                      # scalar card values (see read_deck)
    z_level: np.ndarray              # (0:L)
    ob: np.ndarray                   # (n_ob, 7): node1 node2 eta_type harmonic_id eta_id salt_id temp_id
    qb: np.ndarray                   # (n_qb, 6): node1 node2 q_ser_id portion salt_id temp_id (portion float)
    series: dict = field(default_factory=dict)   # kind -> (times list, values list); kind in eta q salt temp
    salt_init: np.ndarray | None = None          # (N_n, L)
    temp_init: np.ndarray | None = None

    def to_npz(self, path):
        arrs = dict(x=self.x, y=self.y, h=self.h, tri_or_quad=self.tri_or_quad, cells=self.cells,
                    z_level=self.z_level, ob=self.ob, qb=self.qb)
        keys = sorted(self.cards)
        arrs["card_keys"] = np.array(keys)
        arrs["card_vals"] = np.array([float(self.cards[k]) for k in keys])
        for kind, (ts, vs) in self.series.items():
            for s, (t, v) in enumerate(zip(ts, vs)):
                arrs[f"ser_{kind}_{s}_t"] = t
                arrs[f"ser_{kind}_{s}_v"] = v
        if self.salt_init is not None:
            arrs["salt_init"] = self.salt_init
        if self.temp_init is not None:
            arrs["temp_init"] = self.temp_init
        arrs["name"] = np.array(self.name)
        np.savez_compressed(path, **arrs)

    @staticmethod
    def from_npz(path) -> "DeckData":
        z = np.load(path)
        cards = {str(k): float(v) for k, v in zip(z["card_keys"], z["card_vals"])}
        series: dict = {}
        for key in z.files:
            if key.startswith("ser_") and key.endswith("_t"):
                _, kind, s, _ = key.split("_")
                ts, vs = series.setdefault(kind, ({}, {}))
                ts[int(s)] = z[key]
                vs[int(s)] = z[key[:-2] + "_v"]
        series = {k: ([t[i] for i in sorted(t)], [v[i] for i in sorted(v)]) for k, (t, v) in series.items()}
        return DeckData(name=str(z["name"]), x=z["x"], y=z["y"], h=z["h"], tri_or_quad=z["tri_or_quad"],
                        cells=z["cells"], cards=cards, z_level=z["z_level"], ob=z["ob"], qb=z["qb"],
                        series=series, salt_init=z["salt_init"] if "salt_init" in z.files else None,
                        temp_init=z["temp_init"] if "temp_init" in z.files else None)


def _init_file(path, n_nodes: int, n_layers: int) -> np.ndarray:
    """read_salt_init.f90 / read_temp_init.f90: `node_id v(1..L)` per node."""
    rec = _records(path)
    out = np.zeros((n_nodes, n_layers))
    for r in rec[:n_nodes]:
        out[int(r[0]) - 1, :] = [float(v) for v in r[1:1 + n_layers]]
    return out


def read_deck(directory, overrides: dict | None = None) -> DeckData:
    """Parse a GOM deck directory (node.inp, cell.inp, main.inp, series and initial-tracer files).
    ``overrides`` replaces card values after parsing (e.g. hurricane_flag 0 where the deck's
    hurricane file is missing)."""
    d = Path(directory)
    c = parse_main_inp(d / "main.inp")
    v = {}

    def num(card, row, col):
        return float(c[card][row][col])

    v["gravity"], v["rho_o"], v["max_nb"] = num("C01", 0, 0), num("C01", 0, 1), num("C01", 0, 3)
    r = c["C1"][0]
    v["maxnod"], v["maxele"], v["h_node_adjust"], v["ana_depth"] = float(r[0]), float(r[1]), float(r[2]), float(r[3])
    v["coordinate_system"], v["lon"], v["lat"], v["voronoi"] = float(r[4]), float(r[5]), float(r[6]), float(r[7])
    L = int(num("C2", 0, 0))
    v["n_layers"], v["msl"] = L, num("C2", 0, 1)
    z = np.zeros(L + 1)
    z[0] = num("C2", 0, 2)
    for rec in c["C2_1"][:L]:
        z[int(rec[0])] = float(rec[1])
    r = c["C3"][0]
    v["dt"], v["ndt"], v["data_start_year"], v["data_time_shift"] = float(r[0]), float(r[1]), float(r[2]), float(r[3])
    v["start_year"], v["start_month"], v["start_day"] = float(r[4]), float(r[5]), float(r[6])
    v["start_hour"], v["start_minute"], v["start_second"] = float(r[7]), float(r[8]), float(r[9])
    r = c["C5_01"][0]
    for k, val in zip(("theta", "advection_flag", "adv_onoff_depth", "elm_backtrace_flag", "elm_sub_iter",
                       "elm_min_iter", "elm_max_iter"), r):
        v[k] = float(val)
    r = c["C5_02"][0]
    for k, val in zip(("bf_flag", "bf_varying", "manning", "bf_height", "von_karman"), r):
        v[k] = float(val)
    r = c["C5_03"][0]
    for k, val in zip(("baroclinic_flag", "ana_density", "ref_salt", "ref_temp", "dry_depth", "coriolis_option"), r):
        v[k] = float(val)
    r = c["C5_04"][0]
    for k, val in zip(("smagorinsky", "ah_0", "kh_0", "av_0", "kv_0"), r):
        v[k] = float(val)
    r = c["C6"][0]
    v["max_iteration_pcg"], v["error_tolerance"] = float(r[0]), float(r[1])
    r = c["C7"][0]
    v["transport_flag"], v["transport_solver"] = float(r[0]), float(r[1])
    r = c["C7_1"][0]
    v["trans_sub_iter"], v["h_flux_limiter"], v["v_flux_limiter"] = float(r[0]), float(r[1]), float(r[2])
    salt_row, temp_row = c["C7_2"][0], c["C7_2"][1]
    v["is_salt"], v["num_salt_ser"], v["salt_ser_shape"] = float(salt_row[0]), float(salt_row[1]), float(salt_row[2])
    v["is_temp"], v["num_temp_ser"], v["temp_ser_shape"] = float(temp_row[0]), float(temp_row[1]), float(temp_row[2])
    v["heat_option"] = num("C7_3", 0, 0)
    # cards C7_3 / C7_4: the heat balance of heat_term_by_term.f90
    for k, val in zip(("heat_option", "sol_swr", "fwz_a", "fwz_b", "fwz_c", "wind_height"), c["C7_3"][0]):
        v[k] = float(val)
    for k, val in zip(("light_extinction", "sol_absorb", "sed_water_exchange", "t_sed", "sed_temp_coeff"),
                      c.get("C7_4", [[]])[0]):
        v[k] = float(val)
    r20 = c["C20"]
    n_ob = int(r20[0][0])
    v["n_ob"], v["num_harmonic_ser"] = n_ob, float(r20[1][1])
    v["num_eta_ser"], v["eta_ser_shape"] = float(r20[2][1]), float(r20[2][3])
    ob = np.array([[int(x) for x in rec[1:8]] for rec in c.get("C20_1", [])[:n_ob]], dtype=np.int64).reshape(-1, 7)
    v["tide_spinup"], v["tide_spinup_period"] = num("C21", 0, 0), num("C21", 0, 1)
    v["baroclinic_spinup"], v["baroclinic_spinup_period"] = num("C21", 1, 0), num("C21", 1, 1)
    r22 = c["C22"][0]
    n_qb = int(r22[0])
    v["n_qb"], v["num_q_ser"], v["q_ser_shape"] = n_qb, float(r22[2]), float(r22[4])
    qb = np.array([[float(x) for x in rec[1:7]] for rec in c.get("C22_1", [])[:n_qb]]).reshape(-1, 6)
    v["wind_flag"] = num("C30", 0, 0)
    v["hurricane_flag"] = num("C31", 0, 0)
    if overrides:
        v.update(overrides)
    x, y, h = read_node_inp(d / "node.inp")
    h = h + v["h_node_adjust"]
    tq, cells = read_cell_inp(d / "cell.inp")
    series = {}
    if v["num_eta_ser"] > 0:
        shape = int(v["eta_ser_shape"])
        t, val, _ = _series_file(d / f"eta_ser{shape}.inp", int(v["num_eta_ser"]), shape)
        series["eta"] = (t, val)
    if v["num_q_ser"] > 0:
        shape = int(v["q_ser_shape"])
        t, val, method = _series_file(d / f"q_ser{shape}.inp", int(v["num_q_ser"]), shape, with_method=True)
        series["q"] = (t, val)
        v["q_interp_method"] = float(method)
    for kind, key in (("salt", "num_salt_ser"), ("temp", "num_temp_ser")):
        if v[key] > 0:
            shape = int(v[f"{kind}_ser_shape"])
            t, val, _ = _series_file(d / f"{kind}_ser{shape}.inp", int(v[key]), shape)
            series[kind] = (t, val)
    nn = len(x)
    if int(v["heat_option"]) == 1 and (d / "air_ser.inp").exists():
        # read_air_ser.f90:21-26: count, time conversion and adjustment, then rows of time, air and
        # dew-point temperature, wind speed, short-wave radiation, cloud (rain and evaporation unused)
        rec = _records(d / "air_ser.inp")
        n, conv, adj = int(rec[0][0]), float(rec[0][1]), float(rec[0][2])
        rows = rec[1:1 + n]
        t = np.array([(float(r[0]) + adj) * conv for r in rows])
        series["air"] = ([t] * 5, [np.array([float(r[col]) for r in rows]) for col in range(1, 6)])
    salt_init = _init_file(d / "salt_init.inp", nn, L) if (d / "salt_init.inp").exists() else None
    temp_init = _init_file(d / "temp_init.inp", nn, L) if (d / "temp_init.inp").exists() else None
    return DeckData(name=d.parent.name, x=x, y=y, h=h, tri_or_quad=tq, cells=cells, cards=v, z_level=z, ob=ob,
                    qb=qb, series=series, salt_init=salt_init, temp_init=temp_init)


# ----------------------------------------------------------------------------- deck
def julian_day0(cards: dict) -> float:
    """julian.f90:10-84 for the start date of card C3 (jday, not jday_1900)."""
    month_start = [0.0, 31.0, 59.0, 90.0, 120.0, 151.0, 181.0, 212.0, 243.0, 273.0, 304.0, 334.0]
    year, month = int(cards["start_year"]), int(cards["start_month"])
    jday = month_start[month - 1]
    if year % 4 == 0 and year != 1900 and month >= 3:
        jday = jday + 1
    return (jday + (int(cards["start_day"]) - 1) + int(cards["start_hour"]) / 24.0 +
            int(cards["start_minute"]) / 1440.0 + int(cards["start_second"]) / 86400.0)


def reference_diff_days(cards: dict) -> int:
    """calculate_reference_diff_days.f90:8-43 (the reference's year lengths, 364 for years
    divisible by 4, kept as they are)."""
    y1, y2 = int(cards["data_start_year"]), int(cards["start_year"])
    days = 0
    while y1 != y2:
        days += 365 if y1 % 4 != 0 else 364
        y1 += 1
    return days - int(cards["data_time_shift"])


def deck_from_data(data: DeckData, n_steps: int | None = None) -> Deck:
    """The Deck of a parsed reference deck: set_geometry_1/2 (mesh.py), the vertical grid of
    cards C2/C2_1, parameters of cards C5-C7, open and river boundaries of C20_1/C22_1, the
    initial tracers of salt_init.inp / temp_init.inp (a cold start: setup_cold_start.f90)."""
    v = data.cards
    if int(v["coordinate_system"]) != 1 or int(v.get("ana_depth", 0)) != 0:
        raise ValueError("only coordinate_system 1 with depths from node.inp is supported")
    L = int(v["n_layers"])
    params = Params(
        gravity=v["gravity"], rho_o=v["rho_o"], msl=v["msl"], dt=v["dt"], theta=v["theta"],
        adv_onoff_depth=v["adv_onoff_depth"], von_karman=v["von_karman"], dry_depth=v["dry_depth"],
        smagorinsky=v["smagorinsky"], ah_0=v["ah_0"], kh_0=v["kh_0"], error_tolerance=v["error_tolerance"],
        advection_flag=int(v["advection_flag"]), elm_backtrace_flag=int(v["elm_backtrace_flag"]),
        elm_sub_iter=int(v["elm_sub_iter"]), elm_min_iter=int(v["elm_min_iter"]), elm_max_iter=int(v["elm_max_iter"]),
        bf_flag=int(v["bf_flag"]), baroclinic_flag=int(v["baroclinic_flag"]), ana_density=int(v["ana_density"]),
        max_iteration_pcg=int(v["max_iteration_pcg"]), transport_flag=int(v["transport_flag"]),
        transport_solver=int(v["transport_solver"]), trans_sub_iter=int(v["trans_sub_iter"]),
        h_flux_limiter=int(v["h_flux_limiter"]), v_flux_limiter=int(v["v_flux_limiter"]),
        is_salt=int(v["is_salt"]), is_temp=int(v["is_temp"]), heat_option=int(v["heat_option"]),
        av_0=v["av_0"], kv_0=v["kv_0"], coriolis_lat=v["lat"] if int(v["coriolis_option"]) == 1 else 0.0,
        manning=v["manning"], bf_height=v["bf_height"], ref_salt=v["ref_salt"], ref_temp=v["ref_temp"])
    raw = RawMesh(x=data.x, y=data.y, h=data.h, tri_or_quad=data.tri_or_quad, cells=data.cells)
    ob_pairs = [(int(r[0]), int(r[1])) for r in data.ob]
    q_pairs = [(int(r[0]), int(r[1])) for r in data.qb]
    q_portion = [float(r[3]) for r in data.qb]
    deck = _finish_levels(data.name, raw, np.asarray(data.z_level, dtype=np.float64), params, ob_pairs, q_pairs,
                          q_portion, voronoi=int(v["voronoi"]), max_nb=int(v["max_nb"]),
                          coriolis_on=int(v["coriolis_option"]) != 0,
                          tide=dict(amplitude=[], period_h=[], phase=[], nodal=[], eq_arg=[], shift=0.0),
                          n_steps=int(v["ndt"]) if n_steps is None else n_steps)
    deck.init_salt_node = data.salt_init
    deck.init_temp_node = data.temp_init
    deck.meta = dict(reference=data)
    return deck


# ----------------------------------------------------------------------------- forcing
def _interp(times, values, u2, v2_prev):
    """The interval search of compute_boundary_eta.f90:100-111 (and calculate_Q.f90,
    solve_transport_equation_v19.f90:245-257): the first t2 with u1 <= u2 <= u3, then
    v2 = (u2 - u1)(v3 - v1)/(u3 - u1) + v1; with no such interval v2 keeps its previous value."""
    for t2 in range(1, len(times)):
        u1, u3 = times[t2 - 1], times[t2]
        if u1 <= u2 <= u3:
            v1, v3 = values[t2 - 1], values[t2]
            return (u2 - u1) * (v3 - v1) / (u3 - u1) + v1
    return v2_prev


class SeriesForcing(HostForcing):
    """Per-step host forcing of a reference deck, from its series and cards: setup_spinup.f90,
    compute_boundary_eta.f90 (types 1 and 2), calculate_Q.f90 (methods 1 and 2) and the boundary
    tracers of solve_transport_equation_v19.f90:229-397 for every subcycle.  Wind, air pressure
    and the heat-balance terms are zero (their readers are not part of the core)."""

    def __init__(self, deck: Deck):
        super().__init__(deck)
        data: DeckData = deck.meta["reference"]
        self.data = data
        v = data.cards
        self.julian_day = julian_day0(v)
        # reference_diff_days * 86400.0: an integer times a default-REAL constant, in single precision
        self.rdd_s = float(np.float32(reference_diff_days(v)) * np.float32(86400.0))
        self.q_add = np.zeros(deck.n_qb)
        self.wind_normal = np.zeros(deck.n_faces)
        self.wind_tangnt = np.zeros(deck.n_faces)
        self.v2_eta_old = math.nan
        self.v2_eta_new = math.nan

    def _times(self, kind, sid):
        t, v = self.data.series[kind]
        return t[sid - 1] - self.rdd_s, v[sid - 1]

    def spinups(self, elapsed):
        """setup_spinup.f90:10-48."""
        v = self.data.cards
        p = self.deck.params
        st = 1.0
        if int(v["tide_spinup"]) == 1:
            per = v["tide_spinup_period"] * 86400.0
            st = math.tanh(2.0 * elapsed / per) if elapsed < per else 1.0
        sb = 1.0
        if p.baroclinic_flag == 1 and int(v["baroclinic_spinup"]) == 1:
            per = v["baroclinic_spinup_period"] * 86400.0
            sb = math.tanh(2.0 * elapsed / per) if elapsed < per else 1.0
        return st, sb

    def step(self, it: int) -> dict:
        d = self.deck
        p = d.params
        elapsed = it * p.dt
        self.julian_day = self.julian_day + p.dt / 86400.0
        spin, spin_bc = self.spinups(elapsed)
        jd_s = self.julian_day * 86400.0
        # compute_boundary_eta.f90:22-125
        old = np.zeros(d.n_ob)
        new = np.zeros(d.n_ob)
        for i, row in enumerate(self.data.ob):
            etype = int(row[2])
            if etype == 2:
                t, vals = self._times("eta", int(row[4]))
                self.v2_eta_old = _interp(t, vals, jd_s - p.dt, self.v2_eta_old)
                old[i] = spin * self.v2_eta_old
                self.v2_eta_new = _interp(t, vals, jd_s, self.v2_eta_new)
                new[i] = spin * self.v2_eta_new
            elif etype != 0:
                raise ValueError(f"open-boundary elevation type {etype} is not supported by this forcing")
        out = dict(elapsed_time=elapsed, spinup_tide=spin, spinup_baroclinic=spin_bc,
                   eta_at_ob_old=old, eta_at_ob_new=new)
        # calculate_Q.f90:21-75
        if d.n_qb:
            method = int(self.data.cards.get("q_interp_method", 1))
            for i, row in enumerate(self.data.qb):
                t, vals = self._times("q", int(row[2]))
                if method == 1:
                    v2 = _interp(t, vals, jd_s, None)
                    if v2 is not None:
                        self.q_add[i] = v2 * row[3]
                else:
                    tt, qq = self.data.series["q"][0][int(row[2]) - 1], self.data.series["q"][1][int(row[2]) - 1]
                    self.q_add[i] = _lagrange2(tt, qq, jd_s) * row[3]
            out["q_add"] = self.q_add.copy()
        # solve_transport_equation_v19.f90:229-397, every subcycle
        nt = self.nt
        dt2 = p.dt / nt
        cob = np.zeros((d.n_ob, 2, nt))
        cqb = np.zeros((d.n_qb, 2, nt))
        v2 = math.nan
        for s in range(nt):
            u2 = (jd_s - p.dt) + (s + 1) * dt2
            for i, row in enumerate(self.data.ob):
                if p.is_salt and int(row[5]) > 0:
                    t, vals = self._times("salt", int(row[5]))
                    v2 = _interp(t, vals, u2, v2)
                    cob[i, 0, s] = spin_bc * v2
                if p.is_temp and int(row[6]) > 0:
                    t, vals = self._times("temp", int(row[6]))
                    v2 = _interp(t, vals, u2, v2)
                    cob[i, 1, s] = spin_bc * v2
            for i, row in enumerate(self.data.qb):
                if p.is_salt and int(row[4]) > 0:
                    t, vals = self._times("salt", int(row[4]))
                    v2 = _interp(t, vals, u2, v2)
                    cqb[i, 0, s] = spin_bc * v2
                if p.is_temp and int(row[5]) > 0:
                    t, vals = self._times("temp", int(row[5]))
                    v2 = _interp(t, vals, u2, v2)
                    cqb[i, 1, s] = spin_bc * v2
        out["con_at_ob"] = cob
        if d.n_qb:
            out["con_at_qb"] = cqb
        if self.first:
            out.update(self.static())
            self.first = False
        return out


def _lagrange2(times, values, u2):
    """calculate_Q.f90:47-75: second-order Lagrange interpolation through the three samples
    starting one before the first sample at or after u2 (series times as read, no offset)."""
    diff = np.where(times - u2 >= 0.0, times - u2, np.inf)
    # no sample at or after u2: minloc lands on the first padding entry past the series
    # (difference = 9999999 there), which the steps below turn into the last three samples
    min_index = int(np.argmin(diff)) + 1 if np.isfinite(diff).any() else len(times)
    if min_index == 1:
        min_index += 1
    min_index -= 1
    shift = (min_index + 2) - len(times)
    if shift > 0:
        min_index -= shift
    x = [times[min_index - 1 + k] for k in range(3)]
    y = [values[min_index - 1 + k] for k in range(3)]
    total = 0.0
    for ii in range(3):
        prod = y[ii]
        for jj in range(3):
            if jj != ii:
                prod = prod * (u2 - x[jj]) / (x[ii] - x[jj])
        total = total + prod
    return total


__all__ = ["DeckData", "read_deck", "deck_from_data", "SeriesForcing", "julian_day0", "reference_diff_days",
           "parse_main_inp", "read_node_inp", "read_cell_inp"]
_ = PI, f32
