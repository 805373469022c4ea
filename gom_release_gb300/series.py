"""Boundary series held on the device (``gom_set_boundary_series``).

GOM's Fortran driver turns its boundary tables into per-step forcing on the host every step:
setup_spinup.f90 (tide and baroclinic spin-up), compute_boundary_eta.f90 (open-boundary elevation,
ob_eta_type -1 / 1 harmonic / 2 time series), calculate_Q.f90 (river discharge, linear or
second-order Lagrange) and the boundary-concentration interpolation of
solve_transport_equation_v19.f90:229-397.  ``BoundarySeries`` is the set of tables those routines
read -- the harmonic constituents of read_harmonic_ser.f90 and the series of read_eta_ser.f90,
read_q_ser.f90, read_salt_ser.f90 and read_temp_ser.f90 with the per-boundary ids of cards C20_1
and C22_1 -- in the flat layout the C ABI takes.  Once set on a context, every ``step_all`` /
``step_launch`` evaluates them on the device before the first phase, so a run needs no host
forcing per step.

Station wind (card C30, ``wind_flag`` 1 with ``windp_ser.inp``) rides along: with it set, the
device also forms get_windp_at_face.f90 / IDW_windp_ser.f90 and calculate_wind_stress.f90 every
step.

Builders:

* ``from_deck_data(deck)``  a reference deck read by ``gom_inputs.read_deck``;
* ``from_synthetic(deck)``  a synthetic deck of ``deck.py``: one harmonic series from its tide,
                            constant discharge and boundary-tracer series -- the same forcing
                            ``deck.HostForcing`` computes on the host;
* ``with_station_wind(bs, deck, n_stations)``  adds seeded station-wind series (one to three
                            stations on nodes spread over the mesh);
* ``with_hurricane_frames(bs, deck, ...)``  adds hurricane node frames (card C31, method 1) and
                            returns the records to push at the later read steps.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class BoundarySeries:
    """The argument of ``gom_set_boundary_series`` as numpy arrays (ids are 1-based, 0 = none)."""

    julian_day: float                     # julian_day before the next step
    step: int                             # it of the last step taken
    reference_diff_days: int
    tide_spinup: int
    tide_spinup_period: float             # days
    baroclinic_spinup: int
    baroclinic_spinup_period: float       # days
    q_interp_method: int
    ob_eta_type: np.ndarray               # (n_ob)
    ob_harmonic_id: np.ndarray
    ob_eta_id: np.ndarray
    ob_salt_id: np.ndarray
    ob_temp_id: np.ndarray
    qb_q_id: np.ndarray                   # (n_qb)
    qb_salt_id: np.ndarray
    qb_temp_id: np.ndarray
    qb_portion: np.ndarray
    # harmonic series: per series a dict of constituent arrays amplitude, period_h, nodal,
    # eq_arg, phase and the scalar phase_shift
    harmonics: list = field(default_factory=list)
    # kind -> list of (times, values) per series; kinds eta, q, salt, temp, and wind_u / wind_v
    # (one series per wind station, the same times)
    series: dict = field(default_factory=dict)
    # station wind (card C30): flag, formular, spinup, spinup_period (days), rho_a, station_node
    wind: dict = field(default_factory=dict)
    # hurricane node frames (card C31): flag, read_interval (steps), start_jday, end_jday, frames
    # (3 frames, 3 components u / v / air_p in Pa, n_nodes) = frames 0, 1 and 2, interp_method
    # (1 or 2), and for method 2 the track [x1, y1, t1, x2, y2, t2] (julian days)
    hurricane: dict = field(default_factory=dict)
    # heat balance (heat_option 1, sol_swr 2): flag, card C7_3 / C7_4 values (fwz_a, fwz_b, fwz_c,
    # wind_height, light_extinction, sol_absorb, sed_water_exchange, t_sed, sed_temp_coeff),
    # air_time (n_air) and air_values (5, n_air): T_air, T_dew, wind speed, solar radiation, cloud
    heat: dict = field(default_factory=dict)

    def flat(self, kind: str):
        """(start, time, value) of one kind: offsets (n + 1) and the concatenated samples."""
        ser = self.series.get(kind, [])
        start = np.zeros(len(ser) + 1, np.int32)
        for k, (t, _) in enumerate(ser):
            start[k + 1] = start[k] + len(t)
        t = np.concatenate([np.asarray(t, np.float64) for t, _ in ser]) if ser else np.zeros(0)
        v = np.concatenate([np.asarray(v, np.float64) for _, v in ser]) if ser else np.zeros(0)
        return start, t, v

    def flat_harmonics(self):
        """(start, amplitude, period_h, nodal, eq_arg, phase, phase_shift) of the harmonic series."""
        start = np.zeros(len(self.harmonics) + 1, np.int32)
        cols = {k: [] for k in ("amplitude", "period_h", "nodal", "eq_arg", "phase")}
        for h, s in enumerate(self.harmonics):
            start[h + 1] = start[h] + len(s["amplitude"])
            for k in cols:
                cols[k].extend(float(x) for x in s[k])
        shift = np.array([float(s["phase_shift"]) for s in self.harmonics], np.float64)
        return (start, *[np.asarray(cols[k], np.float64) for k in ("amplitude", "period_h", "nodal", "eq_arg",
                                                                   "phase")], shift)


def from_deck_data(deck, heat: bool = False) -> BoundarySeries:
    """The boundary tables of a reference deck (``deck.meta['reference']``, a ``DeckData``):
    ids from cards C20_1 / C22_1, series as the readers store them (times and values already
    adjusted and converted), start time from card C3 (julian.f90), reference_diff_days from
    calculate_reference_diff_days.f90, spin-up from card C21.  With ``heat`` (and the deck's
    heat_option 1, sol_swr 2 and its air series) also the heat balance of cards C7_3 / C7_4."""
    from .gom_inputs import julian_day0, reference_diff_days

    data = deck.meta["reference"]
    v = data.cards
    ob = np.asarray(data.ob).reshape(-1, 7)
    qb = np.asarray(data.qb).reshape(-1, 6)
    if np.any(ob[:, 2] == 1):
        raise ValueError("harmonic open boundaries need read_harmonic_ser tables, which the deck reader "
                         "does not parse")
    series = {k: list(zip(*data.series[k])) for k in ("eta", "q", "salt", "temp") if k in data.series}
    return BoundarySeries(
        julian_day=julian_day0(v), step=0, reference_diff_days=reference_diff_days(v),
        tide_spinup=int(v.get("tide_spinup", 0)), tide_spinup_period=float(v.get("tide_spinup_period", 0.0)),
        baroclinic_spinup=int(v.get("baroclinic_spinup", 0)),
        baroclinic_spinup_period=float(v.get("baroclinic_spinup_period", 0.0)),
        q_interp_method=int(v.get("q_interp_method", 1)),
        ob_eta_type=ob[:, 2].astype(np.int32), ob_harmonic_id=ob[:, 3].astype(np.int32),
        ob_eta_id=ob[:, 4].astype(np.int32), ob_salt_id=ob[:, 5].astype(np.int32),
        ob_temp_id=ob[:, 6].astype(np.int32),
        qb_q_id=qb[:, 2].astype(np.int32), qb_salt_id=qb[:, 4].astype(np.int32),
        qb_temp_id=qb[:, 5].astype(np.int32), qb_portion=qb[:, 3].astype(np.float64),
        series=series, heat=_deck_heat(data) if heat else {})


def _deck_heat(data) -> dict:
    v = data.cards
    if int(v.get("heat_option", 0)) != 1 or int(v.get("sol_swr", 0)) not in (1, 2) or "air" not in data.series:
        raise ValueError("the deck's heat balance needs heat_option 1, sol_swr 1 or 2 and air_ser.inp")
    ts, vs = data.series["air"]
    return dict(flag=1, sol_swr=int(v["sol_swr"]), year=int(v["start_year"]), month=int(v["start_month"]),
                lon=float(v["lon"]), lat=float(v["lat"]),
                fwz_a=v["fwz_a"], fwz_b=v["fwz_b"], fwz_c=v["fwz_c"], wind_height=v["wind_height"],
                light_extinction=v["light_extinction"], sol_absorb=v["sol_absorb"],
                sed_water_exchange=v["sed_water_exchange"], t_sed=v["t_sed"], sed_temp_coeff=v["sed_temp_coeff"],
                air_time=np.asarray(ts[0], np.float64), air_values=np.stack([np.asarray(x, np.float64) for x in vs]))


def _constant(value: float):
    """A two-sample series holding `value` at every time the run reaches: the interpolation
    (u2 - u1)(v3 - v1)/(u3 - u1) + v1 then returns v1 exactly."""
    return (np.array([-1.0e15, 1.0e15]), np.array([float(value), float(value)]))


def from_synthetic(deck) -> BoundarySeries:
    """The forcing of ``deck.HostForcing`` as device tables: every open boundary harmonic with
    the deck's tide (series 1), the rivers on one constant discharge series of value q_total
    split by q_portion, constant open-boundary and river salinity / temperature series (id 0
    where the deck leaves them unset), tide spin-up over tide_spinup_days, julian day 0."""
    n_ob, n_qb = deck.n_ob, deck.n_qb
    tide = deck.tide
    harm = [dict(amplitude=list(tide["amplitude"]), period_h=list(tide["period_h"]), nodal=list(tide["nodal"]),
                 eq_arg=list(tide["eq_arg"]), phase=list(tide["phase"]), phase_shift=float(tide["shift"]))]
    series = {"eta": [], "q": [], "salt": [], "temp": []}

    def sid(kind, value):
        if value is None:
            return 0
        series[kind].append(_constant(value))
        return len(series[kind])

    ob_salt, ob_temp = sid("salt", deck.ob_salt), sid("temp", deck.ob_temp)
    q_id = sid("q", deck.q_total) if n_qb else 0
    q_salt, q_temp = (sid("salt", deck.q_salt), sid("temp", deck.q_temp)) if n_qb else (0, 0)
    spin_days = float(deck.tide_spinup_days)
    ones_ob = np.ones(n_ob, np.int32)
    ones_qb = np.ones(n_qb, np.int32)
    return BoundarySeries(
        julian_day=0.0, step=0, reference_diff_days=0, tide_spinup=1 if spin_days > 0.0 else 0,
        tide_spinup_period=spin_days, baroclinic_spinup=0, baroclinic_spinup_period=0.0, q_interp_method=1,
        ob_eta_type=ones_ob.copy(), ob_harmonic_id=ones_ob.copy(), ob_eta_id=np.zeros(n_ob, np.int32),
        ob_salt_id=ones_ob * ob_salt, ob_temp_id=ones_ob * ob_temp,
        qb_q_id=ones_qb * q_id, qb_salt_id=ones_qb * q_salt, qb_temp_id=ones_qb * q_temp,
        qb_portion=np.asarray(deck.q_portion, np.float64).copy() if n_qb else np.zeros(0),
        harmonics=harm, series=series)


def with_station_wind(bs: BoundarySeries, deck, n_stations: int, *, hours: float = 6.0, formular: int = 1,
                      spinup_days: float = 0.0, rho_a: float = 1.2, seed: int = 0) -> BoundarySeries:
    """`bs` with `n_stations` (1..3) seeded wind stations: station k on the node nearest the k-th
    of three points spread across the mesh, samples every 10 to 20 minutes from before the run's
    start to `hours` after it (times in seconds since the reference day, as read_windp_ser.f90
    stores them), winds of 5 to 25 m/s turning over the run; the last station's series starts
    an hour late, so that get_windp_at_face.f90 gives it zero wind until then."""
    from dataclasses import replace

    if not 1 <= n_stations <= 3:
        raise ValueError("IDW_windp_ser.f90 takes one to three stations")
    rng = np.random.default_rng(seed)
    x, y = deck.geo["x_node"], deck.geo["y_node"]
    x0, x1, y0, y1 = float(x.min()), float(x.max()), float(y.min()), float(y.max())
    targets = [(0.2, 0.3), (0.8, 0.5), (0.5, 0.9)]
    nodes = [int(np.argmin((x - (x0 + fx * (x1 - x0))) ** 2 + (y - (y0 + fy * (y1 - y0))) ** 2)) + 1
             for fx, fy in targets[:n_stations]]
    t_start = bs.julian_day * 86400.0 + bs.reference_diff_days * 86400.0
    u_ser, v_ser = [], []
    for k in range(n_stations):
        first = t_start - 900.0 + (3600.0 if k == n_stations - 1 and n_stations > 1 else 0.0)
        steps = rng.uniform(600.0, 1200.0, size=int(hours * 3600.0 / 600.0) + 4)
        t = first + np.concatenate([[0.0], np.cumsum(steps)])
        speed = rng.uniform(5.0, 25.0, size=t.size)
        angle = rng.uniform(0.0, 2.0 * np.pi) + np.linspace(0.0, 1.5, t.size)
        u_ser.append((t, speed * np.cos(angle)))
        v_ser.append((t.copy(), speed * np.sin(angle)))
    series = dict(bs.series, wind_u=u_ser, wind_v=v_ser)
    wind = dict(flag=1, formular=int(formular), spinup=1 if spinup_days > 0.0 else 0,
                spinup_period=float(spinup_days), rho_a=float(rho_a), station_node=nodes)
    return replace(bs, series=series, wind=wind)


def hurricane_center(deck, k: int) -> tuple[float, float]:
    """Centre of record k of ``hurricane_record``: it crosses the mesh from west to east one tenth
    of its width per record, along the middle."""
    x, y = deck.geo["x_node"], deck.geo["y_node"]
    x0, x1, y0, y1 = float(x.min()), float(x.max()), float(y.min()), float(y.max())
    return x0 + 0.1 * k * (x1 - x0), y0 + 0.5 * (y1 - y0)


def hurricane_record(deck, k: int, *, radius: float = 0.0, seed: int = 0) -> np.ndarray:
    """Record k of a seeded synthetic hurricane_ser.inp, shape (3, n_nodes): a vortex (peak wind
    about 35 m/s at `radius`, default a quarter of the mesh's width; central pressure 60 hPa below
    101,325 Pa) whose centre crosses the mesh from west to east one tenth of its width per
    record, with a seeded background drift."""
    rng = np.random.default_rng(seed)
    x, y = deck.geo["x_node"], deck.geo["y_node"]
    x0, x1, y0, y1 = float(x.min()), float(x.max()), float(y.min()), float(y.max())
    width = max(x1 - x0, y1 - y0)
    rmax = radius if radius > 0.0 else 0.25 * width
    cx, cy = hurricane_center(deck, k)
    bu, bv = rng.uniform(-3.0, 3.0, size=2)
    dx, dy = x - cx, y - cy
    r = np.sqrt(dx * dx + dy * dy) + 1.0
    speed = 35.0 * (r / rmax) * np.exp(1.0 - r / rmax)
    u = -speed * dy / r + bu
    v = speed * dx / r + bv
    p = 101325.0 - 6000.0 * np.exp(-r / rmax)
    return np.stack([u, v, p])


def with_hurricane_frames(bs: BoundarySeries, deck, *, read_interval: int, n_records: int, start_jday: float,
                          end_jday: float, formular: int = 1, rho_a: float = 1.2, seed: int = 0,
                          interp_method: int = 1, record_days: float = 0.0):
    """`bs` with hurricane node frames (card C31) as read_hurricane_ser_0.f90 leaves them: frame 0 =
    record 0, frame 2 = record 1, frame 1 all zero; and the list of the records 2 .. n_records - 1
    to push with ``GomCore.push_hurricane_frame`` before each read step.  With interp_method 2
    the track holds the centres of records 0 and 1 at julian days start_jday and start_jday +
    record_days, and ``hurricane_centers`` gives the later ones.  The drag formula and air density
    are the station wind's (``wind`` keeps its flag)."""
    from dataclasses import replace

    recs = [hurricane_record(deck, k, seed=seed + k) for k in range(n_records)]
    frames = np.stack([recs[0], np.zeros_like(recs[0]), recs[1]])
    hur = dict(flag=1, read_interval=int(read_interval), start_jday=float(start_jday), end_jday=float(end_jday),
               frames=frames, interp_method=int(interp_method))
    if interp_method == 2:
        (xa, ya), (xb, yb) = hurricane_center(deck, 0), hurricane_center(deck, 1)
        hur["track"] = [xa, ya, float(start_jday), xb, yb, float(start_jday) + float(record_days)]
    wind = dict(bs.wind) if bs.wind else dict(flag=0, spinup=0, spinup_period=0.0)
    wind.setdefault("formular", int(formular))
    wind.setdefault("rho_a", float(rho_a))
    return replace(bs, hurricane=hur, wind=wind), recs[2:]


def with_heat_balance(bs: BoundarySeries, *, hours: float = 48.0, seed: int = 0, sed_temp_coeff: float = 0.3,
                      **cards) -> BoundarySeries:
    """`bs` with a seeded hourly air series (air temperature 15-30 C, dew point 5-10 C below it,
    wind 0-8 m/s, a diurnal short-wave cycle up to 900 W/m2 under seeded cloud cover) from an hour
    before the run's start, and the heat-balance cards of the Mobile Bay deck (C7_3: 9.2, 0.46, 2.0,
    2 m; C7_4: 0.45, 0.45, 0.3, 11.5 C) with the given sediment share; for sol_swr 1 the year,
    month and position of a July run at Mobile Bay (2005, 7, 88 W, 30.5 N); ``cards`` overrides
    them."""
    from dataclasses import replace

    rng = np.random.default_rng(seed)
    n = int(hours) + 3
    t0 = (bs.julian_day + bs.reference_diff_days) * 86400.0 - 3600.0
    t = t0 + 3600.0 * np.arange(n)
    hour_of_day = (t / 3600.0) % 24.0
    ta = 22.5 + 7.5 * np.sin(2.0 * np.pi * (hour_of_day - 9.0) / 24.0) + rng.normal(0.0, 0.5, n)
    td = ta - rng.uniform(5.0, 10.0, n)
    ws = rng.uniform(0.0, 8.0, n)
    cloud = rng.uniform(0.0, 1.0, n)
    sol = np.maximum(0.0, 900.0 * np.sin(np.pi * (hour_of_day - 6.0) / 12.0))
    heat = dict(flag=1, sol_swr=2, fwz_a=9.2, fwz_b=0.46, fwz_c=2.0, wind_height=2.0, light_extinction=0.45,
                sol_absorb=0.45, sed_water_exchange=0.3, t_sed=11.5, sed_temp_coeff=float(sed_temp_coeff),
                air_time=t, air_values=np.stack([ta, td, ws, sol, cloud]), year=2005, month=7, lon=-88.0, lat=30.5)
    heat.update(cards)
    return replace(bs, heat=heat)


def hurricane_centers(deck, n_records: int, start_jday: float, record_days: float) -> list:
    """(x, y, julian day) of the centres of records 2 .. n_records - 1 (method 2), to push with
    ``GomCore.push_hurricane_center`` alongside their frames."""
    return [(*hurricane_center(deck, k), float(start_jday) + k * float(record_days)) for k in range(2, n_records)]


__all__ = ["BoundarySeries", "from_deck_data", "from_synthetic", "with_station_wind", "with_heat_balance",
           "hurricane_record", "hurricane_center", "hurricane_centers", "with_hurricane_frames"]
