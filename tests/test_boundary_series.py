"""Boundary series held by the context (gom_set_boundary_series), on the CPU oracle: the forcing
it forms at the start of every step equals the host forcing GOM's driver computes
(setup_spinup.f90, compute_boundary_eta.f90, calculate_Q.f90, the boundary-concentration
interpolation of solve_transport_equation_v19.f90), bit for bit, on the reference's Mobile Bay deck
(elevation series, linear and Lagrange discharge, salinity / temperature series, 30 subcycles)
and on a synthetic estuary (harmonic tide with spin-up, constant river and boundary tracers); the
interior-mean open boundary (type -1) by hand; and the argument rules."""
import math
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, GomError, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state
from gom_release_gb300.gom_inputs import DeckData, SeriesForcing, deck_from_data
from gom_release_gb300.series import from_deck_data, from_synthetic

FIXTURE = Path(__file__).resolve().parent / "golden" / "mobile_bay.npz"
FORCING = ("eta_at_ob_old", "eta_at_ob_new", "q_add")   # the boundary tracers act through the state
STATE = ("eta_cell", "un_face", "salt_cell", "temp_cell")


def _pair(deck, lib, host_forcing):
    """Two contexts from one deck and state: `a` takes the host forcing every step, `b` holds the
    series and takes only the constant forcing (wind stress, Gamma_T) once."""
    st = initial_state(deck)
    a = GomCore(deck, lib_path=lib)
    b = GomCore(deck, lib_path=lib)
    prepare(a, st)
    prepare(b, st)
    b.set_forcing(host_forcing.static())
    return a, b


def _run_pair(a, b, host_forcing, bs, steps):
    b.set_boundary_series(bs)
    for it in range(1, steps + 1):
        a.set_forcing(host_forcing.step(it) if it > 1 else host_forcing.full(it))
        a.step_all()
        b.step_all()
        for name in FORCING:
            fa, fb = a.get_field(name), b.get_field(name)
            assert np.array_equal(fa, fb), (it, name, np.abs(fa - fb).max())
    for name in STATE:
        assert np.array_equal(a.get_field(name), b.get_field(name)), name


@pytest.mark.parametrize("q_method", [1, 2])
def test_mobile_bay_series_equal_host_forcing(oracle_so, q_method):
    data = DeckData.from_npz(FIXTURE)
    data.cards = dict(data.cards, q_interp_method=float(q_method))
    deck = deck_from_data(data)
    a, b = _pair(deck, oracle_so, SeriesForcing(deck))
    bs = from_deck_data(deck)
    assert bs.q_interp_method == q_method and bs.reference_diff_days == -212
    _run_pair(a, b, SeriesForcing(deck), bs, steps=3)


def test_synthetic_estuary_series_equal_host_forcing(oracle_so):
    deck = estuary(nx=14, ny=6, dx=100.0, n_layers=6, trans_sub_iter=3)
    deck.tide_spinup_days = 0.01      # the ramp runs over the first 14 steps
    a, b = _pair(deck, oracle_so, HostForcing(deck))
    bs = from_synthetic(deck)
    assert bs.tide_spinup == 1 and len(bs.harmonics) == 1
    _run_pair(a, b, HostForcing(deck), bs, steps=4)
    assert 0.0 < b.get_field("eta_at_ob_new")[0] or b.get_field("eta_at_ob_new")[0] < 0.0


def test_restart_from_step_continues_the_clock(oracle_so):
    """A context given the series at step k (julian day advanced k steps) forms the forcing of
    step k + 1 as the host forcing does."""
    deck = estuary(nx=10, ny=5, dx=100.0, n_layers=4, trans_sub_iter=2)
    deck.tide_spinup_days = 0.01
    hf = HostForcing(deck)
    for it in range(1, 8):
        hf.step(it)
    bs = replace(from_synthetic(deck), step=7, julian_day=hf.julian_day)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, initial_state(deck))
    c.set_forcing(hf.static())
    c.set_boundary_series(bs)
    c.step_all()
    want = hf.step(8)
    for name in ("eta_at_ob_old", "eta_at_ob_new"):
        assert np.array_equal(c.get_field(name), want[name]), name


def test_interior_mean_open_boundary(oracle_so):
    """compute_boundary_eta.f90:45-70 (ob_eta_type -1): eta_at_ob_old is the mean elevation of the
    interior cells around the open-boundary cell's nodes, a cell counted once per node it
    shares; eta_at_ob_new keeps its value."""
    deck = estuary(nx=10, ny=5, dx=100.0, n_layers=4, trans_sub_iter=2)
    st = initial_state(deck)
    rng = np.random.default_rng(7)
    st["eta_cell"] = rng.uniform(-0.2, 0.2, deck.n_cells)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, st)
    hf = HostForcing(deck)
    f = hf.full(1)
    f["eta_at_ob_new"] = np.full(deck.n_ob, 0.125)
    c.set_forcing(f)
    bs = from_synthetic(deck)
    bs.ob_eta_type = np.full(deck.n_ob, -1, np.int32)
    c.set_boundary_series(bs)
    eta0 = c.get_field("eta_cell")
    c.step_all()
    g = deck.geo
    want = np.zeros(deck.n_ob)
    for i, cell in enumerate(deck.ob_cell_id):
        vals = []
        for l in range(int(g["tri_or_quad"][cell - 1])):
            nd = int(g["nodenum_at_cell"][cell - 1, l])
            for i2 in range(int(g["adj_cells_at_node"][nd - 1])):
                ie = int(g["adj_cellnum_at_node"][nd - 1, i2])
                if g["ob_element_flag"][ie - 1] == 0:
                    vals.append(eta0[ie - 1])
        s = 0.0
        for v in vals:
            s = s + v
        want[i] = s / len(vals)
    assert np.array_equal(c.get_field("eta_at_ob_old"), want)
    assert np.all(c.get_field("eta_at_ob_new") == 0.125)


def _bad_series(deck):
    bs = from_synthetic(deck)
    yield replace(bs, ob_eta_type=np.full(deck.n_ob, 4, np.int32))
    yield replace(bs, ob_harmonic_id=np.full(deck.n_ob, 2, np.int32))
    yield replace(bs, qb_q_id=np.full(deck.n_qb, 5, np.int32))
    yield replace(bs, q_interp_method=3)
    s = dict(bs.series)
    s["q"] = [(np.array([2.0, 1.0]), np.array([1.0, 1.0]))]      # times decrease
    yield replace(bs, series=s)


def test_argument_rules(oracle_so):
    deck = estuary(nx=8, ny=4, dx=100.0, n_layers=3, trans_sub_iter=1)
    c = GomCore(deck, lib_path=oracle_so)
    for bs in _bad_series(deck):
        with pytest.raises(GomError) as e:
            c.set_boundary_series(bs)
        assert e.value.code == 1
    c.set_boundary_series(from_synthetic(deck))


# ----------------------------------------------------------------------------- station wind
def _station_wind_host(deck, bs, julian_day, elapsed):
    """get_windp_at_face.f90:18-85, IDW_windp_ser.f90:27-118, setup_spinup.f90:44-54 and
    calculate_wind_stress.f90:20-74 (heat_model_flag 0) restated in numpy, in the reference's order
    of operations: (wind_stress_normal, wind_stress_tangnt, Gamma_T) of one step."""
    w = bs.wind
    a = deck.geo
    u2 = julian_day * 86400.0
    rdd = float(np.float32(bs.reference_diff_days) * np.float32(86400.0))
    st = []
    for (tu, vu), (tv, vv) in zip(bs.series["wind_u"], bs.series["wind_v"]):
        val = [0.0, 0.0]
        for comp, (t, v) in enumerate(((tu, vu), (tv, vv))):
            for q in range(1, len(t)):
                u1, u3 = t[q - 1] - rdd, t[q] - rdd
                if u1 <= u2 <= u3:
                    val[comp] = (v[q] - v[q - 1]) / (u3 - u1) * (u2 - u1) + v[q - 1]
                    break
        st.append(val)
    n = len(st)
    if n == 1:
        u = np.full(deck.n_faces, st[0][0])
        v = np.full(deck.n_faces, st[0][1])
    else:
        x, y = a["x_node"], a["y_node"]
        dist = [np.sqrt((x - x[s - 1]) ** 2 + (y - y[s - 1]) ** 2) for s in w["station_node"]]
        if n == 2:
            r = [dist[1], dist[0]]
        else:
            r = [dist[1] * dist[2], dist[0] * dist[2], dist[0] * dist[1]]
        den = r[0] + r[1] if n == 2 else r[0] + r[1] + r[2]
        un = (r[0] * st[0][0] + r[1] * st[1][0]) if n == 2 else (r[0] * st[0][0] + r[1] * st[1][0] + r[2] * st[2][0])
        vn = (r[0] * st[0][1] + r[1] * st[1][1]) if n == 2 else (r[0] * st[0][1] + r[1] * st[1][1] + r[2] * st[2][1])
        un, vn = un / den, vn / den
        n1, n2 = a["nodenum_at_face"][:, 0] - 1, a["nodenum_at_face"][:, 1] - 1
        u = (un[n1] + un[n2]) * 0.5
        v = (vn[n1] + vn[n2]) * 0.5
    speed = np.sqrt(u * u + v * v)
    normal = u * a["cos_theta"] + v * a["sin_theta"]
    tangent = -u * a["sin_theta"] + v * a["cos_theta"]
    base, slope, lo = {1: (0.75, 0.067, 4.0), 2: (0.61, 0.063, 6.0), 3: (0.80, 0.065, 1.0)}[w["formular"]]
    f32 = np.float32
    cmin = 0.001 * float(f32(base) + f32(slope) * f32(lo))
    cmax = 0.001 * float(f32(base) + f32(slope) * f32(50.0))
    cda = np.minimum(np.maximum(0.001 * (base + slope * speed), cmin), cmax)
    per = w["spinup_period"] * 86400.0 if w["spinup"] == 1 else 0.0
    spin = math.tanh(2.0 * elapsed / per) if per > 0.0 and elapsed < per else 1.0   # the C library's tanh
    gamma = cda * (w["rho_a"] / deck.params.rho_o) * speed
    return gamma * normal * spin, gamma * tangent * spin, gamma


@pytest.mark.parametrize("n_stations,formular", [(1, 1), (2, 2), (3, 3), (3, 1)])
def test_station_wind_equals_host_restatement(oracle_so, n_stations, formular):
    """The wind stresses and Gamma_T the context forms from the station series equal the numpy
    restatement every step (spin-up on, the last station silent for its first hour), and a context
    fed that host forcing every step ends in the same state bit for bit."""
    from gom_release_gb300.series import with_station_wind

    deck = estuary(nx=14, ny=6, dx=100.0, n_layers=6, trans_sub_iter=2)
    deck.tide_spinup_days = 0.01
    bs = with_station_wind(from_synthetic(deck), deck, n_stations, formular=formular, spinup_days=0.02,
                           seed=n_stations)
    hf = HostForcing(deck)
    a, b = _pair(deck, oracle_so, hf)
    b.set_boundary_series(bs)
    dt = deck.params.dt
    steps = 6
    for it in range(1, steps + 1):
        f = hf.full(it) if it == 1 else hf.step(it)
        tn, tt, gt = _station_wind_host(deck, bs, hf.julian_day, it * dt)
        f.update(wind_stress_normal=tn, wind_stress_tangnt=tt, gamma_t=gt)
        a.set_forcing(f)
        a.step_all()
        b.step_all()
        for name, ref in (("wind_stress_normal", tn), ("wind_stress_tangnt", tt), ("gamma_t", gt)):
            got = b.get_field(name)
            assert np.array_equal(got, ref), (it, name, float(np.abs(got - ref).max()))
    assert float(np.abs(b.get_field("wind_stress_normal")).max()) > 0.0
    for name in STATE:
        assert np.array_equal(a.get_field(name), b.get_field(name)), name


def test_station_wind_argument_rules(oracle_so):
    from gom_release_gb300.series import with_station_wind

    deck = estuary(nx=8, ny=4, dx=100.0, n_layers=3, trans_sub_iter=1)
    c = GomCore(deck, lib_path=oracle_so)
    good = with_station_wind(from_synthetic(deck), deck, 2)
    bad = [replace(good, wind=dict(good.wind, flag=2)), replace(good, wind=dict(good.wind, formular=4)),
           replace(good, wind=dict(good.wind, station_node=[1, deck.n_nodes + 1])),
           replace(good, wind=dict(good.wind, rho_a=0.0)),
           replace(good, series=dict(good.series, wind_v=good.series["wind_v"][:1]))]
    for bs in bad:
        with pytest.raises(GomError) as e:
            c.set_boundary_series(bs)
        assert e.value.code == 1
    c.set_boundary_series(good)


# ----------------------------------------------------------------------------- hurricane frames
class _HurricaneHost:
    """read_hurricane_ser_1.f90:20-86 under main.f90:115-127 and the hurricane branch of
    calculate_wind_stress.f90:105-137, restated in numpy in the reference's order of operations."""

    def __init__(self, deck, bs):
        self.deck, self.h, self.w = deck, bs.hurricane, bs.wind
        self.frames = np.array(self.h["frames"], np.float64)        # (frame, component, node)
        self.face_u = np.zeros(deck.n_faces)
        self.face_v = np.zeros(deck.n_faces)
        self.next = None

    def step(self, it, julian_day):
        a = self.deck.geo
        w0, w1, w2 = self.frames
        if self.h["start_jday"] <= julian_day <= self.h["end_jday"]:
            if it % self.h["read_interval"] == 0:
                w0[:] = w2
                w1[:] = w2
                w2[:] = self.next
                self.next = None
            else:
                den = float(np.float32(self.h["read_interval"]))
                w1[:] = w1 + (w2 - w0) / den
            n1, n2 = a["nodenum_at_face"][:, 0] - 1, a["nodenum_at_face"][:, 1] - 1
            self.face_u = (w1[0][n1] + w1[0][n2]) * 0.5
            self.face_v = (w1[1][n1] + w1[1][n2]) * 0.5
        u, v = self.face_u, self.face_v
        speed = np.sqrt(u * u + v * v)
        normal = u * a["cos_theta"] + v * a["sin_theta"]
        tangent = -u * a["sin_theta"] + v * a["cos_theta"]
        base, slope = {1: (0.75, 0.067), 3: (0.80, 0.065)}.get(self.w["formular"], (0.61, 0.063))
        cda = np.minimum(float(np.float32(0.003)), 0.001 * (base + slope * speed))
        gamma = cda * (self.w["rho_a"] / self.deck.params.rho_o) * speed
        return dict(wind_stress_normal=gamma * normal, wind_stress_tangnt=gamma * tangent, gamma_t=gamma,
                    air_p=w1[2].copy())


@pytest.mark.parametrize("formular", [1, 2, 5])
def test_hurricane_frames_equal_host_restatement(oracle_so, formular):
    """Node frames every third step inside a window that opens after step 2 and closes after
    step 8 (the face winds then stay), frame 1 ramping from zero as read_hurricane_ser_0 leaves it:
    the stresses, Gamma_T and air pressure equal the numpy restatement every step, and a context
    fed that host forcing ends in the same state bit for bit."""
    from gom_release_gb300.series import with_hurricane_frames

    deck = estuary(nx=14, ny=6, dx=100.0, n_layers=6, trans_sub_iter=2)
    dt = deck.params.dt
    bs, records = with_hurricane_frames(from_synthetic(deck), deck, read_interval=3, n_records=6,
                                        start_jday=2.5 * dt / 86400.0, end_jday=8.5 * dt / 86400.0,
                                        formular=formular, seed=3)
    host = _HurricaneHost(deck, bs)
    hf = HostForcing(deck)
    a, b = _pair(deck, oracle_so, hf)
    b.set_boundary_series(bs)
    pending = list(records)
    for it in range(1, 12):
        f = hf.full(it) if it == 1 else hf.step(it)
        if it % 3 == 0 and 2.5 * dt / 86400.0 <= hf.julian_day <= 8.5 * dt / 86400.0:
            rec = pending.pop(0)
            b.push_hurricane_frame(rec)
            host.next = rec
        ref = host.step(it, hf.julian_day)
        f.update(ref)
        a.set_forcing(f)
        a.step_all()
        b.step_all()
        for name, val in ref.items():
            got = b.get_field(name)
            assert np.array_equal(got, val), (it, name, float(np.abs(got - val).max()))
    assert b.status().code == 0
    assert float(np.abs(b.get_field("wind_stress_normal")).max()) > 0.0
    for name in STATE:
        assert np.array_equal(a.get_field(name), b.get_field(name)), name


def test_hurricane_read_step_without_a_record(oracle_so):
    from gom_release_gb300.series import with_hurricane_frames

    deck = estuary(nx=8, ny=4, dx=100.0, n_layers=3, trans_sub_iter=1)
    bs, _ = with_hurricane_frames(from_synthetic(deck), deck, read_interval=2, n_records=3, start_jday=0.0,
                                  end_jday=1.0)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, initial_state(deck))
    c.set_forcing(HostForcing(deck).static())
    c.set_boundary_series(bs)
    c.step_all()
    assert c.status().code == 0
    try:
        c.step_all()          # step 2 reads a record that was never pushed
    except GomError:
        pass
    st = c.status()
    assert st.code == 1 and st.site == 34 and st.value == 2.0, (st.code, st.site, st.value)
    for bad in (dict(bs.hurricane, read_interval=0), dict(bs.hurricane, flag=2), dict(bs.hurricane, frames=None)):
        with pytest.raises(GomError):
            c.set_boundary_series(replace(bs, hurricane=bad))


class _Hurricane2Host(_HurricaneHost):
    """read_hurricane_ser_2.f90:19-146 with find_neighbour_nodes.f90 and IDW_5.f90 restated in
    numpy: the frames moved with the storm centre between reads."""

    FAR = float(np.float32(1.0e15))

    def __init__(self, deck, bs):
        super().__init__(deck, bs)
        self.track = list(bs.hurricane["track"])
        self.next_center = None
        x, y = deck.geo["x_node"], deck.geo["y_node"]
        self.lists = []
        for i in range(len(x)):
            d = np.sqrt((x[i] - x) * (x[i] - x) + (y[i] - y) * (y[i] - y))
            d[i] = self.FAR
            md = d.min()
            rng = 20000.0 if md < 5000 else md * 4
            self.lists.append(np.nonzero(d <= rng)[0])

    def idw5(self, i, xn, yn, v):
        x, y = self.deck.geo["x_node"], self.deck.geo["y_node"]
        lst = self.lists[i]
        d = np.sqrt((xn - x[lst]) * (xn - x[lst]) + (yn - y[lst]) * (yn - y[lst]))
        sel, md = [], []
        for _ in range(3):
            ii = int(np.argmin(d))
            sel.append(lst[ii])
            md.append(d[ii])
            d[ii] = self.FAR
        r1, r2, r3 = md[1] * md[2], md[0] * md[2], md[0] * md[1]
        return (r1 * v[:, sel[0]] + r2 * v[:, sel[1]] + r3 * v[:, sel[2]]) / (r1 + r2 + r3)

    def step(self, it, julian_day):
        h = self.h
        w0, w1, w2 = self.frames
        inside = h["start_jday"] <= julian_day <= h["end_jday"]
        if inside and it % h["read_interval"] != 0:
            t = self.track
            tr = (julian_day - t[2]) / (t[5] - t[2])
            dx, dy = t[3] - t[0], t[4] - t[1]
            t[0], t[1] = t[0] + dx * tr, t[1] + dy * tr
            t[2] = t[2] + self.deck.params.dt / 86400.0
            x, y = self.deck.geo["x_node"], self.deck.geo["y_node"]
            new = np.empty_like(w1)
            for i in range(len(x)):
                a = self.idw5(i, x[i] - dx * tr, y[i] - dy * tr, w1)
                b = self.idw5(i, x[i] + dx * (1.0 - tr), y[i] + dy * (1.0 - tr), w2)
                new[:, i] = (1.0 - tr) * a + tr * b
            w1[:] = new
            a = self.deck.geo
            n1, n2 = a["nodenum_at_face"][:, 0] - 1, a["nodenum_at_face"][:, 1] - 1
            self.face_u = (w1[0][n1] + w1[0][n2]) * 0.5
            self.face_v = (w1[1][n1] + w1[1][n2]) * 0.5
            return self.stress(w1)
        if inside:
            t = self.track
            t[0], t[1] = t[3], t[4]
            t[3], t[4], t[5] = self.next_center
        return super().step(it, julian_day)

    def stress(self, w1):
        a = self.deck.geo
        u, v = self.face_u, self.face_v
        speed = np.sqrt(u * u + v * v)
        normal = u * a["cos_theta"] + v * a["sin_theta"]
        tangent = -u * a["sin_theta"] + v * a["cos_theta"]
        base, slope = {1: (0.75, 0.067), 3: (0.80, 0.065)}.get(self.w["formular"], (0.61, 0.063))
        cda = np.minimum(float(np.float32(0.003)), 0.001 * (base + slope * speed))
        gamma = cda * (self.w["rho_a"] / self.deck.params.rho_o) * speed
        return dict(wind_stress_normal=gamma * normal, wind_stress_tangnt=gamma * tangent, gamma_t=gamma,
                    air_p=w1[2].copy())


def test_hurricane_method2_equals_host_restatement(oracle_so):
    """Method 2 (read_hurricane_ser_2.f90): frames moved with the storm centre through IDW_5 over
    find_neighbour_nodes' lists and blended, centres pushed with the frames; stresses, Gamma_T and
    air pressure equal the numpy restatement every step, and a context fed that host forcing ends in
    the same state bit for bit."""
    from gom_release_gb300.series import hurricane_centers, with_hurricane_frames

    deck = estuary(nx=12, ny=5, dx=100.0, n_layers=5, trans_sub_iter=2)
    dt = deck.params.dt
    rec_days = 3 * dt / 86400.0
    bs, records = with_hurricane_frames(from_synthetic(deck), deck, read_interval=3, n_records=5, start_jday=0.0,
                                        end_jday=1.0, seed=7, interp_method=2, record_days=rec_days)
    centers = hurricane_centers(deck, 5, 0.0, rec_days)
    host = _Hurricane2Host(deck, bs)
    hf = HostForcing(deck)
    a, b = _pair(deck, oracle_so, hf)
    b.set_boundary_series(bs)
    pending, pending_c = list(records), list(centers)
    for it in range(1, 10):
        f = hf.full(it) if it == 1 else hf.step(it)
        if it % 3 == 0:
            rec, cen = pending.pop(0), pending_c.pop(0)
            b.push_hurricane_frame(rec)
            b.push_hurricane_center(*cen)
            host.next, host.next_center = rec, cen
        ref = host.step(it, hf.julian_day)
        f.update(ref)
        a.set_forcing(f)
        a.step_all()
        b.step_all()
        for name, val in ref.items():
            got = b.get_field(name)
            assert np.array_equal(got, val), (it, name, float(np.abs(got - val).max()))
    assert b.status().code == 0
    for name in STATE:
        assert np.array_equal(a.get_field(name), b.get_field(name)), name


# ----------------------------------------------------------------------------- heat balance
def _local_hour(year, state, jday):
    """julian_to_localtime.f90:16-86 with its saved month table (state: [month, table set])."""
    leap = [0, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335]
    normal = [0, 31, 59, 90, 120, 151, 181, 212, 243, 273, 304, 334]
    leap_top = [31, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335]
    normal_top = [31, 59, 90, 120, 151, 181, 212, 243, 273, 304, 334]
    if year % 4 == 0:
        if year != 1900 and state[0] >= 3:
            state[0] = 1 + sum(1 for t in leap_top if jday > t)
            state[1] = 1
        m = float(leap[state[0] - 1]) if state[1] else 0.0
    else:
        state[0] = 1 + sum(1 for t in normal_top if jday > t)
        m = float(normal[state[0] - 1])
    day_temp = jday - m
    day = int(day_temp) + 1
    return int((day_temp + 1 - day) * 24.0)


def _solar_short_wave(h, julian_day, c2, f32, state):
    """heat_term_by_term.f90:64-83 (sol_swr 1): the sun's elevation at the local hour; 0 below the
    horizon (the reference leaves the term unset there)."""
    hr = _local_hour(h["year"], state, julian_day)
    pi = 3.141592653589793
    deg2rad, rad2deg = pi / 180.0, 180.0 / pi
    j_day = julian_day + 1
    tau_d = 2.0 * pi * float(int(j_day + 1) - 1) / 365.0
    sdec = (f32(0.006918) - f32(0.399912) * math.cos(tau_d) + f32(0.070257) * math.sin(tau_d)
            - f32(0.006758) * math.cos(2.0 * tau_d) + f32(0.000907) * math.sin(2.0 * tau_d)
            - f32(0.002697) * math.cos(3.0 * tau_d) + f32(0.001480) * math.sin(3.0 * tau_d))
    eqt = (f32(0.170) * math.sin(4.0 * pi * float(int(j_day) - 80) / 373.0)
           - f32(0.129) * math.sin(2.0 * pi * float(int(j_day) - 8) / 355.0))
    sm = 15.0 * float(int(h["lon"] / 15.0))
    lha = f32(0.261799) * (float(hr) - (h["lon"] - sm) * f32(0.0666667) + eqt - 12.0)
    a0 = math.asin(math.sin(h["lat"] * deg2rad) * math.sin(sdec)
                   + math.cos(h["lat"] * deg2rad) * math.cos(sdec) * math.cos(lha)) * rad2deg
    if not a0 > 0.0:
        return 0.0
    a2 = a0 * a0
    a3, a4 = a2 * a0, a2 * a2
    poly = f32(2.0444) * a0 + f32(0.1296) * a2 - f32(1.941e-3) * a3 + f32(7.591e-6) * a4
    return (1.0 - f32(0.65) * c2) * 24.0 * poly * f32(0.1314)


def _heat_host(deck, bs, julian_day, temp, dz, top, state=None):
    """heat_term_by_term.f90:27-156 (sol_swr 2) restated with Python floats and the C library's
    exp / log / pow (as the oracle calls them): (phi_sz (L, NC), phi_sw (NC)) of one step from the
    temperatures and thicknesses at the step's start and the tops after its layer update."""
    h = bs.heat
    f32 = lambda x: float(np.float32(x))
    rdd = float(np.float32(bs.reference_diff_days) * np.float32(86400.0))
    u2 = julian_day * 86400.0
    t, av = np.asarray(h["air_time"]), np.asarray(h["air_values"])
    v = [0.0] * 5
    for q in range(1, len(t)):
        u1, u3 = float(t[q - 1]) - rdd, float(t[q]) - rdd
        if u1 <= u2 <= u3:
            v = [(u2 - u1) * (float(av[c, q]) - float(av[c, q - 1])) / (u3 - u1) + float(av[c, q - 1]) for c in range(5)]
            break
    ta, tdew, ws, sol, cloud = v
    c2 = cloud * cloud
    if h["sol_swr"] == 1:
        phi_sn = _solar_short_wave(h, julian_day, c2, f32, state)
    else:
        phi_sn = (1.0 - f32(0.65) * c2) * sol
    xa = ta + 273.15
    if ta >= 5.0:
        x3 = xa * xa * xa
        phi_ac = f32(5.31e-13) * (x3 * x3)
    else:
        x2 = xa * xa
        phi_ac = f32(5.67e-8) * (x2 * x2) * (1.0 - f32(0.261) * math.exp(-(f32(7.77e-4) * (ta * ta))))
    phi_an = phi_ac * (1.0 + f32(0.17) * c2) * 0.97
    z0 = f32(0.001) if ws <= f32(2.3) else f32(0.005)
    alpha = math.log(h["wind_height"] / z0) / math.log(2.0 / z0)
    fwz = h["fwz_a"] + h["fwz_b"] / math.pow(alpha, h["fwz_c"]) * math.pow(ws, h["fwz_c"])
    ea = math.exp(2.3026 * (7.5 * tdew / (tdew + 237.3) + f32(0.6609)))
    L, nc = deck.n_layers, deck.n_cells
    bottom = deck.geo["bottom_layer_at_element"]
    phi_sz = np.zeros((nc, L))
    phi_sw = np.zeros(nc)
    for i in range(nc):
        tl, b = int(top[i]), int(bottom[i])
        if tl == 0:
            continue
        tw = float(temp[tl - 1, i])
        xw = tw + f32(273.15)
        x2 = xw * xw
        phi_br = float(np.float32(np.float32(0.97) * np.float32(5.67e-8))) * (x2 * x2)
        if tw < 0.0:
            es = math.exp(2.3026 * (9.5 * tw / (tw + 265.5) + f32(0.6609)))
        else:
            es = math.exp(2.3026 * (7.5 * tw / (tw + 237.3) + f32(0.6609)))
        phi_n = phi_sn + phi_an - phi_br - fwz * (es - ea) - 0.47 * fwz * (tw - ta)
        sw = h["sed_water_exchange"] * (h["t_sed"] - float(temp[b - 1, i]))
        phi_sw[i] = sw
        sol_out = (1.0 - h["sol_absorb"]) * phi_sn * math.exp(-(h["light_extinction"] * float(dz[tl - 1, i])))
        phi_sz[i, tl - 1] = phi_n - sol_out
        for k in range(tl - 1, b - 1, -1):
            sol_in = sol_out
            sol_out = sol_in * math.exp(-(h["light_extinction"] * float(dz[k - 1, i])))
            phi_sz[i, k - 1] = sol_in - sol_out
        for k in range(b, tl + 1):
            phi_sz[i, k - 1] = phi_sz[i, k - 1] + sol_out * h["sed_temp_coeff"]
            phi_sz[i, k - 1] = phi_sz[i, k - 1] + sw
    return phi_sz, phi_sw


def test_heat_balance_equals_host_restatement(oracle_so):
    """heat_term_by_term (sol_swr 2) formed by the context before every transport equals the Python
    restatement on the same state bit for bit (both on the C library's exp, log and pow)."""
    from gom_release_gb300.series import with_heat_balance

    deck = estuary(nx=12, ny=5, dx=100.0, n_layers=5, trans_sub_iter=2)
    deck = replace(deck, params=replace(deck.params, heat_option=1))
    bs = with_heat_balance(from_synthetic(deck), hours=6, seed=4)
    hf = HostForcing(deck)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, initial_state(deck))
    c.set_forcing(hf.static())
    c.set_boundary_series(bs)
    L, nc = deck.n_layers, deck.n_cells
    jd = 0.0
    for it in range(1, 7):
        temp = c.get_field("temp_cell").reshape(nc, L).T.copy()
        dz = c.get_field("dz_cell").reshape(nc, L).T.copy()
        c.step_all()
        jd = jd + deck.params.dt / 86400.0
        top = c.get_field("top_layer_cell")
        sz, sw = _heat_host(deck, bs, jd, temp, dz, top)
        got_sz = c.get_field("phi_sz").reshape(nc, L)
        wet = top > 0
        assert np.array_equal(c.get_field("phi_sw")[wet], sw[wet]), it
        for i in np.nonzero(wet)[0]:
            b = int(deck.geo["bottom_layer_at_element"][i])
            assert np.array_equal(got_sz[i, b - 1:top[i]], sz[i, b - 1:top[i]]), (it, i)
    assert float(np.abs(c.get_field("phi_sz")).max()) > 0.0


def test_heat_balance_argument_rules(oracle_so):
    from gom_release_gb300.series import with_heat_balance

    deck = estuary(nx=8, ny=4, dx=100.0, n_layers=3, trans_sub_iter=1)       # heat_option 2
    c = GomCore(deck, lib_path=oracle_so)
    with pytest.raises(GomError):
        c.set_boundary_series(with_heat_balance(from_synthetic(deck)))
    deck1 = replace(deck, params=replace(deck.params, heat_option=1))
    c1 = GomCore(deck1, lib_path=oracle_so)
    for bad in (dict(sol_swr=3), dict(sol_swr=1, month=13)):
        with pytest.raises(GomError):
            c1.set_boundary_series(with_heat_balance(from_synthetic(deck1), **bad))
    c1.set_boundary_series(with_heat_balance(from_synthetic(deck1)))


def test_mobile_bay_heat_balance_equals_host_restatement(oracle_so):
    """The reference's Mobile Bay deck with its own air series and heat cards (heat_option 1,
    sol_swr 2): the heat terms the context forms equal the Python restatement bit for bit."""
    data = DeckData.from_npz(FIXTURE)
    deck = deck_from_data(data)
    bs = from_deck_data(deck, heat=True)
    assert bs.heat["air_values"].shape == (5, 961)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, initial_state(deck))
    c.set_forcing(SeriesForcing(deck).static())
    c.set_boundary_series(bs)
    L, nc = deck.n_layers, deck.n_cells
    jd = bs.julian_day
    for it in range(1, 3):
        temp = c.get_field("temp_cell").reshape(nc, L).T.copy()
        dz = c.get_field("dz_cell").reshape(nc, L).T.copy()
        c.step_all()
        jd = jd + deck.params.dt / 86400.0
        top = c.get_field("top_layer_cell")
        sz, sw = _heat_host(deck, bs, jd, temp, dz, top)
        wet = top > 0
        assert np.array_equal(c.get_field("phi_sw")[wet], sw[wet]), it
        got = c.get_field("phi_sz").reshape(nc, L)
        bottom = deck.geo["bottom_layer_at_element"]
        for i in np.nonzero(wet)[0]:
            assert np.array_equal(got[i, bottom[i] - 1:top[i]], sz[i, bottom[i] - 1:top[i]]), (it, i)
    assert float(np.abs(c.get_field("phi_sz")).max()) > 0.0


@pytest.mark.parametrize("year,month", [(2005, 7), (2004, 7), (2004, 1)])
def test_heat_balance_solar_elevation_equals_host_restatement(oracle_so, year, month):
    """sol_swr 1: the short-wave term from the sun's elevation at the local hour of
    julian_to_localtime (a common year; a leap year from July, with the leap month table; a leap
    year from January, whose saved table stays zero) equals the Python restatement bit for bit
    over the hour of sunrise (the local hour turns from 4 to 5 half-way)."""
    from gom_release_gb300.series import with_heat_balance

    deck = estuary(nx=10, ny=4, dx=100.0, n_layers=4, trans_sub_iter=1)
    deck = replace(deck, params=replace(deck.params, heat_option=1))
    bs = with_heat_balance(replace(from_synthetic(deck), julian_day=190.19), hours=3, seed=2, sol_swr=1,
                           year=year, month=month)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, initial_state(deck))
    c.set_forcing(HostForcing(deck).static())
    c.set_boundary_series(bs)
    L, nc = deck.n_layers, deck.n_cells
    state = [month, 0]
    jd = bs.julian_day
    seen_day = seen_night = False
    for it in range(1, 61):
        temp = c.get_field("temp_cell").reshape(nc, L).T.copy()
        dz = c.get_field("dz_cell").reshape(nc, L).T.copy()
        c.step_all()
        jd = jd + deck.params.dt / 86400.0
        top = c.get_field("top_layer_cell")
        sz, sw = _heat_host(deck, bs, jd, temp, dz, top, state)
        got = c.get_field("phi_sz").reshape(nc, L)
        bottom = deck.geo["bottom_layer_at_element"]
        for i in np.nonzero(top > 0)[0]:
            assert np.array_equal(got[i, bottom[i] - 1:top[i]], sz[i, bottom[i] - 1:top[i]]), (it, i)
        sun = _solar_short_wave(bs.heat, jd, 0.0, lambda x: float(np.float32(x)), list(state))
        seen_day = seen_day or sun > 0.0
        seen_night = seen_night or sun == 0.0
    assert seen_day and seen_night
