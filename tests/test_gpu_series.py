"""Boundary series evaluated on the device (gom_set_boundary_series) against the CPU oracle's
restatement and against host forcing: on the reference's Mobile Bay deck (elevation, discharge,
salinity and temperature series, linear and Lagrange discharge) the device forcing equals the
oracle's bit for bit every step; on a synthetic estuary with a harmonic tide and spin-up it agrees
to the last bits of cos and tanh (CUDA's and the C library's differ by an ulp or two); the
interior-mean boundary (type -1) bit for bit; the captured step graph runs the series."""
from pathlib import Path

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, GomError, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state
from gom_release_gb300.gom_inputs import DeckData, SeriesForcing, deck_from_data
from gom_release_gb300.series import from_deck_data, from_synthetic

pytestmark = pytest.mark.gpu

FIXTURE = Path(__file__).resolve().parent / "golden" / "mobile_bay.npz"
FIELD_RTOL = 1e-9      # after a run, relative to the field's largest magnitude
TIDE_ATOL = 1e-14      # metres: cos / tanh of CUDA against the C library, tide of 0.6 m


def _close(a, b, rtol=FIELD_RTOL):
    scale = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a - b).max()) / scale < rtol


def _ctx(deck, st, **lib):
    c = GomCore(deck, **lib)
    prepare(c, st)
    return c


@pytest.mark.parametrize("q_method", [1, 2])
def test_mobile_bay_device_series_equal_oracle(oracle_so, gpu_lib, q_method):
    data = DeckData.from_npz(FIXTURE)
    data.cards = dict(data.cards, q_interp_method=float(q_method))
    deck = deck_from_data(data)
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    static = SeriesForcing(deck).static()
    bs = from_deck_data(deck)
    for c in (ref, gpu):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    for it in range(1, 11):
        ref.step_all()
        gpu.step_all()
        for name in ("eta_at_ob_old", "eta_at_ob_new", "q_add"):
            a, b = gpu.get_field(name), ref.get_field(name)
            assert np.array_equal(a, b), (it, name, float(np.abs(a - b).max()))
    for name in ("eta_cell", "un_face", "salt_cell", "temp_cell"):
        assert _close(gpu.get_field(name), ref.get_field(name)), name


def test_mobile_bay_device_series_equal_host_series(gpu_lib):
    """The same GPU path with the series on the device and with the host forcing every step."""
    deck = deck_from_data(DeckData.from_npz(FIXTURE))
    st = initial_state(deck)
    host = _ctx(deck, st, lib=gpu_lib)
    dev = _ctx(deck, st, lib=gpu_lib)
    f = SeriesForcing(deck)
    dev.set_forcing(f.static())
    dev.set_boundary_series(from_deck_data(deck))
    for it in range(1, 11):
        host.set_forcing(f.full(it) if it == 1 else f.step(it))
        host.step_all()
        dev.step_all()
    for name in ("eta_cell", "un_face", "salt_cell", "temp_cell", "eta_at_ob_new", "q_add"):
        assert np.array_equal(host.get_field(name), dev.get_field(name)), name


def test_estuary_harmonic_series(oracle_so, gpu_lib):
    deck = estuary(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=3)
    deck.tide_spinup_days = 0.01
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    hf = HostForcing(deck)
    bs = from_synthetic(deck)
    for c in (ref, gpu):
        c.set_forcing(hf.static())
        c.set_boundary_series(bs)
    for it in range(1, 21):
        ref.step_all()
        gpu.step_all()
        for name in ("eta_at_ob_old", "eta_at_ob_new"):
            err = float(np.abs(gpu.get_field(name) - ref.get_field(name)).max())
            assert err < TIDE_ATOL, (it, name, err)
        assert np.array_equal(gpu.get_field("q_add"), ref.get_field("q_add"))
    for name in ("eta_cell", "un_face", "salt_cell", "temp_cell"):
        assert _close(gpu.get_field(name), ref.get_field(name), 1e-8), name


def test_interior_mean_boundary_equals_oracle(oracle_so, gpu_lib):
    deck = estuary(nx=16, ny=8, dx=100.0, n_layers=4, trans_sub_iter=2)
    st = initial_state(deck)
    st["eta_cell"] = np.random.default_rng(3).uniform(-0.2, 0.2, deck.n_cells)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    bs = from_synthetic(deck)
    bs.ob_eta_type = np.full(deck.n_ob, -1, np.int32)
    f = HostForcing(deck).full(1)
    for c in (ref, gpu):
        c.set_forcing(f)
        c.set_boundary_series(bs)
        c.step_all()
    assert np.array_equal(gpu.get_field("eta_at_ob_old"), ref.get_field("eta_at_ob_old"))
    assert np.array_equal(gpu.get_field("eta_at_ob_new"), ref.get_field("eta_at_ob_new"))


def test_graph_launch_runs_the_series(gpu_lib):
    """step_launch / step_wait (the captured graph) and step_all advance the same clock."""
    deck = estuary(nx=20, ny=8, dx=100.0, n_layers=6, trans_sub_iter=2)
    deck.tide_spinup_days = 0.01
    st = initial_state(deck)
    a = _ctx(deck, st, lib=gpu_lib)
    b = _ctx(deck, st, lib=gpu_lib)
    hf = HostForcing(deck)
    for c in (a, b):
        c.set_forcing(hf.static())
        c.set_boundary_series(from_synthetic(deck))
    for _ in range(8):
        a.step_all()
        b.step_launch()
        b.step_wait()
    for name in ("eta_at_ob_new", "eta_cell", "salt_cell"):
        assert np.array_equal(a.get_field(name), b.get_field(name)), name


def test_argument_rules_and_storm_exclusion(gpu_lib):
    deck = estuary(nx=8, ny=4, dx=100.0, n_layers=3, trans_sub_iter=1)
    c = GomCore(deck, lib=gpu_lib)
    bs = from_synthetic(deck)
    bad = from_synthetic(deck)
    bad.qb_q_id = np.full(deck.n_qb, 9, np.int32)
    with pytest.raises(GomError):
        c.set_boundary_series(bad)
    c.set_boundary_series(bs)
    with pytest.raises(GomError):
        c.set_storms([object()])


@pytest.mark.parametrize("n_stations,spinup_days", [(1, 0.0), (2, 0.0), (3, 0.0), (3, 0.02)])
def test_station_wind_equals_oracle(oracle_so, gpu_lib, n_stations, spinup_days):
    """Station wind (get_windp_at_face.f90, IDW_windp_ser.f90, calculate_wind_stress.f90) formed on
    the device equals the oracle's bit for bit without spin-up (sqrt and division are correctly
    rounded on both); with the wind spin-up on, CUDA's tanh may differ from the C library's in
    the last bit."""
    from gom_release_gb300.series import with_station_wind

    deck = estuary(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=3)
    deck.tide_spinup_days = 0.01
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    bs = with_station_wind(from_synthetic(deck), deck, n_stations, formular=n_stations, spinup_days=spinup_days,
                           seed=10 + n_stations)
    static = HostForcing(deck).static()
    for c in (ref, gpu):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    for it in range(1, 11):
        ref.step_all()
        gpu.step_all()
        for name in ("wind_stress_normal", "wind_stress_tangnt", "gamma_t"):
            a, b = gpu.get_field(name), ref.get_field(name)
            if spinup_days == 0.0:
                assert np.array_equal(a, b), (it, name, float(np.abs(a - b).max()))
            else:
                assert float(np.abs(a - b).max()) <= 4e-16 * float(np.abs(b).max()), (it, name)
    assert float(np.abs(gpu.get_field("wind_stress_normal")).max()) > 0.0
    for name in ("eta_cell", "un_face", "salt_cell", "temp_cell"):
        assert _close(gpu.get_field(name), ref.get_field(name)), name


def _hurricane_case(deck, formular=1):
    from gom_release_gb300.series import with_hurricane_frames

    dt = deck.params.dt
    start, end = 2.5 * dt / 86400.0, 14.5 * dt / 86400.0
    bs, records = with_hurricane_frames(from_synthetic(deck), deck, read_interval=4, n_records=6, start_jday=start,
                                        end_jday=end, formular=formular, seed=5)
    read_steps = [it for it in range(1, 19) if it % 4 == 0 and start <= it * dt / 86400.0 <= end]
    return bs, dict(zip(read_steps, records))


@pytest.mark.parametrize("formular", [1, 3])
def test_hurricane_frames_equal_oracle(oracle_so, gpu_lib, formular):
    """Hurricane node frames (read_hurricane_ser_1.f90, calculate_wind_stress.f90:105-137) on the
    device equal the oracle's bit for bit every step: ramps between reads, reads inside the
    window, face winds kept after it closes."""
    deck = estuary(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=3)
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    bs, pushes = _hurricane_case(deck, formular)
    static = HostForcing(deck).static()
    for c in (ref, gpu):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    for it in range(1, 19):
        if it in pushes:
            ref.push_hurricane_frame(pushes[it])
            gpu.push_hurricane_frame(pushes[it])
        ref.step_all()
        gpu.step_all()
        for name in ("wind_stress_normal", "wind_stress_tangnt", "gamma_t", "air_p"):
            a, b = gpu.get_field(name), ref.get_field(name)
            assert np.array_equal(a, b), (it, name, float(np.abs(a - b).max()))
    assert gpu.status().code == 0
    for name in ("eta_cell", "un_face", "salt_cell", "temp_cell"):
        assert _close(gpu.get_field(name), ref.get_field(name)), name


def test_hurricane_records_pushed_between_graph_launches(gpu_lib):
    """Records pushed while earlier captured steps still run are taken at their read step: the
    launched run ends where the synchronous one does, bit for bit."""
    deck = estuary(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=3)
    st = initial_state(deck)
    sync = _ctx(deck, st, lib=gpu_lib)
    lau = _ctx(deck, st, lib=gpu_lib)
    bs, pushes = _hurricane_case(deck)
    static = HostForcing(deck).static()
    for c in (sync, lau):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    for it in range(1, 19):
        if it in pushes:
            sync.push_hurricane_frame(pushes[it])
            lau.push_hurricane_frame(pushes[it])
        sync.step_all()
        lau.step_launch()
    lau.step_wait()
    for name in ("eta_cell", "un_face", "wind_stress_normal", "air_p", "salt_cell"):
        assert np.array_equal(lau.get_field(name), sync.get_field(name)), name


def test_hurricane_method2_equals_oracle(oracle_so, gpu_lib):
    """Method 2 (read_hurricane_ser_2.f90 with IDW_5.f90 over find_neighbour_nodes' lists, built on
    the device) equals the oracle bit for bit every step: the nearest three nodes, their weights
    and the blend of the two moved frames."""
    from gom_release_gb300.series import hurricane_centers, with_hurricane_frames

    deck = estuary(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=3)
    dt = deck.params.dt
    rec_days = 4 * dt / 86400.0
    bs, records = with_hurricane_frames(from_synthetic(deck), deck, read_interval=4, n_records=6, start_jday=0.0,
                                        end_jday=1.0, seed=9, interp_method=2, record_days=rec_days)
    centers = hurricane_centers(deck, 6, 0.0, rec_days)
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    static = HostForcing(deck).static()
    for c in (ref, gpu):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    for it in range(1, 17):
        if it % 4 == 0:
            k = it // 4 - 1
            for c in (ref, gpu):
                c.push_hurricane_frame(records[k])
                c.push_hurricane_center(*centers[k])
        ref.step_all()
        gpu.step_all()
        for name in ("wind_stress_normal", "wind_stress_tangnt", "gamma_t", "air_p"):
            a, b = gpu.get_field(name), ref.get_field(name)
            assert np.array_equal(a, b), (it, name, float(np.abs(a - b).max()))
    assert gpu.status().code == 0 and ref.status().code == 0
    for name in ("eta_cell", "un_face", "salt_cell", "temp_cell"):
        assert _close(gpu.get_field(name), ref.get_field(name)), name


@pytest.mark.parametrize("precision", [0, 1])
def test_heat_balance_equals_oracle(oracle_so, gpu_lib, precision):
    """heat_term_by_term (sol_swr 2) on the device against the oracle: phi_sz and phi_sw of every
    step within the last bits of CUDA's exp, log and pow against the C library's (1e-12 of the
    field's magnitude; FP64 context), and the temperatures after the run; the mixed context reads
    FP32 temperatures and thicknesses (1e-4)."""
    import dataclasses

    from gom_release_gb300.series import with_heat_balance

    deck = estuary(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=3)
    deck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, heat_option=1))
    bs = with_heat_balance(from_synthetic(deck), hours=6, seed=6, sed_temp_coeff=0.3)
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    dg = dataclasses.replace(deck, params=dataclasses.replace(deck.params, precision=precision))
    gpu = _ctx(dg, st, lib=gpu_lib)
    static = HostForcing(deck).static()
    for c in (ref, gpu):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    tol = 1e-12 if precision == 0 else 1e-4
    for it in range(1, 11):
        ref.step_all()
        gpu.step_all()
        for name in ("phi_sz", "phi_sw"):
            a, b = gpu.get_field(name), ref.get_field(name)
            scale = max(float(np.abs(b).max()), 1e-30)
            assert float(np.abs(a - b).max()) <= tol * scale, (it, name, float(np.abs(a - b).max()) / scale)
    assert gpu.status().code == 0
    assert _close(gpu.get_field("temp_cell"), ref.get_field("temp_cell"), rtol=1e-9 if precision == 0 else 1e-4)


def test_mobile_bay_heat_balance_equals_oracle(oracle_so, gpu_lib):
    """The reference's Mobile Bay deck with its boundary series, air series and heat cards all on
    the device: phi_sz / phi_sw within the last bits of CUDA's transcendental functions of the
    oracle's every step, the temperatures after ten steps within 1e-9."""
    deck = deck_from_data(DeckData.from_npz(FIXTURE))
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    bs = from_deck_data(deck, heat=True)
    static = SeriesForcing(deck).static()
    for c in (ref, gpu):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    for it in range(1, 11):
        ref.step_all()
        gpu.step_all()
        for name in ("phi_sz", "phi_sw"):
            a, b = gpu.get_field(name), ref.get_field(name)
            scale = max(float(np.abs(b).max()), 1e-30)
            assert float(np.abs(a - b).max()) <= 1e-12 * scale, (it, name)
    assert gpu.status().code == 0
    for name in ("temp_cell", "salt_cell", "eta_cell"):
        assert _close(gpu.get_field(name), ref.get_field(name)), name


def test_heat_balance_solar_elevation_equals_oracle(oracle_so, gpu_lib):
    """sol_swr 1 on the device: the local hour of julian_to_localtime (integer arithmetic, the same
    on both) and the sun's elevation through CUDA's sin, cos and asin, across the hour of sunrise:
    phi_sz / phi_sw within 1e-12 of the oracle's every step."""
    import dataclasses

    from gom_release_gb300.series import with_heat_balance

    deck = estuary(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=3)
    deck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, heat_option=1))
    bs = with_heat_balance(dataclasses.replace(from_synthetic(deck), julian_day=190.19), hours=3, seed=3,
                           sol_swr=1, year=2004, month=7)
    st = initial_state(deck)
    ref = _ctx(deck, st, lib_path=oracle_so)
    gpu = _ctx(deck, st, lib=gpu_lib)
    static = HostForcing(deck).static()
    for c in (ref, gpu):
        c.set_forcing(static)
        c.set_boundary_series(bs)
    for it in range(1, 61):
        ref.step_all()
        gpu.step_all()
        if it % 5 == 0 or 28 <= it <= 32:
            for name in ("phi_sz", "phi_sw"):
                a, b = gpu.get_field(name), ref.get_field(name)
                scale = max(float(np.abs(b).max()), 1e-30)
                assert float(np.abs(a - b).max()) <= 1e-12 * scale, (it, name)
    assert gpu.status().code == 0
