"""Boundary series held by the context (gom_set_boundary_series), on the CPU oracle: the forcing
it forms at the start of every step equals the host forcing GOM's driver computes
(setup_spinup.f90, compute_boundary_eta.f90, calculate_Q.f90, the boundary-concentration
interpolation of solve_transport_equation_v19.f90), bit for bit, on the reference's Mobile Bay deck
(elevation series, linear and Lagrange discharge, salinity / temperature series, 30 subcycles)
and on a synthetic estuary (harmonic tide with spin-up, constant river and boundary tracers); the
interior-mean open boundary (type -1) by hand; and the argument rules."""
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
