"""The reference's own deck (Mobile Bay: 35,127 irregular triangles, 5 z-levels, 75 open-boundary
cells forced by elevation series, a river, salinity and temperature series) read from the
committed fixture, built into a Deck and stepped by the CPU oracle.  The fixture is pinned against
the reference's files where they are mounted."""
from pathlib import Path

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, prepare
from gom_release_gb300.deck import initial_state
from gom_release_gb300.gom_inputs import DeckData, SeriesForcing, deck_from_data, julian_day0, read_deck, \
    reference_diff_days

FIXTURE = Path(__file__).resolve().parent / "golden" / "mobile_bay.npz"
REF_DECK = Path("/root/reference/GOM_Rv1.1.0/Projects/MB_test/2_baroclinic_test/input")


def _deck():
    return deck_from_data(DeckData.from_npz(FIXTURE))


def test_fixture_matches_the_reference_files():
    if not REF_DECK.exists():
        pytest.skip("the reference deck is not mounted here")
    a = read_deck(REF_DECK, overrides={"hurricane_flag": 0.0})
    b = DeckData.from_npz(FIXTURE)
    for k in ("x", "y", "h", "tri_or_quad", "cells", "z_level", "ob", "qb", "salt_init", "temp_init"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert a.cards == b.cards
    for kind in a.series:
        for ta, tb in zip(a.series[kind][0], b.series[kind][0]):
            assert np.array_equal(ta, tb), kind
        for va, vb in zip(a.series[kind][1], b.series[kind][1]):
            assert np.array_equal(va, vb), kind


def test_deck_geometry_and_boundaries():
    d = _deck()
    assert (d.n_nodes, d.n_cells, d.n_layers, d.n_ob, d.n_qb) == (18718, 35127, 5, 75, 1)
    g = d.geo
    assert np.all(g["area"] > 0) and np.all(g["tri_or_quad"] == 3)
    # every face is shared by at most two cells and every interior face twice
    assert d.n_faces == int((g["adj_cellnum_at_face"][:, 1] != 0).sum() + (g["adj_cellnum_at_face"][:, 1] == 0).sum())
    assert np.count_nonzero(g["boundary_type_of_face"] > 0) == 75
    assert np.count_nonzero(g["isflowside3"] > 0) == 1
    # voronoi 0: centres are centroids
    c = g["nodenum_at_cell"][:, :3] - 1
    assert np.array_equal(g["x_cell"], (g["x_node"][c[:, 0]] + g["x_node"][c[:, 1]] + g["x_node"][c[:, 2]]) / 3)
    # Manning's n, uniform
    assert np.all(g["manning"] == 0.01)


def test_series_forcing_interpolates_as_the_reference():
    """compute_boundary_eta.f90:100-124 on the fixture's series, by hand: julian day 212 of 2010
    (1 August) plus the step, against series times shifted by reference_diff_days = -212."""
    d = _deck()
    data = d.meta["reference"]
    assert julian_day0(data.cards) == 212.0 and reference_diff_days(data.cards) == -212
    f = SeriesForcing(d)
    out = f.step(1)
    t, v = data.series["eta"][0][0], data.series["eta"][1][0]
    tt = t - float(np.float32(-212) * np.float32(86400.0))   # series times in model time
    u2 = (212.0 + 150.0 / 86400.0) * 86400.0                  # julian_day * 86400 after one step
    k = int(np.nonzero((tt[:-1] <= u2) & (u2 <= tt[1:]))[0][0]) + 1
    expect = (u2 - tt[k - 1]) * (v[k] - v[k - 1]) / (tt[k] - tt[k - 1]) + v[k - 1]
    first = [i for i, r in enumerate(data.ob) if int(r[4]) == 1][0]
    assert out["eta_at_ob_new"][first] == expect
    assert out["q_add"][0] == 287.45        # first day of the river series, portion 1
    assert np.all(out["con_at_ob"][:, 0, :] > 30.0) and np.all(out["con_at_ob"][:, 1, :] == 20.0)
    assert out["con_at_ob"].shape == (75, 2, 30)


def test_oracle_steps_the_reference_deck(oracle_so):
    d = _deck()
    c = GomCore(d, lib_path=oracle_so)
    prepare(c, initial_state(d))
    f = SeriesForcing(d)
    for it in range(1, 6):
        c.set_forcing(f.step(it))
        c.step_all()
    eta = c.get_field("eta_cell")
    assert np.isfinite(eta).all() and np.abs(eta).max() > 1e-3
    assert np.count_nonzero(c.get_field("elm_foot")) > 0      # the walk ran
