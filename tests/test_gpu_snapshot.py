"""Asynchronous snapshots on the GPU: a snapshot begun after step N, with steps N+1 and N+2
launched before it is waited for, holds the state of step N (the state of a second context
stepped to N), in both precisions."""
import dataclasses

import numpy as np
import pytest

from gom_release_gb300.core import FIELDS, GomCore, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state
from gom_release_gb300.output import RESTART_FIELDS, Snapshot

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_snapshot_holds_the_state_it_was_taken_at(gpu_lib, precision):
    deck = estuary(nx=24, ny=12, dx=100.0, n_layers=8, trans_sub_iter=2)
    deck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, precision=precision))
    st = initial_state(deck)
    a, b = GomCore(deck, lib=gpu_lib), GomCore(deck, lib=gpu_lib)
    prepare(a, st)
    prepare(b, st)
    fa, fb = HostForcing(deck), HostForcing(deck)
    for it in range(1, 5):
        a.set_forcing(fa.step(it))
        a.step_all()
        b.set_forcing(fb.step(it))
        b.step_all()
    names = RESTART_FIELDS + ("top_layer_cell", "elm_foot")
    snap = Snapshot(a, names)
    snap.begin()
    for it in range(5, 7):
        a.set_forcing(fa.step(it))
        a.step_launch()
        a.step_wait()
    got = snap.wait()
    assert snap.ready()
    for name in names:
        assert np.array_equal(got[name], b.get_field(name)), name
    # the context itself moved on
    assert not np.array_equal(a.get_field("eta_cell"), b.get_field("eta_cell"))
    snap.close()
