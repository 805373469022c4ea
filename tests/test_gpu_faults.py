"""Failure reporting of the CUDA library: reference `stop` sites become status codes, and every
bounded device-side wait returns instead of hanging.  No test faults, traps or hangs the GPU:
failures are planted in the inputs, and the timeout case waits for a barrier participant that
does not exist until the bounded wait expires."""
import time

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, GomError, TIME_LOOP, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state
from gom_release_gb300.driver import Run

pytestmark = pytest.mark.gpu


def _deck(**kw):
    d = estuary(nx=12, ny=6, dx=100.0, n_layers=8, trans_sub_iter=2)
    for k, v in kw.items():
        setattr(d.params, k, v)
    return d


def _before(core, deck, phase):
    prepare(core, initial_state(deck))
    core.set_forcing(HostForcing(deck).full(1))
    for ph in TIME_LOOP[:TIME_LOOP.index(phase)]:
        core.step(ph)


def test_not_positive_definite_is_reported(gpu_lib):
    deck = _deck()
    c = GomCore(deck, lib=gpu_lib)
    _before(c, deck, "free_surface")
    bad = c.get_field("ainvdz1")
    bad[:] = -1.0
    c.set_field("ainvdz1", bad)
    with pytest.raises(GomError) as e:
        c.step("free_surface")
    assert e.value.code == 3 and e.value.status.site == 100 and e.value.status.entity > 0


def test_zero_pivot_is_reported(gpu_lib):
    deck = _deck()
    c = GomCore(deck, lib=gpu_lib)
    _before(c, deck, "momentum")
    dz = c.get_field("dz_face")
    dz[:] = 0.0
    c.set_field("dz_face", dz)
    with pytest.raises(GomError) as e:
        c.step("momentum")
    assert e.value.code == 4 and e.value.status.site == 587


def test_pcg_iteration_cap(gpu_lib):
    deck = _deck(max_iteration_pcg=2)
    r = Run(deck, GomCore(deck, lib=gpu_lib), initial_state(deck))
    r.advance(2)
    assert r.pcg_iters == [2, 2]


def test_barrier_wait_expires_and_device_stays_usable(gpu_lib):
    deck = _deck(test_barrier_phantom_blocks=1)
    c = GomCore(deck, lib=gpu_lib)
    _before(c, deck, "free_surface")
    t0 = time.time()
    with pytest.raises(GomError) as e:
        c.step("free_surface")
    assert e.value.code == 10           # GOM_E_TIMEOUT, from the bounded wait
    assert time.time() - t0 < 30
    c.close()
    # a fresh context on the same device runs normally afterwards
    deck2 = _deck()
    r = Run(deck2, GomCore(deck2, lib=gpu_lib), initial_state(deck2))
    r.advance(2)
    assert all(0 < i < deck2.params.max_iteration_pcg for i in r.pcg_iters)


def test_contexts_created_one_after_another_give_identical_runs(gpu_lib):
    """Context set-up zeroes and uploads its arrays through the legacy default stream while its
    kernels run on a non-blocking stream: every set-up write must have finished before the first
    kernel.  When they were not, a context created after another one (its memory recycled, its
    set-up kernels racing the zeroing) followed another trajectory from the second step on; two
    contexts of one 480k-cell basin, one after the other, must now agree bit for bit."""
    import math

    from gom_release_gb300.deck import HostForcing, tidal_basin

    ny = int(round(math.sqrt(480_000 / 1.5)))
    deck = tidal_basin(nx=int(round(480_000 / ny)), ny=ny, dx=250.0, n_layers=20, dt=60.0)
    runs = []
    for _ in range(2):
        c = GomCore(deck, lib=gpu_lib)
        p = deck.params
        c.cold_start(p.ref_salt, p.ref_temp, p.av_0, p.kv_0)
        c.step("density")
        hf = HostForcing(deck)
        for it in range(1, 6):
            c.set_forcing(hf.step(it))
            c.step_all()
        runs.append({n: c.get_field(n) for n in ("eta_cell", "un_face", "salt_cell")})
        c.close()
    for n in runs[0]:
        assert np.array_equal(runs[0][n], runs[1][n]), n
