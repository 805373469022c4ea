"""Continuous batching: runs admitted at different times, stepped together with their graphs
queued on separate streams, give the same result as each run alone."""
import time

import numpy as np
import pytest

from gom_release_gb300.ensemble import storm_run
from gom_release_gb300.serve import Request, Server, storm_context

pytestmark = pytest.mark.gpu

OUT = ("eta_cell", "un_face", "salt_cell", "top_layer_cell", "wetdry_node")


def _requests():
    decks = [storm_run(31, 500, 1.2, 12, max_layers=14), storm_run(32, 900, 2.5, 14, max_layers=14),
             storm_run(33, 300, 1.0, 10, max_layers=14)]
    steps = [9, 14, 5, 11]
    return [Request(rid=i, deck=decks[i % 3], storm=decks[i % 3].meta["storm"], steps=steps[i], arrival=0.0)
            for i in range(4)]


@pytest.mark.parametrize("precision", [0, 1])
def test_each_request_same_alone_and_in_the_mix(gpu_lib, precision):
    got = {}

    def keep(req, core):
        got[req.rid] = {k: core.get_field(k) for k in OUT}

    srv = Server(gpu_lib, budget_bytes=64e9, precision=precision, on_finish=keep)
    reqs = _requests()
    srv.waiting.append(reqs[0])
    srv.admit(0.0)
    clock = time.perf_counter
    # the other requests arrive while the first is in flight
    for tick in range(20):
        if tick == 2:
            srv.waiting.append(reqs[1])
        if tick == 4:
            srv.waiting += reqs[2:]
        srv.admit(0.0)
        if not srv.active and not srv.waiting:
            break
        srv.tick(clock)
    assert sorted(got) == [0, 1, 2, 3]
    for req in reqs:
        alone = storm_context(gpu_lib, req.deck, precision, [req.storm])
        for _ in range(req.steps):
            alone.step_launch()
            alone.step_wait()
        for k in OUT:
            assert np.array_equal(alone.get_field(k), got[req.rid][k]), (req.rid, k)
        alone.close()


@pytest.mark.parametrize("precision,rtol", [(0, 1e-8), (1, 1e-4)])
def test_packed_server_same_alone_and_in_the_mix(gpu_lib, precision, rtol):
    """Runs admitted into a packed context at different times (repacks move the in-flight runs
    with gom_copy_run) end as they end alone, within the free-surface solver's round-off."""
    from gom_release_gb300.ensemble import split
    from gom_release_gb300.serve import PackedServer

    got = {}

    def keep(req, core, run, deck):
        got[req.rid] = {k: split(deck, k, core.get_field(k))[run] for k in OUT}

    srv = PackedServer(gpu_lib, budget_bytes=64e9, precision=precision, min_interval=0.0, on_finish=keep)
    reqs = _requests()
    clock = time.perf_counter
    srv.waiting.append(reqs[0])
    for tick in range(24):
        if tick == 2:
            srv.waiting.append(reqs[1])
        if tick == 4:
            srv.waiting += reqs[2:]
        srv.maybe_repack(float(tick))
        if not srv.active() and not srv.waiting:
            break
        srv.tick(clock)
    assert sorted(got) == [0, 1, 2, 3]
    assert srv.repacks >= 3
    for req in reqs:
        alone = storm_context(gpu_lib, req.deck, precision, [req.storm])
        for _ in range(req.steps):
            alone.step_launch()
            alone.step_wait()
        for k in OUT:
            a, b = alone.get_field(k), got[req.rid][k]
            if a.dtype.kind == "i":
                assert np.array_equal(a, b), (req.rid, k)
            else:
                scale = max(float(np.abs(a).max()), 1e-30)
                assert float(np.abs(a - b).max()) <= rtol * scale, (req.rid, k)
        alone.close()
