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
