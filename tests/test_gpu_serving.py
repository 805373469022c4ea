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


def _faulty_packed_server(lib, precision, victim_rid, at_tick, on_finish):
    """A PackedServer whose chosen run fails at a chosen tick: before that step, the run's
    elevation is set above the highest level on the host (the device reports an impossible
    elevation for one of its entities)."""
    from gom_release_gb300.serve import PackedServer

    class Faulty(PackedServer):
        ticks = 0

        def _step(self):
            Faulty.ticks += 1
            if Faulty.ticks == at_tick:
                run = [r.rid for r in self.members].index(victim_rid)
                cs = self.deck.runs["run_cell_start"]
                for name in ("eta_cell", "eta_cell_new"):
                    eta = self.core.get_field(name)
                    eta[cs[run]:cs[run + 1]] = self.deck.z_level[-1] + 5.0
                    self.core.set_field(name, eta)
            return super()._step()

    return Faulty(lib, budget_bytes=64e9, precision=precision, min_interval=0.0, on_finish=on_finish)


@pytest.mark.parametrize("precision,rtol", [(0, 1e-8), (1, 1e-4)])
def test_packed_server_retires_only_the_failing_run(gpu_lib, precision, rtol):
    """One run of a pack fails: only it is retired with the error, the others finish and end as
    they end alone (within the free-surface solver's round-off, as above)."""
    from gom_release_gb300.ensemble import split

    got = {}

    def keep(req, core, run, deck):
        got[req.rid] = {k: split(deck, k, core.get_field(k))[run] for k in OUT}

    reqs = _requests()[:3]
    srv = _faulty_packed_server(gpu_lib, precision, victim_rid=1, at_tick=3, on_finish=keep)
    srv.waiting += reqs
    clock = time.perf_counter
    for tick in range(40):
        srv.maybe_repack(float(tick))
        if not srv.active() and not srv.waiting:
            break
        srv.tick(clock)
    assert sorted(got) == [0, 1, 2]
    assert reqs[1].error and "GOM_E_" in reqs[1].error and reqs[1].done_steps == 3
    assert not reqs[0].error and not reqs[2].error
    assert srv.failed_runs == 1
    for req in (reqs[0], reqs[2]):
        assert req.done_steps == req.steps
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
