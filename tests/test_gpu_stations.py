"""Station time series on the GPU (gom_station_series) against the CPU restatement of
write_tser_out_files.f90 on the same state: bit for bit in FP64, within FP32 storage rounding in a
mixed-precision context; and the records of a packed stepping context after real steps."""
import dataclasses

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state

pytestmark = pytest.mark.gpu


def _oracle_state(oracle_so, deck, steps=4):
    ref = GomCore(deck, lib_path=oracle_so)
    prepare(ref, initial_state(deck))
    f = HostForcing(deck)
    for it in range(1, steps + 1):
        ref.set_forcing(f.step(it))
        ref.step_all()
    rng = np.random.default_rng(11)
    ref.set_field("air_p", 101325.0 + rng.normal(0.0, 80.0, deck.n_nodes))
    return ref


@pytest.mark.parametrize("precision", [0, 1])
def test_station_series_matches_oracle(oracle_so, gpu_lib, precision):
    deck = estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=3)
    ref = _oracle_state(oracle_so, deck)
    mdeck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, precision=precision))
    gpu = GomCore(mdeck, lib=gpu_lib)
    gpu.load_state(ref.state())
    rng = np.random.default_rng(5)
    cells = np.unique(rng.integers(1, deck.n_cells + 1, 40))
    nodes = np.unique(rng.integers(1, deck.n_nodes + 1, 40))
    for hloc, kw in ((1, {"station_cell": cells}), (2, {"station_node": nodes})):
        ref.set_stations(hloc, **kw)
        gpu.set_stations(hloc, **kw)
        a, b = gpu.station_series(), ref.station_series()
        assert a.shape == b.shape == (len(kw[next(iter(kw))]), 7 + 4 * deck.n_layers)
        if precision == 0:
            assert np.array_equal(a, b), f"hloc {hloc}: {np.count_nonzero(a != b)} values differ"
        else:
            # FP32 storage of the layered fields: within a few FP32 roundings of each quantity's
            # largest magnitude (eta, H, u, v, salt, temp, air pressure)
            L = deck.n_layers
            for lo, hi in ((0, 1), (1, 2), (2, 3 + L), (3 + L, 4 + 2 * L), (4 + 2 * L, 5 + 3 * L),
                           (5 + 3 * L, 6 + 4 * L), (6 + 4 * L, 7 + 4 * L)):
                scale = max(float(np.abs(b[:, lo:hi]).max()), 1e-12)
                err = float(np.abs(a[:, lo:hi] - b[:, lo:hi]).max())
                assert err <= 1e-6 * scale, f"hloc {hloc}, slots {lo}:{hi}: {err:.2e} of {scale:.2e}"
        # a second call on the same state gives the same records
        assert np.array_equal(gpu.station_series(), a)


def test_station_series_between_launched_steps(gpu_lib):
    deck = estuary(nx=24, ny=12, dx=100.0, n_layers=8, trans_sub_iter=2)
    a = GomCore(deck, lib=gpu_lib)
    prepare(a, initial_state(deck))
    a.set_stations(1, station_cell=[1, deck.n_cells // 2, deck.n_cells])
    f = HostForcing(deck)
    prev = None
    for it in range(1, 4):
        a.set_forcing(f.step(it))
        a.step_launch()
        a.step_wait()
        rec = a.station_series()
        # ordered after the step: the record reads the state the step left
        assert rec[:, 0].tolist() == a.get_field("eta_cell")[[0, deck.n_cells // 2 - 1, deck.n_cells - 1]].tolist()
        assert prev is None or not np.array_equal(rec, prev)
        prev = rec
