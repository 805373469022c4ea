"""The CUDA library against the CPU oracle on the reference's own deck (Mobile Bay, irregular
triangles, Manning drag, constant ELM substeps, heat_option 1, 30 transport subcycles, open-boundary
elevation series): every phase on the oracle's state bit for bit (the PCG within tolerance), and
a 50-step run with no foot element differing away from an element edge, equal wet/dry masks and
fields at round-off."""
from pathlib import Path

import numpy as np
import pytest

from gom_release_gb300.core import FIELDS, GomCore, TIME_LOOP, prepare
from gom_release_gb300.deck import initial_state
from gom_release_gb300.gom_inputs import DeckData, SeriesForcing, deck_from_data

pytestmark = pytest.mark.gpu

FIXTURE = Path(__file__).resolve().parent / "golden" / "mobile_bay.npz"
ETA_TOL = 1e-10      # metres: the PCG sums in another order
FIELD_RTOL = 1e-9    # after the run, relative to the field's largest magnitude


@pytest.fixture(scope="module")
def deck():
    return deck_from_data(DeckData.from_npz(FIXTURE))


def _mismatch(a, b):
    if a.dtype.kind == "i":
        return int(np.count_nonzero(a != b))
    return int(np.count_nonzero(~((a == b) | (np.isnan(a) & np.isnan(b)))))


@pytest.mark.parametrize("warm_steps", [1, 6])
def test_mobile_bay_each_phase_matches_oracle(deck, oracle_so, gpu_lib, warm_steps):
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    gpu = GomCore(deck, lib=gpu_lib)
    prepare(ref, st)
    fr = SeriesForcing(deck)
    for it in range(1, warm_steps + 1):
        ref.set_forcing(fr.step(it))
        ref.step_all()
    f = fr.full(warm_steps + 1)
    ref.set_forcing(f)
    gpu.set_forcing(f)
    report = []
    for phase in TIME_LOOP:
        gpu.load_state(ref.state())
        ref.step(phase)
        gpu.step(phase)
        for name in FIELDS:
            a, b = gpu.get_field(name), ref.get_field(name)
            if phase == "free_surface" and name in ("eta_cell_new", "eta_node"):
                err = float(np.abs(a - b).max())
                assert err < ETA_TOL, f"{phase}: {name} differs by {err:.3e}"
                continue
            n = _mismatch(a, b)
            if n:
                report.append(f"{phase}: {name} {n} entries differ, max |d|={np.abs(a.astype(float) - b).max():.3e}")
    assert not report, "\n".join(report)


def test_mobile_bay_run_matches_oracle(deck, oracle_so, gpu_lib):
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    gpu = GomCore(deck, lib=gpu_lib)
    prepare(ref, st)
    prepare(gpu, st)
    fr = SeriesForcing(deck)
    walked = mism = near = 0
    for it in range(1, 51):
        f = fr.step(it)
        ref.set_forcing(f)
        gpu.set_forcing(f)
        ref.step_all()
        gpu.step_all()
        fa, fb = gpu.get_field("elm_foot"), ref.get_field("elm_foot")
        edge = ref.get_field("elm_near_edge") != 0
        walked += int(np.count_nonzero(fb))
        near += int(np.count_nonzero(edge))
        mism += int(np.count_nonzero((fa != fb) & ~edge))
    assert walked > 0
    assert mism == 0, f"{mism} of {walked} foot elements differ away from an edge ({near} feet near an edge)"
    for name in ("top_layer_cell", "top_layer_face", "top_layer_node", "wetdry_node"):
        assert np.array_equal(gpu.get_field(name), ref.get_field(name)), name
    for name in ("eta_cell", "eta_node", "un_face", "vn_face", "wn_cell", "u_node", "w_node", "salt_cell",
                 "temp_cell", "rho_cell", "dz_cell"):
        a, b = gpu.get_field(name), ref.get_field(name)
        scale = max(float(np.abs(b).max()), 1e-30)
        assert float(np.abs(a - b).max()) / scale < FIELD_RTOL, f"{name} after 50 steps"
