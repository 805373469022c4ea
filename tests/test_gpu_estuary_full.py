"""The benchmark deck itself (the full estuary: 154,796 cells, 20 layers, TVD limiter, 4 transport
subcycles, Pacanowski-Philander closure) checked phase by phase against the CPU oracle, under the
launch variants the autotuner picks on it: every field bit for bit, the PCG within tolerance."""
import numpy as np
import pytest

from gom_release_gb300.core import FIELDS, GomCore, TIME_LOOP, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state

pytestmark = pytest.mark.gpu

ETA_TOL = 1e-10
CHOICES = ([0, 3, 3, 1], [1, 3, 3, 1], [0, 1, 3, 0])   # launch variants chosen on this deck (ELM, momentum, solve, limiter)


def _mismatch(a, b):
    if a.dtype.kind == "i":
        return int(np.count_nonzero(a != b))
    return int(np.count_nonzero(~((a == b) | (np.isnan(a) & np.isnan(b)))))


def test_full_estuary_each_phase_matches_oracle(oracle_so, gpu_lib):
    deck = estuary()
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    prepare(ref, st)
    fr = HostForcing(deck)
    for it in range(1, 3):
        ref.set_forcing(fr.step(it))
        ref.step_all()
    f = fr.full(3)
    ref.set_forcing(f)
    gpus = []
    for choice in CHOICES:
        g = GomCore(deck, lib=gpu_lib)
        g.set_tuning(choice)
        g.set_forcing(f)
        gpus.append(g)
    report = []
    for phase in TIME_LOOP:
        snap = ref.state()
        for g in gpus:
            g.load_state(snap)
            g.step(phase)
        ref.step(phase)
        for name in FIELDS:
            b = ref.get_field(name)
            for choice, g in zip(CHOICES, gpus):
                a = g.get_field(name)
                if phase == "free_surface" and name in ("eta_cell_new", "eta_node"):
                    err = float(np.abs(a - b).max())
                    assert err < ETA_TOL, f"{choice} {phase}: {name} differs by {err:.3e}"
                    continue
                n = _mismatch(a, b)
                if n:
                    report.append(f"{choice} {phase}: {name} {n} entries differ")
    assert not report, "\n".join(report)
