"""The reference's own options beside the benchmark's, CUDA library against the CPU oracle.

The benchmark decks use the constant-Cd drag extension, the UNESCO equation of state, the
substep counts of ELM_backtrace_flag 1 and the heat_option 2 surface term.  The reference offers
more, and each option is checked here phase by phase on the oracle's state and over a run:

* bf_flag 1, Manning's n (calculate_bottom_friction.f90:25-44): bit for bit;
* bf_flag 2, log law (:45-60): bit for bit wherever the bottom half-thickness is the static one
  of a column with more than one layer; a column of one layer forms its log on the GPU (CUDA's
  log, not the C library's), and there Cdb may differ by at most 2 ulps;
* ana_density 1, linear equation of state (calculate_density_linear.f90): bit for bit;
* ELM_backtrace_flag 0, a constant substep count ELM_sub_iter (solve_nonlinear_advection.f90):
  bit for bit;
* heat_option 1, the per-layer heat source phi_sz (solve_transport_equation_v19.f90:100-131),
  in the TVD transport and in the ELM transport (solve_transport_equation_ELM_v8.f90:120): bit
  for bit.
"""
import dataclasses

import numpy as np
import pytest

from gom_release_gb300.core import FIELDS, GomCore, TIME_LOOP, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state, tidal_basin

pytestmark = pytest.mark.gpu

ETA_TOL = 1e-10          # metres: the PCG sums in a different order
FIELD_RTOL = 1e-8        # after a run, relative to the field's largest magnitude
CDB_ULPS = 2             # log law on a column of one layer (device log)


class HeatForcing(HostForcing):
    """Host forcing plus a seeded per-layer heat source phi_sz (W/m2), as heat_term_by_term
    would hand it over: absorbed short wave decreasing with depth."""

    def __init__(self, deck, seed=5):
        super().__init__(deck)
        rng = np.random.default_rng(seed)
        L = deck.n_layers
        depth = np.arange(L - 1, -1, -1, dtype=float)     # layer L is the highest
        self.base = 400.0 * np.exp(-0.45 * depth)[None, :] * rng.uniform(0.5, 1.5, size=(deck.n_cells, 1))

    def step(self, it):
        out = super().step(it)
        out["phi_sz"] = self.base * (1.0 + 0.1 * np.sin(it * 0.3))
        return out


def _variant(name):
    if name == "manning":
        return tidal_basin(nx=24, ny=16, dx=250.0, n_layers=10), dict(bf_flag=1)
    if name == "loglaw":
        return tidal_basin(nx=24, ny=16, dx=250.0, n_layers=10), dict(bf_flag=2)
    if name == "linear_eos":
        return estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=3), dict(ana_density=1)
    if name == "elm_flag0":
        return estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=3), dict(elm_backtrace_flag=0,
                                                                                  elm_sub_iter=3)
    if name == "heat_option1":
        return estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=3), dict(heat_option=1)
    if name == "heat_option1_elm":
        return (estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=1),
                dict(heat_option=1, transport_solver=2))
    raise KeyError(name)


VARIANTS = ["manning", "loglaw", "linear_eos", "elm_flag0", "heat_option1", "heat_option1_elm"]


def _deck(name):
    deck, over = _variant(name)
    return dataclasses.replace(deck, params=dataclasses.replace(deck.params, **over))


def _forcing(name, deck):
    return HeatForcing(deck) if name.startswith("heat_option1") else HostForcing(deck)


def _mismatch(a, b):
    if a.dtype.kind == "i":
        return int(np.count_nonzero(a != b))
    return int(np.count_nonzero(~((a == b) | (np.isnan(a) & np.isnan(b)))))


def _single_layer_faces(deck, snap):
    top = snap["top_layer_face"]
    return (top != 0) & (top == deck.geo["bottom_layer_at_face"])


@pytest.mark.parametrize("warm_steps", [1, 6])
@pytest.mark.parametrize("name", VARIANTS)
def test_variant_each_phase_matches_oracle(oracle_so, gpu_lib, name, warm_steps):
    deck = _deck(name)
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    gpu = GomCore(deck, lib=gpu_lib)
    prepare(ref, st)
    fr = _forcing(name, deck)
    for it in range(1, warm_steps + 1):
        ref.set_forcing(fr.step(it))
        ref.step_all()
    f = fr.full(warm_steps + 1)
    ref.set_forcing(f)
    gpu.set_forcing(f)
    report = []
    for phase in TIME_LOOP:
        snap = ref.state()
        gpu.load_state(snap)
        ref.step(phase)
        gpu.step(phase)
        for field in FIELDS:
            a, b = gpu.get_field(field), ref.get_field(field)
            if phase == "free_surface" and field in ("eta_cell_new", "eta_node"):
                assert float(np.abs(a - b).max()) < ETA_TOL, f"{phase}: {field}"
                continue
            n = _mismatch(a, b)
            if n and name == "loglaw" and phase == "bottom_friction" and field in ("cdb", "gamma_b"):
                # only single-layer columns may differ, by at most CDB_ULPS ulps
                diff = a != b
                single = _single_layer_faces(deck, snap)
                assert not np.any(diff & ~single), f"{field}: differs on a column of several layers"
                tol = CDB_ULPS * np.spacing(np.abs(b))
                assert np.all(np.abs(a - b)[diff] <= tol[diff]), f"{field}: beyond {CDB_ULPS} ulps"
                continue
            if n:
                report.append(f"{phase}: {field} {n} entries differ, max |d|={np.abs(a.astype(float) - b).max():.3e}")
    assert not report, "\n".join(report)


@pytest.mark.parametrize("name", VARIANTS)
def test_variant_run_matches_oracle(oracle_so, gpu_lib, name):
    deck = _deck(name)
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    gpu = GomCore(deck, lib=gpu_lib)
    prepare(ref, st)
    prepare(gpu, st)
    fr = _forcing(name, deck)
    mism = 0
    for it in range(1, 21):
        f = fr.step(it)
        ref.set_forcing(f)
        gpu.set_forcing(f)
        ref.step_all()
        gpu.step_all()
        fa, fb = gpu.get_field("elm_foot"), ref.get_field("elm_foot")
        edge = ref.get_field("elm_near_edge") != 0
        mism += int(np.count_nonzero((fa != fb) & ~edge))
    assert mism == 0, f"{mism} foot elements differ away from element edges"
    for field in ("top_layer_cell", "top_layer_face", "top_layer_node", "wetdry_node"):
        assert np.array_equal(gpu.get_field(field), ref.get_field(field)), field
    for field in ("eta_cell", "un_face", "vn_face", "wn_cell", "salt_cell", "temp_cell", "rho_cell", "cdb"):
        a, b = gpu.get_field(field), ref.get_field(field)
        scale = max(float(np.abs(b).max()), 1e-30)
        assert float(np.abs(a - b).max()) / scale < FIELD_RTOL, field
    if name.startswith("heat_option1"):
        # the source did something: the start is uniform over depth, the source decays with depth
        t = gpu.get_field("temp_cell").reshape(deck.n_cells, deck.n_layers)
        top = gpu.get_field("top_layer_cell")
        bot = deck.geo["bottom_layer_at_element"]
        wet = np.nonzero(top > bot)[0]
        assert float(np.max(t[wet, top[wet] - 1] - t[wet, bot[wet] - 1])) > 1e-3


def test_wind_setup_basin_matches_oracle(oracle_so, gpu_lib):
    """The closed wind set-up basin of the oracle's known-answer test, 3000 steps on the GPU:
    the same elevations as the oracle (the PCG sums in another order) and the analytic slope."""
    from test_oracle_kat import wind_basin

    d = wind_basin()
    st = initial_state(d)
    cores = [GomCore(d, lib_path=oracle_so), GomCore(d, lib=gpu_lib)]
    for c in cores:
        prepare(c, st)
        f = HostForcing(d)
        for it in range(1, 3001):
            c.set_forcing(f.full(it) if it == 1 else f.step(it))
            c.step_all()
    a, b = (c.get_field("eta_cell") for c in cores)
    assert float(np.abs(a - b).max()) < 1e-12
    xc = d.geo["x_cell"]
    slope = np.polyfit(xc, b, 1)[0]
    assert abs(slope / (1e-4 / (d.params.gravity * 5.0)) - 1.0) < 2e-3
