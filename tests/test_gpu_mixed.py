"""Mixed-precision contexts (FP32 layered state, FP64 elevations / free-surface solve / densities /
conservation sums) against the FP64 CPU oracle on the same inputs.

Per phase: the oracle's state is uploaded (rounded to FP32 where the mixed context stores FP32),
both run one reference subroutine, and every field must agree to FP32 accuracy relative to the
field's magnitude; layer indices and wet/dry masks must agree exactly.  Over a multi-step run the
fields must stay within the stated tolerances and volume must be conserved to FP64 round-off of
the FP32-stored thicknesses.
"""
import dataclasses

import numpy as np
import pytest

from gom_release_gb300.core import FIELDS, GomCore, TIME_LOOP, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state, tidal_basin

pytestmark = pytest.mark.gpu

PHASE_RTOL = 2e-5        # one phase from identical inputs, relative to the field's max magnitude
# the ELM velocities of one advection phase: the FP32 walk decides edge crossings and substep
# counts on FP32 offsets, so on the oblique coastal triangles a foot within FP32 resolution of
# an edge follows another path than the FP64 walk
ELM_RTOL = 1e-4
ETA_ATOL_PHASE = 1e-7    # metres, one free-surface solve
INT_FIELDS = ("top_layer_cell", "top_layer_face", "top_layer_node", "wetdry_node")
# after 25 steps (relative to the field's max magnitude; eta in metres)
RUN_RTOL = {"un_face": 1e-4, "vn_face": 1e-4, "wn_cell": 1e-4, "u_node": 1e-4, "w_node": 1e-3,
            "salt_cell": 2e-5, "temp_cell": 2e-5, "salt_node": 2e-5, "rho_cell": 1e-6, "dz_cell": 1e-6}
RUN_ETA_ATOL = 1e-5


def mixed(deck):
    return dataclasses.replace(deck, params=dataclasses.replace(deck.params, precision=1))


def _decks():
    return [tidal_basin(nx=24, ny=16, dx=250.0, n_layers=10),
            estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=3)]


@pytest.fixture(scope="module", params=[0, 1], ids=["basin", "estuary"])
def deck(request):
    return _decks()[request.param]


def rel_err(a, b):
    if a.size == 0:
        return 0.0
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    scale = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a - b).max()) / scale


def test_mixed_field_storage_rounds_to_fp32(gpu_lib):
    deck = mixed(estuary(nx=12, ny=8, dx=100.0, n_layers=6, trans_sub_iter=2))
    g = GomCore(deck, lib=gpu_lib)
    st = initial_state(deck)
    prepare(g, st)
    rng = np.random.default_rng(3)
    for name in ("salt_cell", "un_face", "eta_cell", "rho_node"):
        v = rng.normal(size=g.get_field(name).shape) * 10.0
        g.set_field(name, v)
        back = g.get_field(name)
        want = v if name in ("eta_cell", "rho_node") else v.astype(np.float32).astype(np.float64)
        assert np.array_equal(back, want), name


@pytest.mark.parametrize("warm_steps", [1, 6])
def test_each_phase_tracks_oracle(deck, oracle_so, gpu_lib, warm_steps):
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    gpu = GomCore(mixed(deck), lib=gpu_lib)
    prepare(ref, st)
    fr = HostForcing(deck)
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
            if name in INT_FIELDS:
                if not np.array_equal(a, b):
                    report.append(f"{phase}: {name} {int(np.count_nonzero(a != b))} entries differ")
                continue
            if a.dtype.kind == "i":
                continue   # ELM foot elements and substep counts: compared in the FP64 tests
            if phase == "free_surface" and name in ("eta_cell_new", "eta_node"):
                err = float(np.abs(a - b).max())
                if err > ETA_ATOL_PHASE:
                    report.append(f"{phase}: {name} differs by {err:.3e} m")
                continue
            err = rel_err(a, b)
            if err > (ELM_RTOL if name in ("un_elm", "vn_elm") else PHASE_RTOL):
                report.append(f"{phase}: {name} relative error {err:.3e}")
    assert not report, "\n".join(report)


def test_run_tracks_oracle(deck, oracle_so, gpu_lib):
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    gpu = GomCore(mixed(deck), lib=gpu_lib)
    prepare(ref, st)
    prepare(gpu, st)
    fa, fb = HostForcing(deck), HostForcing(deck)
    v0, _ = ref.conservation()
    n = 25
    for it in range(1, n + 1):
        ref.set_forcing(fa.step(it))
        gpu.set_forcing(fb.step(it))
        ref.step_all()
        gpu.step_all()
    for name in INT_FIELDS:
        a, b = gpu.get_field(name), ref.get_field(name)
        assert np.count_nonzero(a != b) <= 0.001 * a.size, name
    eta_err = float(np.abs(gpu.get_field("eta_cell") - ref.get_field("eta_cell")).max())
    assert eta_err < RUN_ETA_ATOL, f"eta differs by {eta_err:.3e} m after {n} steps"
    for name, tol in RUN_RTOL.items():
        err = rel_err(gpu.get_field(name), ref.get_field(name))
        assert err < tol, f"{name}: relative error {err:.3e} after {n} steps"
    va, sa = gpu.conservation()
    vb, sb = ref.conservation()
    assert abs(va - vb) <= 1e-6 * abs(vb)
    assert abs(sa - sb) <= 1e-6 * abs(sb)


def test_mixed_volume_conserved_in_closed_basin(gpu_lib):
    """FP64 conservation sums over the FP64 elevations: a closed basin keeps its volume to
    round-off when the free-surface system is solved to a ratio of 1e-24."""
    deck = tidal_basin(nx=14, ny=10, closed=True)
    deck.params.error_tolerance = 1e-24
    deck = mixed(deck)
    x = deck.geo["x_cell"]
    st = initial_state(deck, 0.2 * np.cos(np.pi * x / x.max()))
    g = GomCore(deck, lib=gpu_lib)
    prepare(g, st)
    fr = HostForcing(deck)
    v0, _ = g.conservation()
    for it in range(1, 41):
        g.set_forcing(fr.step(it))
        g.step_all()
    v1, _ = g.conservation()
    assert abs(v1 - v0) <= 1e-12 * v0, f"volume drift {abs(v1 - v0) / v0:.3e}"
    assert np.abs(g.get_field("eta_cell")).max() > 1e-3


def test_elm_transport_mixed_tracks_fp64(gpu_lib):
    """The ELM transport in a mixed-precision context tracks the FP64 one (15 steps)."""
    deck = estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=1)
    deck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, transport_solver=2))
    st = initial_state(deck)
    a = GomCore(deck, lib=gpu_lib)
    b = GomCore(mixed(deck), lib=gpu_lib)
    prepare(a, st)
    prepare(b, st)
    fa, fb = HostForcing(deck), HostForcing(deck)
    for it in range(1, 16):
        a.set_forcing(fa.step(it))
        b.set_forcing(fb.step(it))
        a.step_all()
        b.step_all()
    for name in ("salt_cell", "temp_cell", "salt_node"):
        assert rel_err(b.get_field(name), a.get_field(name)) < 2e-5, name
