"""Packed ensembles on the GPU: every run advanced in one launch per phase, one PCG per run.

* the packed FP64 context tracks the packed oracle (which equals each run alone bit for bit);
* each run's result is the same alone and in the mix, within the free-surface solver's
  round-off (the per-run PCG sums its dot products over a different block split);
* the mixed-precision packed context tracks the FP64 one within the mixed-precision tolerances.
"""
import dataclasses

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, prepare
from gom_release_gb300.deck import initial_state
from gom_release_gb300.ensemble import PackedForcing, StormForcing, pack, split, storm_run

pytestmark = pytest.mark.gpu

FIELDS_CHECKED = ("eta_cell", "eta_node", "un_face", "vn_face", "wn_cell", "u_node", "w_node", "salt_cell",
                  "dz_cell")
INT_FIELDS = ("top_layer_cell", "top_layer_face", "top_layer_node", "wetdry_node")


def runs():
    return [storm_run(21, 700, 1.5, 12, max_layers=14), storm_run(22, 300, 3.0, 14, max_layers=14),
            storm_run(23, 1100, 1.0, 10, max_layers=14), storm_run(24, 450, 2.0, 13, max_layers=14)]


def rel(a, b):
    scale = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a - b).max()) / scale


def advance(core, forcing, n):
    for it in range(1, n + 1):
        core.set_forcing(forcing.step(it))
        core.step_all()


def test_packed_gpu_tracks_packed_oracle(oracle_so, gpu_lib):
    pk = pack(runs())
    st = initial_state(pk)
    ref = GomCore(pk, lib_path=oracle_so)
    gpu = GomCore(pk, lib=gpu_lib)
    prepare(ref, st)
    prepare(gpu, st)
    advance(ref, PackedForcing(pk), 15)
    advance(gpu, PackedForcing(pk), 15)
    for name in INT_FIELDS:
        assert np.array_equal(gpu.get_field(name), ref.get_field(name)), name
    for name in FIELDS_CHECKED:
        err = rel(gpu.get_field(name), ref.get_field(name))
        assert err < 1e-8, f"{name}: relative error {err:.3e}"


def test_each_run_same_alone_and_in_the_mix(gpu_lib):
    members = runs()
    pk = pack(members)
    gpu = GomCore(pk, lib=gpu_lib)
    prepare(gpu, initial_state(pk))
    advance(gpu, PackedForcing(pk), 15)
    for r, d in enumerate(members):
        c = GomCore(d, lib=gpu_lib)
        prepare(c, initial_state(d))
        advance(c, StormForcing(d), 15)
        for name in INT_FIELDS:
            assert np.array_equal(c.get_field(name), split(pk, name, gpu.get_field(name))[r]), (name, r)
        for name in FIELDS_CHECKED:
            err = rel(split(pk, name, gpu.get_field(name))[r], c.get_field(name))
            assert err < 1e-8, f"run {r} {name}: relative error {err:.3e}"


def test_mixed_packed_tracks_fp64_packed(gpu_lib):
    pk = pack(runs())
    pm = dataclasses.replace(pk, params=dataclasses.replace(pk.params, precision=1))
    st = initial_state(pk)
    a = GomCore(pk, lib=gpu_lib)
    b = GomCore(pm, lib=gpu_lib)
    prepare(a, st)
    prepare(b, st)
    advance(a, PackedForcing(pk), 15)
    advance(b, PackedForcing(pk), 15)
    assert float(np.abs(a.get_field("eta_cell") - b.get_field("eta_cell")).max()) < 1e-5
    for name in ("un_face", "vn_face", "u_node", "salt_cell"):
        err = rel(b.get_field(name), a.get_field(name))
        assert err < 1e-4, f"{name}: relative error {err:.3e}"
    for name in INT_FIELDS:
        assert np.count_nonzero(a.get_field(name) != b.get_field(name)) <= 0.001 * a.get_field(name).size


def test_device_storm_forcing_matches_host(gpu_lib):
    """gom_set_storms: the forcing the device writes each step equals the host restatement
    (transcendental functions differ in the last bits between CUDA and numpy)."""
    members = runs()
    pk = pack(members)
    g = GomCore(pk, lib=gpu_lib)
    prepare(g, initial_state(pk))
    g.set_forcing(PackedForcing(pk).step(1))       # boundary tracer concentrations
    g.set_storms([d.meta["storm"] for d in members], elapsed_time=0.0)
    host = PackedForcing(pk)
    for it in range(1, 6):
        g.step_all()
        h = host.step(it)
        for name in ("wind_stress_normal", "wind_stress_tangnt", "gamma_t", "air_p", "eta_at_ob_old",
                     "eta_at_ob_new"):
            a, b = g.get_field(name), h[name]
            scale = max(float(np.abs(b).max()), 1e-30)
            assert float(np.abs(a - b).max()) <= 1e-12 * scale, (name, it)
    assert float(np.abs(g.get_field("wind_stress_normal")).max()) > 0.0


def test_device_forced_run_tracks_host_forced_run(gpu_lib):
    members = runs()
    pk = pack(members)
    st = initial_state(pk)
    a = GomCore(pk, lib=gpu_lib)
    b = GomCore(pk, lib=gpu_lib)
    prepare(a, st)
    prepare(b, st)
    advance(a, PackedForcing(pk), 15)
    b.set_forcing(PackedForcing(pk).step(1))
    b.set_storms([d.meta["storm"] for d in members], elapsed_time=0.0)
    for _ in range(15):
        b.step_all()
    for name in FIELDS_CHECKED:
        err = rel(b.get_field(name), a.get_field(name))
        assert err < 1e-8, f"{name}: relative error {err:.3e}"


@pytest.mark.parametrize("precision", [0, 1])
def test_device_cold_start_equals_host_initial_state(gpu_lib, precision):
    pk = pack(runs())
    pk = dataclasses.replace(pk, params=dataclasses.replace(pk.params, precision=precision))
    st = initial_state(pk)
    a = GomCore(pk, lib=gpu_lib)
    b = GomCore(pk, lib=gpu_lib)
    prepare(a, st)
    b.cold_start(30.0, 20.0, pk.params.av_0, pk.params.kv_0)
    b.step("density")
    from gom_release_gb300.core import FIELDS
    for name in FIELDS:
        assert np.array_equal(a.get_field(name), b.get_field(name)), name


@pytest.mark.parametrize("precision", [0, 1])
def test_every_launch_variant_gives_the_same_results(gpu_lib, precision):
    """Each compiled variant of each tunable launch (gom_set_tuning) changes the launch shape only:
    twelve storm-forced steps of a packed ensemble end bit for bit where variant 0 ends, ELM foot
    elements included."""
    from gom_release_gb300.core import FIELDS
    members = runs()
    pk = pack(members)
    pk = dataclasses.replace(pk, params=dataclasses.replace(pk.params, precision=precision))
    st = initial_state(pk)
    storms = [d.meta["storm"] for d in members]

    def run(choice):
        c = GomCore(pk, lib=gpu_lib)
        prepare(c, st)
        c.set_tuning(choice)
        c.set_forcing(PackedForcing(pk).step(1))
        c.set_storms(storms, elapsed_time=0.0)
        for _ in range(12):
            c.step_all()
        out = {n: c.get_field(n) for n in FIELDS}
        c.close()
        return out

    base = run([0, 0, 0, 0])
    assert np.count_nonzero(base["elm_foot"]) > 0
    counts = GomCore(pk, lib=gpu_lib).tuning_variants()
    for site, n in enumerate(counts):
        for v in range(1, n):
            choice = [0, 0, 0, 0]
            choice[site] = v
            got = run(choice)
            for name in FIELDS:
                a, b = got[name], base[name]
                assert a.tobytes() == b.tobytes(), (site, v, name)


@pytest.mark.parametrize("precision", [0, 1])
def test_strongest_storm_runs_a_full_day(gpu_lib, precision):
    """The strongest vortex of the ensemble's range (80 hPa, Rmax 20 km, B 1.8: 68 m/s winds)
    crossing a 30-layer shelf run, 1440 steps of 60 s with the storm forcing on the device, in
    FP64 and in mixed precision: no failure, currents and surge within storm-surge bounds."""
    from gom_release_gb300.serve import storm_context

    d = storm_run(3, 4000, 4.0, 30)
    s = dataclasses.replace(d.meta["storm"], dp=8000.0, b=1.8, rmax=20e3)
    core = storm_context(gpu_lib, d, precision, [s])
    umax = etamax = 0.0
    for hour in range(24):
        for _ in range(60):
            core.step_launch()
        core.step_wait()
        umax = max(umax, float(np.abs(core.get_field("un_face")).max()))
        etamax = max(etamax, float(np.abs(core.get_field("eta_cell")).max()))
    assert core.status().code == 0
    assert 0.5 < umax < 6.0, umax
    assert 0.3 < etamax < 6.0, etamax
