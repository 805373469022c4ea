"""Packed ensembles on the CPU oracle: a packed deck is the disjoint union of its runs, and the
oracle advances it exactly as it advances each run alone (per-run PCG, per-run stale-rtemp0
walk), bit for bit."""
import numpy as np

from gom_release_gb300.core import FIELDS, GomCore, prepare
from gom_release_gb300.deck import initial_state
from gom_release_gb300.ensemble import PackedForcing, StormForcing, pack, split, storm_run


def small_runs():
    return [storm_run(11, 600, 1.5, 12, max_layers=14), storm_run(12, 300, 3.0, 14, max_layers=14),
            storm_run(13, 900, 1.0, 10, max_layers=14)]


def test_pack_offsets_and_ranges():
    runs = small_runs()
    pk = pack(runs)
    r = pk.runs
    assert list(r["run_cell_start"]) == list(np.cumsum([0] + [d.n_cells for d in runs]))
    assert list(r["run_face_start"]) == list(np.cumsum([0] + [d.n_faces for d in runs]))
    assert list(r["run_ob_start"]) == list(np.cumsum([0] + [d.n_ob for d in runs]))
    g = pk.geo
    for k in range(len(runs)):
        c0, c1 = r["run_cell_start"][k], r["run_cell_start"][k + 1]
        n0, n1 = r["run_node_start"][k], r["run_node_start"][k + 1]
        f0, f1 = r["run_face_start"][k], r["run_face_start"][k + 1]
        nodes = g["nodenum_at_cell"][c0:c1]
        assert nodes[nodes != 0].min() > n0 and nodes.max() <= n1
        faces = g["facenum_at_cell"][c0:c1]
        assert faces[faces != 0].min() > f0 and faces.max() <= f1
        adj = g["adj_cellnum_at_cell"][c0:c1]
        assert adj[adj != 0].min() > c0 and adj.max() <= c1
        bt = g["boundary_type_of_face"][f0:f1]
        o0, o1 = r["run_ob_start"][k], r["run_ob_start"][k + 1]
        assert bt[bt > 0].min() > o0 and bt.max() <= o1


def test_packed_oracle_equals_runs_alone(oracle_so):
    runs = small_runs()
    pk = pack(runs)
    alone = []
    for d in runs:
        c = GomCore(d, lib_path=oracle_so)
        prepare(c, initial_state(d))
        alone.append((c, StormForcing(d)))
    cp = GomCore(pk, lib_path=oracle_so)
    prepare(cp, initial_state(pk))
    fp = PackedForcing(pk)
    for it in range(1, 13):
        for c, f in alone:
            c.set_forcing(f.step(it))
            c.step_all()
        cp.set_forcing(fp.step(it))
        cp.step_all()
    assert np.abs(cp.get_field("eta_cell")).max() > 1e-3
    for name in FIELDS:
        if name == "qu_boundary":
            continue
        parts = split(pk, name, cp.get_field(name))
        for r, (c, _) in enumerate(alone):
            b = parts[r]
            if name == "elm_foot":
                b = np.where(b != 0, b - pk.runs["run_cell_start"][r], 0)
            assert np.array_equal(c.get_field(name), b), (name, r)
