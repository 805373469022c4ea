"""Output snapshots and the reference's file formats, on the CPU restatement (whose snapshot is
synchronous): the snapshot equals gom_get_field, the restart file has the record layout of
write_restart.f90 and reads back, the dump has the shape and number format of write_dump3D.f90."""
import io

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, GomError, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state
from gom_release_gb300.output import (DUMP3D_FIELDS, RESTART_FIELDS, Snapshot, _fortran_e, read_restart,
                                      restart_file_name, tser_header, tser_row, tser_time_value, tser_values,
                                      write_dump3d, write_restart)


def _advanced(oracle_so, steps=2):
    deck = estuary(nx=10, ny=6, dx=100.0, n_layers=5, trans_sub_iter=2)
    core = GomCore(deck, lib_path=oracle_so)
    prepare(core, initial_state(deck))
    f = HostForcing(deck)
    for it in range(1, steps + 1):
        core.set_forcing(f.step(it))
        core.step_all()
    return deck, core


def test_snapshot_equals_get_field(oracle_so):
    deck, core = _advanced(oracle_so)
    snap = Snapshot(core, RESTART_FIELDS)
    snap.begin()
    st = snap.wait()
    for name in RESTART_FIELDS:
        assert np.array_equal(st[name], core.get_field(name)), name
    snap.close()


def test_restart_file_round_trip(oracle_so, tmp_path):
    deck, core = _advanced(oracle_so)
    st = core.state(RESTART_FIELDS)
    path = tmp_path / restart_file_name("restart_", 42)
    assert path.name == "restart_0000042.out"
    write_restart(path, st, deck.n_layers)
    L, nc, nf, nn = deck.n_layers, deck.n_cells, deck.n_faces, deck.n_nodes
    widths = [(nc, 2), (nn, 1), (nf, 2 * L), (nn, 2 * (L + 1)), (nc, L + 1), (nn, L + 1), (nc, 3 * L), (nn, 3 * L),
              (nf, 3 * L)]
    assert path.stat().st_size == sum(n * (8 * w + 8) for n, w in widths)
    raw = path.read_bytes()
    assert int.from_bytes(raw[:4], "little") == 16 and int.from_bytes(raw[20:24], "little") == 16
    back = read_restart(path, nc, nf, nn, L)
    for name in RESTART_FIELDS:
        assert np.array_equal(back[name], st[name]), name


def test_fortran_e_format():
    assert _fortran_e(1.2345) == "  0.12345E+0001"
    assert _fortran_e(-0.000123456) == " -0.12346E-0003"
    assert _fortran_e(0.0) == "  0.00000E+0000"
    assert _fortran_e(999999.5) == "  0.10000E+0007"
    assert _fortran_e(35.0) == "  0.35000E+0002"


def test_dump3d_text_and_binary(oracle_so):
    deck, core = _advanced(oracle_so)
    st = core.state(DUMP3D_FIELDS)
    L = deck.n_layers
    buf = io.StringIO()
    write_dump3d(buf, 1.5, st, L)
    lines = buf.getvalue().splitlines()
    assert lines[0] == "        1.50000" and len(lines) == 1 + deck.n_nodes
    assert all(len(x) == 15 * (1 + 6 * L + 3) for x in lines[1:])
    first = [float(lines[1][15 * q:15 * (q + 1)]) for q in range(1 + 6 * L + 3)]
    assert np.allclose(first[0], st["eta_node"][0], rtol=1e-4, atol=1e-9)
    bbuf = io.BytesIO()
    write_dump3d(bbuf, 1.5, st, L, binary=True)
    assert len(bbuf.getvalue()) == (8 + 8) + deck.n_nodes * (8 * (6 * L + 4) + 8)


def _tser_records_py(deck, st, air_p, hloc, ids):
    """write_tser_out_files.f90:9-330 (with the node means of update_variables.f90:36-72) in
    plain Python loops over the downloaded fields: the check on the CPU restatement."""
    g, L = deck.geo, deck.n_layers
    nn = deck.n_nodes
    un = st["u_node"].reshape(nn, L + 1)
    vn = st["v_node"].reshape(nn, L + 1)
    recs = []
    for e in ids:
        if hloc == 1:
            ie = e - 1
            eta = st["eta_cell"][ie]
            top, bot = int(st["top_layer_cell"][ie]), int(g["bottom_layer_at_element"][ie])
            sc = st["salt_cell"].reshape(-1, L)[ie]
            tc = st["temp_cell"].reshape(-1, L)[ie]
            u = [0.0] * (L + 1)
            v = [0.0] * (L + 1)
            ub = vb = sb = tb = 0.0
            if top != 0:
                tq = int(g["tri_or_quad"][ie])
                for k in range(bot, top + 1):
                    for l in range(tq):
                        nd = int(g["nodenum_at_cell"][ie, l]) - 1
                        u[k] = u[k] + un[nd, k - 1] + un[nd, k]
                        v[k] = v[k] + vn[nd, k - 1] + vn[nd, k]
                    u[k] = u[k] / (tq * 2)
                    v[k] = v[k] / (tq * 2)
                n = top - bot + 1
                for k in range(bot, top + 1):
                    ub += u[k]
                    vb += v[k]
                    sb += sc[k - 1]
                    tb += tc[k - 1]
                ub, vb, sb, tb = ub / n, vb / n, sb / n, tb / n
            rec = [eta, g["h_cell"][ie] + eta, ub, *u[1:], vb, *v[1:], sb, *sc, tb, *tc,
                   air_p[ie] if e <= nn else 0.0]
        else:
            i = e - 1
            eta = st["eta_node"][i]
            top, bot = int(st["top_layer_node"][i]), int(g["bottom_layer_at_node"][i])
            sn = st["salt_node"].reshape(nn, L)[i]
            tn = st["temp_node"].reshape(nn, L)[i]
            n = top - bot + 1
            ub = vb = sb = tb = 0.0
            if n != 0:
                su = sv = ss = stt = 0.0
                for k in range(bot - 1, top + 1):
                    su += un[i, k]
                    sv += vn[i, k]
                for k in range(bot, top + 1):
                    ss += sn[k - 1]
                    stt += tn[k - 1]
                ub, vb, sb, tb = su / (n + 1), sv / (n + 1), ss / n, stt / n
            rec = [eta, g["h_node"][i] + eta, ub, *un[i, 1:], vb, *vn[i, 1:], sb, *sn, tb, *tn, air_p[i]]
        recs.append(rec)
    return np.array(recs, dtype=np.float64)


def test_station_series_follows_write_tser_out_files(oracle_so):
    deck, core = _advanced(oracle_so, steps=3)
    rng = np.random.default_rng(3)
    air_p = 101325.0 + rng.normal(0.0, 50.0, deck.n_nodes)
    core.set_field("air_p", air_p)
    st = core.state()
    cells = [1, 7, deck.n_cells // 2, deck.n_cells - 1, deck.n_cells]
    nodes = [1, 5, deck.n_nodes // 3, deck.n_nodes]
    core.set_stations(1, station_cell=cells)
    got = core.station_series()
    assert got.shape == (len(cells), 7 + 4 * deck.n_layers)
    assert np.array_equal(got, _tser_records_py(deck, st, air_p, 1, cells))
    core.set_stations(2, station_node=nodes)
    got = core.station_series()
    assert np.array_equal(got, _tser_records_py(deck, st, air_p, 2, nodes))
    assert np.any(got[:, 2] != 0.0) and np.all(got[:, 4 + 2 * deck.n_layers] > 0.0)
    with pytest.raises(GomError):
        core.set_stations(1, station_cell=[deck.n_cells + 1])


def test_tser_file_formats():
    L = 2
    recs = np.arange(2 * (7 + 4 * L), dtype=np.float64).reshape(2, -1) * 0.5
    assert tser_header("eta", 1, 3, ["A", "B"], L) == (
        'Title = "Water elevation time series from msl at cell"\n'
        'Variables = "Elapsed Time [hr]", "A", "B"\n')
    assert tser_header("salt", 2, 1, ["S1"], L, fmt="vtk") == (
        '"Elapsed Time [sec]", "S1_(00)", "S1_(01)", "S1_(02)"\n')
    row = tser_row("eta", tser_time_value(0.5, 3), recs, L)
    assert row == "  0.12000E+0002,  0.00000E+0000,  0.75000E+0001\n"
    row = tser_row("u", 12.0, recs, L)
    vals = [float(x) for x in row.strip().split(",")]
    assert vals == [12.0, 1.0, 1.5, 2.0, 8.5, 9.0, 9.5]
    assert tser_values("airp", recs, L).ravel().tolist() == [7.0, 14.5]
