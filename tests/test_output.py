"""Output snapshots and the reference's file formats, on the CPU restatement (whose snapshot is
synchronous): the snapshot equals gom_get_field, the restart file has the record layout of
write_restart.f90 and reads back, the dump has the shape and number format of write_dump3D.f90."""
import io

import numpy as np

from gom_release_gb300.core import GomCore, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state
from gom_release_gb300.output import (DUMP3D_FIELDS, RESTART_FIELDS, Snapshot, _fortran_e, read_restart,
                                      restart_file_name, write_dump3d, write_restart)


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
