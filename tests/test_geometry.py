"""Start-up geometry (read_cell_inp.f90 areas, set_geometry_1.f90, calculate_voronoi_center.f90,
set_geometry_2.f90, find_element_and_face.f90): the oracle's loop-for-loop restatement
(gom_geometry_build of the CPU library) against the vectorised host builder (mesh.py and
deck._finish_levels) on the reference's Mobile Bay mesh, the synthetic estuary and basin, and
jittered mixed triangle / quadrangle meshes with and without Voronoi centres -- every array bit for
bit, the angles included (both call the C library) -- and the reference's stops as status sites."""
from pathlib import Path

import numpy as np
import pytest

from gom_release_gb300.core import GomError, geometry_build, load_library
from gom_release_gb300.deck import estuary, tidal_basin
from gom_release_gb300.gom_inputs import DeckData, deck_from_data
from gom_release_gb300.mesh import RawMesh, build_geometry, square_strip_mesh

FIXTURE = Path(__file__).resolve().parent / "golden" / "mobile_bay.npz"
IDS = ("ob_cell_id", "ob_face_id", "qb_cell", "qb_face")


def deck_inputs(d, voronoi):
    """The mesh, vertical grid and boundary node pairs a deck was built from."""
    g = d.geo
    raw = RawMesh(x=g["x_node"], y=g["y_node"], h=g["h_node"], tri_or_quad=g["tri_or_quad"],
                  cells=g["nodenum_at_cell"])
    ob = [tuple(g["nodenum_at_face"][f - 1]) for f in d.ob_face_id]
    qb = [tuple(g["nodenum_at_face"][f - 1]) for f in d.qb_face]
    return dict(raw=raw, max_nb=d.max_nb, voronoi=voronoi, z_level=d.z_level, msl=d.params.msl, ob_pairs=ob,
                q_pairs=qb)


def decks():
    data = DeckData.from_npz(FIXTURE)
    yield "mobile_bay", deck_from_data(data), int(data.cards["voronoi"])
    yield "estuary", estuary(nx=40, ny=14, dx=100.0, n_layers=8, trans_sub_iter=2), 1
    yield "basin", tidal_basin(nx=16, ny=10), 1


def jittered(seed, voronoi, nx=14, ny=9, tri_rows=3):
    """A strip mesh (quads and triangles) with every node moved by up to 12 % of the spacing."""
    x, y, cells, tq = square_strip_mesh(nx, ny, 100.0, tri_rows)
    rng = np.random.default_rng(seed)
    x = x + rng.uniform(-12.0, 12.0, len(x))
    y = y + rng.uniform(-12.0, 12.0, len(y))
    h = 5.0 + rng.uniform(0.0, 10.0, len(x))
    raw = RawMesh(x=x, y=y, h=h, tri_or_quad=tq.astype(np.int32), cells=cells.astype(np.int32))
    z_level = np.linspace(-20.0, 2.0, 12)
    return dict(raw=raw, max_nb=12, voronoi=voronoi, z_level=z_level, msl=0.5, ob_pairs=[], q_pairs=[])


def host_arrays(kw):
    """The same arrays from the host builder: build_geometry plus set_geometry_2's by hand."""
    from gom_release_gb300.deck import Params, _finish_levels

    p = Params(msl=kw["msl"], dry_depth=0.05)
    d = _finish_levels("x", kw["raw"], np.asarray(kw["z_level"], float), p, kw["ob_pairs"], kw["q_pairs"],
                       [1.0] * len(kw["q_pairs"]), voronoi=kw["voronoi"], max_nb=kw["max_nb"],
                       tide=dict(amplitude=[], period_h=[], phase=[], nodal=[], eq_arg=[], shift=0.0))
    out = dict(d.geo)
    out.update(ob_cell_id=d.ob_cell_id, ob_face_id=d.ob_face_id, qb_cell=d.qb_cell, qb_face=d.qb_face)
    return out


def assert_same(r, ref, skip=()):
    bad = []
    for k, v in r.items():
        if k == "n_faces" or k in skip:
            continue
        if not np.array_equal(np.asarray(ref[k]).reshape(v.shape), v):
            bad.append(k)
    assert not bad, bad


@pytest.fixture(scope="module")
def oracle(oracle_so):
    return load_library(oracle_so)


@pytest.mark.parametrize("name", ["mobile_bay", "estuary", "basin"])
def test_oracle_equals_host_builder_on_decks(oracle, name):
    d, vor = next((d, v) for n, d, v in decks() if n == name)
    kw = deck_inputs(d, vor)
    r = geometry_build(oracle, **kw)
    assert r["n_faces"] == d.n_faces
    ref = dict(d.geo)
    ref.update(ob_cell_id=d.ob_cell_id, ob_face_id=d.ob_face_id, qb_cell=d.qb_cell, qb_face=d.qb_face)
    assert_same(r, ref)
    # set_geometry_1.f90:164-184 tests nd == i inside its loop over the list: a node that is the
    # first local node of its first cell lists itself
    an = r["adj_nodenum_at_node"]
    selfs = np.nonzero(an[:, 1] == np.arange(1, len(an) + 1))[0]
    assert len(selfs) >= 1
    first_cell = r["adj_cellnum_at_node"][selfs, 0]
    assert np.all(kw["raw"].cells[first_cell - 1, 0] == selfs + 1)


@pytest.mark.parametrize("seed,voronoi", [(1, 0), (2, 1), (3, 1)])
def test_oracle_equals_host_builder_on_jittered_meshes(oracle, seed, voronoi):
    kw = jittered(seed, voronoi)
    r = geometry_build(oracle, **kw)
    assert_same(r, host_arrays(kw))


def _expect(oracle, kw, site, entity=None):
    with pytest.raises(GomError) as e:
        geometry_build(oracle, **kw)
    st = e.value.status
    assert st is not None and st.site == site, (st.site if st else None, site)
    if entity is not None:
        assert st.entity == entity
    return st


def test_stops_of_the_reference(oracle):
    from gom_release_gb300 import core

    base = jittered(5, 1)
    raw = base["raw"]
    # an extra quadrangle and an extra triangle whose nodes are collinear: calculate_area takes the
    # absolute value, so the reference's tests catch degenerate cells (read_cell_inp.f90:76-86)
    nn, nc = len(raw.x), len(raw.tri_or_quad)

    def extra(k):
        xs = np.append(raw.x, 1.0e4 + 10.0 * np.arange(k))
        ys = np.append(raw.y, np.full(k, 1.0e4))
        cell = np.zeros((1, 4), np.int32)
        cell[0, :k] = nn + 1 + np.arange(k)
        return dict(base, raw=RawMesh(x=xs, y=ys, h=np.append(raw.h, np.full(k, 5.0)),
                                      tri_or_quad=np.append(raw.tri_or_quad, k).astype(np.int32),
                                      cells=np.vstack([raw.cells, cell]).astype(np.int32)))

    _expect(oracle, extra(4), core.GOM_GEO["CONCAVE"], entity=nc + 1)
    _expect(oracle, extra(3), core.GOM_GEO["AREA"], entity=nc + 1)
    # a node no cell uses (set_geometry_1.f90:130-134)
    kw = dict(base, raw=RawMesh(x=np.append(raw.x, 0.0), y=np.append(raw.y, 0.0), h=np.append(raw.h, 5.0),
                                tri_or_quad=raw.tri_or_quad, cells=raw.cells))
    _expect(oracle, kw, core.GOM_GEO["HANGING"], entity=len(raw.x) + 1)
    # max_nb too small for the mesh (set_geometry_1.f90:119-123)
    _expect(oracle, dict(base, max_nb=3), core.GOM_GEO["MAX_NB"])
    # a boundary pair given clockwise (set_geometry_2.f90:37-41)
    g = geometry_build(oracle, **base)
    bf = int(np.nonzero(g["adj_cellnum_at_face"][:, 1] == 0)[0][0])
    n1, n2 = g["nodenum_at_face"][bf]
    _expect(oracle, dict(base, ob_pairs=[(n2, n1)]), core.GOM_GEO["BOUNDARY"], entity=1)
    # a vertical grid above the deepest node (set_geometry_2.f90:101-189)
    st = _expect(oracle, dict(base, z_level=np.linspace(-8.0, 2.0, 6)), core.GOM_GEO["VERTICAL"])
    assert st.entity_kind in (1, 2, 3)
