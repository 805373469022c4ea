"""Geometry restated from set_geometry_1.f90 / calculate_voronoi_center.f90 on synthetic meshes."""
import math

import numpy as np

from gom_release_gb300.deck import estuary, tidal_basin
from gom_release_gb300.mesh import RawMesh, build_geometry, square_strip_mesh


def test_counts_and_euler_characteristic():
    deck = tidal_basin(nx=12, ny=8, tri_rows=4)
    nx, ny = 12, 8
    tris = 4 * (2 * nx - 1)
    assert deck.n_cells == nx * ny + tris
    assert deck.n_nodes == (nx + 1) * (ny + 1) + 2 * nx + 2 * (nx + 1)
    # planar, simply connected: V - E + F = 1 (outer face excluded)
    assert deck.n_nodes - deck.n_faces + deck.n_cells == 1


def test_face_cell_consistency():
    deck = estuary(nx=15, ny=7, dx=100.0, n_layers=6)
    g = deck.geo
    for i in range(deck.n_cells):
        for l in range(g["tri_or_quad"][i]):
            j = g["facenum_at_cell"][i, l] - 1
            a1, a2 = g["adj_cellnum_at_face"][j]
            assert i + 1 in (a1, a2)
            assert g["sign_in_outflow"][i, l] == (1 if a1 == i + 1 else -1)
            nb = g["adj_cellnum_at_cell"][i, l]
            assert nb == (a2 if a1 == i + 1 else a1)
    a1 = g["adj_cellnum_at_face"][:, 0]
    a2 = g["adj_cellnum_at_face"][:, 1]
    assert np.all(a1 > 0) and np.all((a2 == 0) | (a2 > a1))


def test_orthogonality_and_voronoi_centres():
    deck = tidal_basin(nx=10, ny=6, tri_rows=4)
    g = deck.geo
    inner = g["adj_cellnum_at_face"][:, 1] != 0
    # orthogonal mesh: the line between the centres of two cells is normal to their face
    assert np.allclose(g["cos_theta2"][inner], 1.0, atol=1e-12)
    assert np.allclose(g["sin_theta2"][inner], 0.0, atol=1e-12)
    tri = g["tri_or_quad"] == 3
    cx = np.zeros(deck.n_cells)
    for l in range(3):
        cx += g["x_node"][g["nodenum_at_cell"][:, l] - 1]
    assert np.allclose(g["x_cell"][tri], cx[tri] / 3.0, atol=1e-9)   # equilateral: circumcentre = centroid


def test_areas():
    x, y, cells, tq = square_strip_mesh(4, 3, 250.0, 2)
    geo = build_geometry(RawMesh(x=x, y=y, h=np.full(len(x), 10.0), tri_or_quad=tq, cells=cells))
    a = geo.arrays["area"]
    assert np.allclose(a[tq == 4], 250.0 ** 2)
    assert np.allclose(a[tq == 3], math.sqrt(3) / 4 * 250.0 ** 2)


def test_layers_and_wet_columns():
    deck = tidal_basin(nx=8, ny=6)
    z = deck.z_level
    b = deck.geo["bottom_layer_at_element"]
    h = deck.geo["h_cell"]
    assert np.all(z[b - 1] <= -h) and np.all(-h < z[b])
