"""Run decks: mesh + vertical grid + parameters + boundaries + initial state + forcing.

A deck holds what GOM's start-up (scan_gom, read_main_inp, set_geometry_2, prepare_gom) leaves
in ``mod_global_variables`` before the time loop of main.f90:53 starts, for synthetic
configurations generated from a seed:

* ``tidal_basin``  -- 120x80 squares of 250 m plus a 4-row equilateral-triangle strip on the
  closed north edge, 10 z-layers, harmonic M2 tide on the southern open boundary;
* ``estuary``      -- the same generator at 100 m, a river at the channel head, an ocean
  boundary with salinity and temperature series, baroclinic, TVD limiter on, 20 z-layers.

Per-step host forcing (setup_spinup.f90, compute_boundary_eta.f90, calculate_Q.f90 and the
boundary series interpolation of solve_transport_equation_v19.f90:229-534) is produced by
``HostForcing``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .mesh import (RawMesh, build_geometry, coastal_strip, bottom_layers, find_elements_and_faces,
                   fourier_noise, square_strip_mesh)

PI = 3.141592653589793          # mod_global_variables.f90: pi
DEG2RAD = PI / 180.0


def f32(v: float) -> float:
    """Value of a default-REAL (single precision) Fortran literal promoted to double."""
    return float(np.float32(v))


@dataclass
class Params:
    gravity: float = 9.81
    rho_o: float = 1000.0
    msl: float = 0.0
    dt: float = 120.0
    theta: float = 0.6
    adv_onoff_depth: float = 0.01
    von_karman: float = 0.41
    cd_const: float = 0.0025
    dry_depth: float = 0.01
    smagorinsky: float = 0.021
    ah_0: float = 0.0
    kh_0: float = 0.0
    error_tolerance: float = 1e-10
    delta_z_min: float = 0.0
    denominator_min_for_matrix: float = 0.0
    advection_flag: int = 1
    elm_backtrace_flag: int = 1
    elm_sub_iter: int = 1
    elm_min_iter: int = 1
    elm_max_iter: int = 20
    bf_flag: int = 3
    baroclinic_flag: int = 0
    ana_density: int = 0
    max_iteration_pcg: int = 1000
    transport_flag: int = 1
    trans_sub_iter: int = 1
    h_flux_limiter: int = 0
    v_flux_limiter: int = 0
    is_salt: int = 1
    is_temp: int = 1
    heat_option: int = 2
    test_barrier_phantom_blocks: int = 0
    precision: int = 0              # 0 FP64, 1 mixed (FP32 layered state)
    # turbulence_closure_v1.f90: 0 off (reference time loop), 1 step-Ri, 2 Pacanowski-Philander;
    # the coefficients are the closure's usual values (the reference reads none of them)
    turbulence_flag: int = 0
    transport_solver: int = 1     # 1 TVD (solve_transport_equation_v19), 2 ELM (..._ELM_v8)
    pp_h1: float = 20.0
    pp_h2: float = 50.0
    pp_vdmax1: float = 1.0e-2
    pp_vdmax2: float = 1.0e-2
    pp_vdmin1: float = 1.0e-5
    pp_vdmin2: float = 1.0e-5
    pp_tdmin: float = 1.0e-5
    # not part of the C ABI params (host-side start-up values)
    av_0: float = 1e-3
    kv_0: float = 1e-4
    coriolis_lat: float = 30.0
    manning: float = 0.02
    bf_height: float = 0.001
    ref_salt: float = 30.0
    ref_temp: float = 20.0


@dataclass
class Deck:
    name: str
    geo: dict                       # geometry arrays (numpy, layout of mesh.py)
    n_nodes: int
    n_cells: int
    n_faces: int
    n_layers: int
    max_nb: int
    params: Params
    z_level: np.ndarray             # (L+1,)
    delta_z: np.ndarray             # (L,)
    ob_cell_id: np.ndarray          # (n_ob,)
    ob_face_id: np.ndarray
    qb_cell: np.ndarray             # (n_qb,)
    qb_face: np.ndarray
    q_portion: np.ndarray
    tide: dict                      # harmonic constituents for the open boundary
    ob_salt: float | None = None
    ob_temp: float | None = None
    q_total: float = 0.0
    q_salt: float | None = None
    q_temp: float | None = None
    wind_stress: tuple[float, float] = (0.0, 0.0)   # Pa, x/y
    tide_spinup_days: float = 0.25
    n_steps: int = 720
    seed: int = 0
    init_salt_node: np.ndarray | None = None        # (N_n, L)
    init_temp_node: np.ndarray | None = None
    meta: dict = field(default_factory=dict)
    runs: dict | None = None        # packed runs: run_{cell,face,node,ob}_start (n_runs + 1)

    @property
    def n_ob(self) -> int:
        return len(self.ob_cell_id)

    @property
    def n_qb(self) -> int:
        return len(self.qb_cell)


# ----------------------------------------------------------------------------- vertical grid
def uniform_z_levels(z_bottom: float, z_top: float, n_layers: int) -> tuple[np.ndarray, np.ndarray, float]:
    """z_level(0:L) and delta_z(1:L) as read_main_inp.f90 card C2/C2_1 derives them."""
    z = np.array([z_bottom + (z_top - z_bottom) * k / n_layers for k in range(n_layers + 1)])
    dz = np.array([z[k] - z[k - 1] for k in range(1, n_layers + 1)])
    return z, dz, float(dz.min())


def _boundaries(geo, pairs):
    cells, faces = find_elements_and_faces(geo, pairs)
    if np.any(cells == 0) or np.any(faces == 0):
        raise ValueError("boundary node pair not found in CCW order")
    return cells.astype(np.int32), faces.astype(np.int32)


def _finish(name, raw, L, z_bottom, z_top, params, ob_pairs, q_pairs, q_portion, **kw) -> Deck:
    z_level, _, _ = uniform_z_levels(z_bottom, z_top, L)
    return _finish_levels(name, raw, z_level, params, ob_pairs, q_pairs, q_portion, **kw)


def _device_geometry(lib, raw, z_level, msl, ob_pairs, q_pairs, voronoi, max_nb):
    """set_geometry_1/2 through gom_geometry_build of `lib` (the CUDA library): the arrays of
    build_geometry plus the boundary and bottom-layer arrays _finish_levels derives."""
    from .core import geometry_build

    r = geometry_build(lib, raw, max_nb, voronoi, z_level, msl, ob_pairs, q_pairs)
    a = dict(x_node=raw.x, y_node=raw.y, h_node=raw.h, tri_or_quad=raw.tri_or_quad.astype(np.int32),
             nodenum_at_cell=raw.cells.astype(np.int32))
    ids = {k: r.pop(k) for k in ("ob_cell_id", "ob_face_id", "qb_cell", "qb_face")}
    nf = r.pop("n_faces")
    a.update(r)
    return a, nf, ids


def _finish_levels(name, raw, z_level, params, ob_pairs, q_pairs, q_portion, voronoi: int = 1, max_nb: int = 12,
                   coriolis_on: bool = True, geometry_lib=None, **kw) -> Deck:
    """Geometry, vertical grid and boundaries of a deck whose level heights z_level(0:L) are given
    (read_main_inp.f90 cards C2/C2_1, set_geometry_1.f90, set_geometry_2.f90).  With
    ``geometry_lib`` (a loaded CUDA library) set_geometry_1/2 run on the GPU."""
    if geometry_lib is not None:
        return _finish_device(name, raw, z_level, params, ob_pairs, q_pairs, q_portion, voronoi, max_nb, coriolis_on,
                              geometry_lib, **kw)
    g = build_geometry(raw, max_nb=max_nb, voronoi=voronoi)
    a = g.arrays
    L, delta_z = _vertical(z_level, params)
    ob_cell_id, ob_face_id = _boundaries(g, ob_pairs) if ob_pairs else (np.zeros(0, np.int32), np.zeros(0, np.int32))
    qb_cell, qb_face = _boundaries(g, q_pairs) if q_pairs else (np.zeros(0, np.int32), np.zeros(0, np.int32))
    nf, nc, nn = g.n_faces, g.n_cells, g.n_nodes
    ob_element_flag = np.zeros(nc, np.int32)
    boundary_type_of_face = np.zeros(nf, np.int32)
    for i, (e, f) in enumerate(zip(ob_cell_id, ob_face_id), start=1):   # set_geometry_2.f90:62-73
        ob_element_flag[e - 1] = i
        boundary_type_of_face[f - 1] = i
    boundary_type_of_face[(a["adj_cellnum_at_face"][:, 1] == 0) & (boundary_type_of_face == 0)] = -1
    qb_element_flag = np.zeros(nc, np.int32)
    isflowside3 = np.zeros(nf, np.int32)
    for i, (e, f) in enumerate(zip(qb_cell, qb_face), start=1):          # read_main_inp.f90:885-888
        isflowside3[f - 1] = i
        qb_element_flag[e - 1] = i
    a.update(
        bottom_layer_at_element=bottom_layers(a["h_cell"], params.msl, z_level),
        bottom_layer_at_face=bottom_layers(a["h_face"], params.msl, z_level),
        bottom_layer_at_node=bottom_layers(a["h_node"], params.msl, z_level),
        initial_wetdry_node=(a["h_node"] <= 0.0).astype(np.int32),    # read_node_inp.f90:72-74
        ob_element_flag=ob_element_flag, qb_element_flag=qb_element_flag,
        boundary_type_of_face=boundary_type_of_face, isflowside3=isflowside3,
    )
    _face_constants(a, nf, params, coriolis_on)
    return Deck(name=name, geo=a, n_nodes=nn, n_cells=nc, n_faces=nf, n_layers=L, max_nb=g.max_nb,
                params=params, z_level=z_level, delta_z=delta_z,
                ob_cell_id=ob_cell_id, ob_face_id=ob_face_id, qb_cell=qb_cell, qb_face=qb_face,
                q_portion=np.asarray(q_portion, dtype=np.float64), **kw)


def _vertical(z_level, params):
    """Cards C2 / C2_1 and C5_03 of read_main_inp.f90: layer thicknesses, the smallest, and
    denominator_min_for_matrix."""
    L = len(z_level) - 1
    delta_z = np.array([z_level[k] - z_level[k - 1] for k in range(1, L + 1)])
    dzmin = float(delta_z.min())
    if np.any(np.abs(z_level[1:] - params.msl) < 1e-5):
        raise ValueError("a z_level coincides with MSL (read_main_inp.f90 card C2_1)")
    params.delta_z_min = dzmin
    # card C5_03: min(dry_depth*(0.5-1.0e-4), delta_z_min*(0.5-1.e-4)), the bracket being a
    # default-REAL constant expression
    c = f32(np.float32(0.5) - np.float32(1.0e-4))
    params.denominator_min_for_matrix = min(params.dry_depth * c, dzmin * c)
    return L, delta_z


def _face_constants(a, nf, params, coriolis_on):
    # calculate_coriolis_factor.f90:17-23 (option 1): omega is a default-REAL literal
    omega = f32(7.292e-5)
    a["coriolis_factor"] = np.full(nf, 2 * omega * math.sin(params.coriolis_lat * DEG2RAD) if coriolis_on else 0.0)
    a["manning"] = np.full(nf, params.manning)
    a["bf_height"] = np.full(nf, params.bf_height)


def _finish_device(name, raw, z_level, params, ob_pairs, q_pairs, q_portion, voronoi, max_nb, coriolis_on, lib,
                   **kw) -> Deck:
    L, delta_z = _vertical(z_level, params)
    a, nf, ids = _device_geometry(lib, raw, z_level, params.msl, ob_pairs, q_pairs, voronoi, max_nb)
    _face_constants(a, nf, params, coriolis_on)
    return Deck(name=name, geo=a, n_nodes=len(raw.x), n_cells=len(raw.tri_or_quad), n_faces=nf, n_layers=L,
                max_nb=max_nb, params=params, z_level=z_level, delta_z=delta_z,
                ob_cell_id=ids["ob_cell_id"], ob_face_id=ids["ob_face_id"], qb_cell=ids["qb_cell"],
                qb_face=ids["qb_face"], q_portion=np.asarray(q_portion, dtype=np.float64), **kw)


# ----------------------------------------------------------------------------- configurations
def tidal_basin(nx: int = 120, ny: int = 80, dx: float = 250.0, tri_rows: int = 4, n_layers: int = 10,
                seed: int = 20240601, n_steps: int = 720, dt: float = 120.0, closed: bool = False,
                geometry_lib=None) -> Deck:
    """Barotropic tidal basin: h = 5 + 15(1 - y/Ly) + seeded Fourier noise (8 modes,
    2-15 km, 1 m), southern open boundary forced by 0.5 cos(2 pi t / 44712 s), closed
    elsewhere, uniform T = 20, S = 30, theta = 0.6, quadratic drag Cd = 0.0025."""
    rng = np.random.default_rng(seed)
    x, y, cells, tq = square_strip_mesh(nx, ny, dx, tri_rows)
    ly = float(y.max())
    scale = dx / 250.0
    h = 5.0 + 15.0 * (1.0 - y / ly) + fourier_noise(x, y, rng, lam_min=2000.0 * scale, lam_max=15000.0 * scale)
    raw = RawMesh(x=x, y=y, h=h, tri_or_quad=tq, cells=cells)
    params = Params(dt=dt, theta=0.6, error_tolerance=1e-10, baroclinic_flag=0,
                    trans_sub_iter=1, h_flux_limiter=0, v_flux_limiter=0)
    # open boundary: south edge, node pairs (SW, SE) of the first row of squares (none if closed)
    ob_pairs = [] if closed else [(i + 1, i + 2) for i in range(nx)]
    L = n_layers
    hmax = float(h.max())
    z_bottom = -math.ceil(hmax + 1.0)
    z_top = 3.0
    deck = _finish("tidal_basin", raw, L, z_bottom, z_top, params, ob_pairs, [], [],
                   tide=dict(amplitude=[0.5], period_h=[12.42], phase=[0.0], nodal=[1.0], eq_arg=[0.0],
                             shift=0.0),
                   ob_salt=30.0, ob_temp=20.0, n_steps=n_steps, seed=seed, geometry_lib=geometry_lib)
    deck.init_salt_node = np.full((deck.n_nodes, L), 30.0)
    deck.init_temp_node = np.full((deck.n_nodes, L), 20.0)
    deck.meta = dict(nx=nx, ny=ny, dx=dx, tri_rows=tri_rows)
    return deck


def estuary(nx: int = 600, ny: int = 250, dx: float = 100.0, tri_rows: int = 4, n_layers: int = 20,
            seed: int = 20240602, n_steps: int = 2880, dt: float = 60.0, n_river: int = 10,
            trans_sub_iter: int = 4, turbulence_flag: int = 2, geometry_lib=None) -> Deck:
    """Baroclinic estuary: ocean open boundary on the west edge (M2 0.6 m, S = 35, T = 18),
    river of 500 m3/s at S = 0, T = 24 over ``n_river`` faces of the east edge (channel head),
    initial salinity linear along the channel, TVD limiter on, turbulence closure on
    (Pacanowski-Philander), uniform wind stress 0.1 Pa at a seeded direction.

    The north coast is a seeded sinusoid: the ``tri_rows`` rows of triangles between the squares
    and the coast follow it (strip height 0.7-1.3 times the equilateral one, so every triangle is
    oblique and acute).  Along the coast an intertidal flat six cells wide rises from 0.9 m to
    0.15 m below MSL, so a band of cells falls dry and floods again with the 0.6 m tide; seaward
    of the flat the bed deepens to the estuary's along-channel profile."""
    rng = np.random.default_rng(seed)
    x, y, cells, tq = square_strip_mesh(nx, ny, dx, tri_rows)
    lx = nx * dx
    y0 = ny * dx
    strip = tri_rows * dx * math.sqrt(3.0) / 2.0
    # the coast's wavelength stays at least 40 cells, so the strip varies slowly over a cell
    lam = max(rng.uniform(0.2, 0.5) * lx, 40.0 * dx)
    phase = rng.uniform(0, 2 * math.pi)

    def coast(xx):
        return y0 + strip * (1.0 + 0.3 * np.sin(2 * math.pi * xx / lam + phase))

    if tri_rows > 0:
        y = coastal_strip(x, y, y0, strip, coast)
    yc = coast(x) if tri_rows > 0 else np.full_like(x, y0)
    ly = float(y.max())
    # depth: the along-channel profile of the estuary seaward of the flat, the flat from 0.9 m
    # to 0.15 m at the coast (land above MSL makes the reference stop: a wet cell whose sides
    # are all dry, update_vertical_layers_1.f90)
    flat = 6.0 * dx
    dist = np.maximum(yc - y, 0.0)
    h_deep = 4.0 + 15.0 * (1.0 - x / lx)
    w = np.clip((dist - flat) / (0.25 * ly), 0.0, 1.0) ** 0.7
    h = np.where(dist < flat, 0.15 + 0.75 * dist / flat, 0.9 + (h_deep - 0.9) * w)
    h = h + fourier_noise(x, y, rng, lam_min=800.0, lam_max=6000.0, amplitude=0.5) * w
    raw = RawMesh(x=x, y=y, h=h, tri_or_quad=tq, cells=cells)
    params = Params(dt=dt, theta=0.6, error_tolerance=1e-10, baroclinic_flag=1, ana_density=0,
                    trans_sub_iter=trans_sub_iter, h_flux_limiter=1, v_flux_limiter=1,
                    smagorinsky=0.021, kh_0=0.1, av_0=1e-3, kv_0=1e-5, turbulence_flag=turbulence_flag)
    # west edge: faces NW -> SW of squares in column 0, i.e. node (0, j+1) -> (0, j)
    row = nx + 1
    ob_pairs = [((j + 1) * row + 1, j * row + 1) for j in range(ny)]
    # river: east edge faces SE -> NE of column nx-1, centred rows
    n_river = max(1, min(n_river, ny - 2))
    j0 = ny // 2 - n_river // 2
    q_pairs = [(j * row + nx + 1, (j + 1) * row + nx + 1) for j in range(j0, j0 + n_river)]
    q_portion = [1.0 / n_river] * n_river
    hmax = float(h.max())
    z_bottom = -math.ceil(hmax + 1.0)
    z_top = 3.0
    # no level within a quarter layer of MSL (read_main_inp.f90 card C2_1 rejects a level at MSL)
    while np.any(np.abs(uniform_z_levels(z_bottom, z_top, n_layers)[0]) < 0.25 * (z_top - z_bottom) / n_layers):
        z_top += 0.25
    alpha = rng.uniform(0.0, 2.0 * math.pi)
    tau = 0.1
    deck = _finish("estuary", raw, n_layers, z_bottom, z_top, params, ob_pairs, q_pairs, q_portion,
                   tide=dict(amplitude=[0.6], period_h=[12.42], phase=[0.0], nodal=[1.0], eq_arg=[0.0],
                             shift=0.0),
                   ob_salt=35.0, ob_temp=18.0, q_total=500.0, q_salt=0.0, q_temp=24.0,
                   wind_stress=(tau * math.cos(alpha), tau * math.sin(alpha)),
                   n_steps=n_steps, seed=seed, geometry_lib=geometry_lib)
    L = n_layers
    s = 35.0 * (1.0 - x / lx)
    t = 18.0 + 6.0 * (x / lx)
    deck.init_salt_node = np.repeat(s[:, None], L, axis=1)
    deck.init_temp_node = np.repeat(t[:, None], L, axis=1)
    deck.meta = dict(nx=nx, ny=ny, dx=dx, tri_rows=tri_rows, wind_dir=alpha)
    return deck


# ----------------------------------------------------------------------------- initial state
def initial_state(deck: Deck, eta0: np.ndarray | None = None) -> dict:
    """State after prepare_gom.f90 for a cold start: setup_cold_start.f90 (zero elevation and
    velocity), update_vertical_layers_0.f90 (layers and thicknesses), read_salt_init.f90 /
    read_temp_init.f90 (tracers), read_main_inp.f90 card C5_04 (Av, Kv) and C5_01
    (num_sub_elm_iteration)."""
    a = deck.geo
    p = deck.params
    L = deck.n_layers
    nc, nf, nn = deck.n_cells, deck.n_faces, deck.n_nodes
    z = deck.z_level
    dzl = deck.delta_z
    msl = p.msl
    st: dict = {}
    eta_cell_new = np.zeros(nc) if eta0 is None else np.asarray(eta0, dtype=np.float64).copy()
    if eta0 is None:
        eta_node = np.zeros(nn)
    else:
        # node elevation = area-weighted mean of its cells (solve_free_surface_equation.f90:353-373)
        num = np.zeros(nn)
        den = np.zeros(nn)
        for l in range(4):
            m = l < a["tri_or_quad"]
            nd = a["nodenum_at_cell"][m, l] - 1
            np.add.at(num, nd, a["area"][m] * eta_cell_new[m])
            np.add.at(den, nd, a["area"][m])
        eta_node = num / den

    def column(h, eta, bottom, with_edges):
        """update_vertical_layers_0.f90:42-140 (cells, with_edges=False) and :146-263, for all
        entities at once with the same per-element arithmetic."""
        n = len(h)
        h = np.asarray(h, dtype=np.float64)
        eta = np.asarray(eta, dtype=np.float64)
        b = np.asarray(bottom, dtype=np.int64)
        total = h + eta
        tmp = msl + eta
        wet = total > p.dry_depth
        t = np.searchsorted(z, tmp, side="left")        # count of z_level below tmp
        t = np.where(wet & (t >= 1) & (t <= L), t, 0)
        if np.any(wet & (t < b)):
            raise ValueError("impossible elevation at start (update_vertical_layers_0.f90:66-81)")
        dz = np.zeros((n, L))
        dzh = np.zeros((n, L + 1))
        single = np.nonzero(wet & (t == b))[0]
        multi = np.nonzero(wet & (t > b))[0]
        tm, bm = t[multi], b[multi]
        dz[multi, tm - 1] = tmp[multi] - z[tm - 1]
        dz[multi, bm - 1] = z[bm] - (msl - h[multi])
        K = np.arange(1, L + 1)[None, :]
        mid = np.zeros((n, L), bool)
        mid[multi] = (K > bm[:, None]) & (K < tm[:, None])
        dz[mid] = np.broadcast_to(dzl[None, :], (n, L))[mid]
        half = np.zeros((n, L + 1))
        half[:, 1:L] = (dz[:, 1:] + dz[:, :-1]) * 0.5
        KK = np.arange(L + 1)[None, :]
        inner = np.zeros((n, L + 1), bool)
        inner[multi] = (KK >= bm[:, None]) & (KK <= tm[:, None] - 1)
        dzh[inner] = half[inner]
        if with_edges in ("face", "node"):
            dzh[multi, tm] = dz[multi, tm - 1]
            dzh[multi, bm - 1] = dz[multi, bm - 1]
        ts = t[single]
        dz[single, ts - 1] = total[single]
        if with_edges == "face":
            dzh[single, ts - 1] = total[single]
        dzh[single, ts] = total[single]
        return t.astype(np.int32), dz, dzh

    top_c, dz_c, dzh_c = column(a["h_cell"], eta_cell_new, a["bottom_layer_at_element"], "cell")
    eta_face = eta_cell_new[a["adj_cellnum_at_face"][:, 0] - 1].copy()
    inner = a["adj_cellnum_at_face"][:, 1] != 0
    e2 = eta_cell_new[np.maximum(a["adj_cellnum_at_face"][:, 1], 1) - 1]
    eta_face = np.where(inner, np.maximum(eta_face, e2), eta_face)
    top_f, dz_f, dzh_f = column(a["h_face"], eta_face, a["bottom_layer_at_face"], "face")
    top_n, dz_n, dzh_n = column(a["h_node"], eta_node, a["bottom_layer_at_node"], "node")
    # dry element if all its nodes are dry (update_vertical_layers_0.f90:270-286)
    tq = a["tri_or_quad"]
    nsum1 = np.zeros(nc, np.int64)
    nsum2 = np.zeros(nc, np.int64)
    for l in range(4):
        m = l < tq
        nsum1[m] += top_n[a["nodenum_at_cell"][m, l] - 1]
        nsum2[m] += top_f[a["facenum_at_cell"][m, l] - 1]
    top_c = np.where(nsum1 == 0, 0, top_c).astype(np.int32)
    if np.any((nsum2 == 0) & (top_c != 0)):
        raise ValueError("wet element with dry sides at start")

    st["eta_cell"] = eta_cell_new.copy()
    st["eta_cell_new"] = eta_cell_new
    st["eta_node"] = eta_node
    st["wetdry_node"] = np.zeros(nn, np.int32)
    for k in ("un_face", "vn_face", "un_face_new", "vn_face_new", "un_elm", "vn_elm",
              "ainvg1", "ainvg2", "ainvdz1", "ainvdz2", "kh"):
        st[k] = np.zeros((nf, L))
    for k in ("wn_cell", "wn_cell_new"):
        st[k] = np.zeros((nc, L + 1))
    for k in ("u_node", "v_node", "w_node"):
        st[k] = np.zeros((nn, L + 1))
    for k in ("u_face_level", "v_face_level"):
        st[k] = np.zeros((nf, L + 1))
    st["dz_cell"], st["dz_cell_new"] = dz_c, np.zeros_like(dz_c)
    st["dzhalf_cell"], st["dzhalf_cell_new"] = dzh_c, np.zeros_like(dzh_c)
    st["dz_face"], st["dz_face_new"] = dz_f, np.zeros_like(dz_f)
    st["dzhalf_face"], st["dzhalf_face_new"] = dzh_f, np.zeros_like(dzh_f)
    st["dz_node"], st["dz_node_new"] = dz_n, np.zeros_like(dz_n)
    st["dzhalf_node"], st["dzhalf_node_new"] = dzh_n, np.zeros_like(dzh_n)
    st["top_layer_cell"], st["top_layer_face"], st["top_layer_node"] = top_c, top_f, top_n
    av = np.zeros((nf, L + 1))
    av[:, 1:] = p.av_0
    kv = np.zeros((nc, L + 1))
    kv[:, 1:] = p.kv_0
    st["av"], st["kv"] = av, kv
    # tracers: read_salt_init.f90:25-53 (node values -> faces -> cells)
    n1 = a["nodenum_at_face"][:, 0] - 1
    n2 = a["nodenum_at_face"][:, 1] - 1

    def tracer(node_vals, fill):
        if node_vals is None:
            return (np.full((nc, L), fill), np.full((nn, L), fill), np.full((nf, L), fill))
        face = (node_vals[n1] + node_vals[n2]) * 0.5
        cell = np.zeros((nc, L))
        for l in range(4):
            m = l < tq
            cell[m] = cell[m] + node_vals[a["nodenum_at_cell"][m, l] - 1]
        cell = cell / tq[:, None]
        return cell, node_vals.copy(), face

    if p.is_salt:
        sc, sn, sf = tracer(deck.init_salt_node, p.ref_salt)
    else:
        sc, sn, sf = tracer(None, p.ref_salt if p.baroclinic_flag else 0.0)
    if p.is_temp:
        tc, tn, tf = tracer(deck.init_temp_node, p.ref_temp)
    else:
        tc, tn, tf = tracer(None, p.ref_temp if p.baroclinic_flag else 20.0)
    st["salt_cell"], st["salt_cell_new"], st["salt_node"], st["salt_face"] = sc, sc.copy(), sn, sf
    st["temp_cell"], st["temp_cell_new"], st["temp_node"], st["temp_face"] = tc, tc.copy(), tn, tf
    for k, n in (("rho_cell", nc), ("rho_node", nn), ("rho_face", nf)):
        st[k] = np.zeros((n, L))
    if p.elm_backtrace_flag == 0:
        st["num_sub_elm"] = np.full((nn, L), p.elm_sub_iter, np.int32)
    elif p.elm_backtrace_flag == 1:
        st["num_sub_elm"] = np.ones((nn, L), np.int32)
    else:
        st["num_sub_elm"] = np.zeros((nn, L), np.int32)
    st["cdb"] = np.zeros(nf)
    st["gamma_b"] = np.zeros(nf)
    return st


def active_cell_layers(deck: Deck, state: dict) -> int:
    """Sum over wet cells of (top - bottom + 1) at t = 0: the cell-layer count of the metric."""
    top = state["top_layer_cell"]
    bot = deck.geo["bottom_layer_at_element"]
    return int(np.sum(np.where(top > 0, top - bot + 1, 0)))


# ----------------------------------------------------------------------------- host forcing
class HostForcing:
    """Per-step forcing the Fortran driver computes on the host before the core runs."""

    def __init__(self, deck: Deck):
        self.deck = deck
        p = deck.params
        self.nt = max(p.trans_sub_iter, 1)
        self.julian_day = 0.0
        nf = deck.n_faces
        a = deck.geo
        tx, ty = deck.wind_stress
        # ana_windp.f90:18-35 with an arbitrary direction: kinematic stress = stress / 1000
        rw2 = 1.0 / 1000.0
        self.wind_normal = (tx * a["cos_theta"] + ty * a["sin_theta"]) * rw2
        self.wind_tangnt = (-tx * a["sin_theta"] + ty * a["cos_theta"]) * rw2
        self.gamma_t = np.zeros(nf)
        self.first = True

    def spinup_tide(self, elapsed):
        """setup_spinup.f90:22-31."""
        period = self.deck.tide_spinup_days * 86400.0
        if period <= 0.0 or elapsed >= period:
            return 1.0
        return math.tanh(2.0 * elapsed / period)

    def eta_ob(self, elapsed, spin):
        """compute_boundary_eta.f90:72-90 (ob_eta_type 1, harmonic), in the reference's order of
        operations: ((spin amp) nodal) cos(((w t + eq) - phase) - shift)."""
        d = self.deck
        if d.n_ob == 0:
            return np.zeros(0), np.zeros(0)
        tide = d.tide
        dt = d.params.dt
        old = 0.0
        new = 0.0
        for j in range(len(tide["amplitude"])):
            w = 2.0 * PI / (tide["period_h"][j] * 3600.0)
            eq, ph, sh = tide["eq_arg"][j] * DEG2RAD, tide["phase"][j] * DEG2RAD, tide["shift"] * DEG2RAD
            a = spin * tide["amplitude"][j] * tide["nodal"][j]
            old = old + a * math.cos(w * (elapsed - dt) + eq - ph - sh)
            new = new + a * math.cos(w * elapsed + eq - ph - sh)
        return np.full(d.n_ob, old), np.full(d.n_ob, new)

    def step(self, it: int) -> dict:
        d = self.deck
        p = d.params
        elapsed = it * p.dt
        self.julian_day = self.julian_day + p.dt / 86400.0
        spin = self.spinup_tide(elapsed)
        spin_bc = 1.0
        old, new = self.eta_ob(elapsed, spin)
        out = dict(elapsed_time=elapsed, spinup_tide=spin, spinup_baroclinic=spin_bc,
                   eta_at_ob_old=old, eta_at_ob_new=new)
        if d.n_qb:
            out["q_add"] = d.q_total * d.q_portion        # calculate_Q.f90:36-42, constant series
        # boundary concentrations per subcycle, (n, 2, Nt): slot 1 salt, slot 2 temperature
        nt = self.nt
        cob = np.zeros((d.n_ob, 2, nt))
        if d.ob_salt is not None:
            cob[:, 0, :] = spin_bc * d.ob_salt
        if d.ob_temp is not None:
            cob[:, 1, :] = spin_bc * d.ob_temp
        out["con_at_ob"] = cob
        if d.n_qb:
            cqb = np.zeros((d.n_qb, 2, nt))
            if d.q_salt is not None:
                cqb[:, 0, :] = spin_bc * d.q_salt
            if d.q_temp is not None:
                cqb[:, 1, :] = spin_bc * d.q_temp
            out["con_at_qb"] = cqb
        if self.first:
            out.update(self.static())
            self.first = False
        return out

    def static(self) -> dict:
        """Forcing that stays constant over the run (uploaded once)."""
        return dict(wind_stress_normal=self.wind_normal, wind_stress_tangnt=self.wind_tangnt, gamma_t=self.gamma_t)

    def full(self, it: int) -> dict:
        """Step forcing plus the constant arrays, for a context that has not seen earlier steps."""
        out = self.step(it)
        out.update(self.static())
        return out
