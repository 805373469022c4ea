"""Storm-surge ensembles: many independent runs advanced together in one context.

``storm_run``  generates one run: the square/triangle-strip generator of the tidal basin on a
               seeded domain (cell count and aspect ratio given), a shelf deepening towards the
               southern open boundary, an M2 tide on that boundary and a parametric Holland
               vortex crossing the domain on a straight track.  All runs of an ensemble share
               one z-level grid (1 m levels), so a run's depth sets how many layers it uses.
``pack``       joins runs into one deck whose mesh is the disjoint union of theirs: entity ids
               are offset run by run (each run's cells, faces, nodes and boundary cells stay
               contiguous) and ``deck.runs`` records where each run starts.  The C ABI then
               advances every run in one launch per phase, with one PCG per run.
``StormForcing``  the per-step host forcing of one run (tide, spin-up, Holland wind stress and
               air pressure) -- the reference's calculate_wind_stress.f90:105-137 drag law on
               winds from the vortex of holland_storm_surge.f90:131-232 generalised to a
               Holland B exponent.
``PackedForcing`` concatenates the runs' host forcing for a packed deck.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .deck import Deck, HostForcing, Params, RawMesh, _finish, square_strip_mesh, fourier_noise

AIR_DENSITY = 1.293          # holland_storm_surge.f90:27
GRADIENT_TO_SURFACE = 0.95   # holland_storm_surge.f90:28
INFLOW_DEG = 18.0            # holland_storm_surge.f90:18
P_FAR = 101300.0             # Pa, holland_storm_surge.f90:29 (1013 hPa)
M2_PERIOD_H = 12.42


def ensemble_z_grid(max_layers: int = 30):
    """Shared vertical grid of an ensemble: 1 m levels from -(max_layers + 0.5) m to +10.5 m, room
    for surge + tide above MSL (no level at MSL, read_main_inp.f90 card C2_1).  The slow, wide
    vortices of the range (Rmax 40 km at 4-5 m/s) pile more than 6 m of surge against the
    shallow northern coast; an elevation above the top level stops the run
    (update_vertical_layers_1.f90)."""
    return -float(max_layers) - 0.5, 10.5, max_layers + 11


@dataclasses.dataclass
class Storm:
    """Holland vortex on a straight track and the run's M2 tide (SI units)."""

    x0: float
    y0: float
    heading: float       # radians from +x
    speed: float         # m/s
    rmax: float          # m
    dp: float            # Pa, central pressure deficit (> 0)
    b: float             # Holland B
    coriolis: float      # 1/s
    tide_amplitude: float
    tide_period: float   # s
    tide_phase: float    # rad
    spinup: float        # s, tanh ramp of tide and wind (setup_spinup.f90:22-31)
    t0: float = 0.0      # context elapsed time at which the run's clock starts


def storm_run(seed: int, n_cells: int, aspect: float, n_layers_run: int, dt: float = 60.0,
              dx: float = 250.0, max_layers: int = 30, tri_rows: int = 2, h_coast: float = 2.0,
              h_min: float = 1.0, av_0: float = 0.5, open_sides: bool = False) -> Deck:
    """One storm-surge run of about ``n_cells`` cells, domain aspect ``aspect`` (x / y), deepest
    water using ``n_layers_run`` of the shared 1 m levels; the shelf rises to ``h_coast`` at the
    closed northern coast, depths at least ``h_min``.

    The vertical eddy viscosity ``av_0`` (m^2/s) is a storm-surge value.  With a constant Av the
    steady shear under a surface stress tau is du/dz = tau / (rho Av), so the column's top-to-
    bottom velocity difference is tau h / (rho Av): a 68 m/s Holland wind gives a kinematic stress
    Gamma_T W = 0.003 (rho_a / rho_o) W^2 = 0.017 m^2/s^2 (calculate_wind_stress.f90:105-137), i.e.
    6 m/s over 18 m of water at Av = 0.05 and 0.6 m/s at Av = 0.5, on top of the bottom-drag
    speed sqrt(tau / Cd) = 2.6 m/s where the wind drives flow through the clamped open boundary.
    At 1e-3 (a calm estuary's value) the surface layer decouples from the column altogether."""
    rng = np.random.default_rng(seed)
    ny = max(6, int(round(math.sqrt(n_cells / aspect))))
    nx = max(6, int(round(n_cells / ny)) - tri_rows)
    x, y, cells, tq = square_strip_mesh(nx, ny, dx, tri_rows)
    ly = float(y.max())
    lx = nx * dx
    hmax = min(float(n_layers_run) - 1.5, max_layers - 1.5)
    shelf = (1.0 - y / ly) ** 1.3
    h = h_coast + (hmax - h_coast) * shelf
    lam = max(4.0 * dx, 0.25 * min(lx, ly))
    h = h + fourier_noise(x, y, rng, lam_min=lam, lam_max=4.0 * lam, amplitude=0.3)
    h = np.clip(h, h_min, hmax)
    raw = RawMesh(x=x, y=y, h=h, tri_or_quad=tq, cells=cells)
    params = Params(dt=dt, theta=0.6, error_tolerance=1e-10, baroclinic_flag=0, trans_sub_iter=1,
                    h_flux_limiter=0, v_flux_limiter=0, cd_const=0.0025, bf_flag=3, av_0=av_0)
    z_bottom, z_top, L = ensemble_z_grid(max_layers)
    ob_pairs = [(i + 1, i + 2) for i in range(nx)]         # southern edge
    if open_sides:
        # western and eastern edges of the square rows above the southern corner cells
        for jrow in range(1, ny):
            ob_pairs.append(((jrow + 1) * (nx + 1) + 1, jrow * (nx + 1) + 1))
            ob_pairs.append((jrow * (nx + 1) + nx + 1, (jrow + 1) * (nx + 1) + nx + 1))
    amp = float(rng.uniform(0.3, 0.8))
    deck = _finish("storm_run", raw, L, z_bottom, z_top, params, ob_pairs, [], [],
                   tide=dict(amplitude=[amp], period_h=[M2_PERIOD_H], phase=[0.0], nodal=[1.0],
                             eq_arg=[0.0], shift=0.0),
                   ob_salt=30.0, ob_temp=20.0, seed=seed)
    deck.init_salt_node = np.full((deck.n_nodes, L), 30.0)
    deck.init_temp_node = np.full((deck.n_nodes, L), 20.0)
    # vortex: enters through the southern boundary and crosses the domain in about 18 h
    speed = float(rng.uniform(3.0, 8.0))
    heading = math.pi / 2 + float(rng.uniform(-0.6, 0.6))
    travel = speed * 18 * 3600.0
    xc = lx * float(rng.uniform(0.3, 0.7))
    storm = Storm(x0=xc - 0.5 * travel * math.cos(heading), y0=ly * 0.5 - 0.5 * travel * math.sin(heading),
                  heading=heading, speed=speed, rmax=float(rng.uniform(20e3, 60e3)),
                  dp=float(rng.uniform(20e2, 80e2)), b=float(rng.uniform(1.0, 1.8)),
                  coriolis=2 * 7.292e-5 * math.sin(math.radians(float(rng.uniform(20.0, 35.0)))),
                  tide_amplitude=amp, tide_period=M2_PERIOD_H * 3600.0, tide_phase=float(rng.uniform(0, 2 * math.pi)),
                  spinup=0.25 * 86400.0)
    deck.tide_spinup_days = storm.spinup / 86400.0
    deck.meta = dict(nx=nx, ny=ny, dx=dx, tri_rows=tri_rows, storm=storm, n_layers_run=n_layers_run,
                     aspect=aspect)
    return deck


def ensemble_decks(n_runs: int = 96, seed: int = 7, min_cells: int = 5000, max_cells: int = 400000,
                   dt: float = 60.0, max_layers: int = 30, dx: float = 250.0, h_coast: float = 2.0,
                   h_min: float = 1.0, open_sides: bool = False):
    """Runs with cell counts log-uniform in [min_cells, max_cells], aspect 1-4, 10-30 layers."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_runs):
        n = int(math.exp(rng.uniform(math.log(min_cells), math.log(max_cells))))
        aspect = float(rng.uniform(1.0, 4.0))
        layers = int(rng.integers(10, max_layers + 1))
        out.append(storm_run(int(rng.integers(1 << 30)), n, aspect, layers, dt=dt, dx=dx, max_layers=max_layers,
                             h_coast=h_coast, h_min=h_min, open_sides=open_sides))
    return out


# ----------------------------------------------------------------------------- packing
_CELL_IDS = {"nodenum_at_cell": "node", "facenum_at_cell": "face", "adj_cellnum_at_cell": "cell"}
_FACE_IDS = {"adj_cellnum_at_face": "cell", "nodenum_at_face": "node"}
_NODE_IDS = {"adj_cellnum_at_node": "cell", "adj_nodenum_at_node": "node"}


def pack(decks: list[Deck], name: str = "packed") -> Deck:
    """One deck holding every run's mesh as a disjoint part of one mesh."""
    d0 = decks[0]
    for d in decks[1:]:
        if not (np.array_equal(d.z_level, d0.z_level) and d.params == d0.params):
            raise ValueError("packed runs need the same vertical grid and parameters")
    nb = max(d.max_nb for d in decks)
    off = {"cell": 0, "face": 0, "node": 0, "ob": 0, "qb": 0}
    starts = {k: [0] for k in ("cell", "face", "node", "ob")}
    geo: dict[str, list] = {k: [] for k in d0.geo}
    ob_cell, ob_face, qb_cell, qb_face, q_add = [], [], [], [], []
    salt, temp = [], []
    for d in decks:
        g = d.geo
        for k, v in g.items():
            v = np.asarray(v)
            if k in _CELL_IDS or k in _FACE_IDS or k in _NODE_IDS:
                kind = _CELL_IDS.get(k) or _FACE_IDS.get(k) or _NODE_IDS.get(k)
                v = np.where(v != 0, v + off[kind], 0).astype(np.int32)
            elif k == "ob_element_flag":
                v = np.where(v > 0, v + off["ob"], 0).astype(np.int32)
            elif k == "qb_element_flag":
                v = np.where(v > 0, v + off["qb"], 0).astype(np.int32)
            elif k == "boundary_type_of_face":
                v = np.where(v > 0, v + off["ob"], v).astype(np.int32)
            elif k == "isflowside3":
                v = np.where(v > 0, v + off["qb"], 0).astype(np.int32)
            if k in ("adj_cellnum_at_node", "node_count_each_element") and v.shape[1] < nb:
                v = np.pad(v, ((0, 0), (0, nb - v.shape[1])))
            if k == "adj_nodenum_at_node" and v.shape[1] < nb + 1:
                v = np.pad(v, ((0, 0), (0, nb + 1 - v.shape[1])))
            geo[k].append(v)
        ob_cell.append(d.ob_cell_id + off["cell"])
        ob_face.append(d.ob_face_id + off["face"])
        qb_cell.append(d.qb_cell + off["cell"])
        qb_face.append(d.qb_face + off["face"])
        q_add.append(d.q_total * d.q_portion)
        salt.append(d.init_salt_node)
        temp.append(d.init_temp_node)
        off["cell"] += d.n_cells
        off["face"] += d.n_faces
        off["node"] += d.n_nodes
        off["ob"] += d.n_ob
        off["qb"] += d.n_qb
        for k in starts:
            starts[k].append(off[k])
    geo = {k: np.concatenate(v) for k, v in geo.items()}
    deck = Deck(name=name, geo=geo, n_nodes=off["node"], n_cells=off["cell"], n_faces=off["face"],
                n_layers=d0.n_layers, max_nb=nb, params=dataclasses.replace(d0.params),
                z_level=d0.z_level.copy(), delta_z=d0.delta_z.copy(),
                ob_cell_id=np.concatenate(ob_cell).astype(np.int32), ob_face_id=np.concatenate(ob_face).astype(np.int32),
                qb_cell=np.concatenate(qb_cell).astype(np.int32), qb_face=np.concatenate(qb_face).astype(np.int32),
                q_portion=np.concatenate(q_add), q_total=1.0, tide=d0.tide, ob_salt=d0.ob_salt,
                ob_temp=d0.ob_temp, n_steps=d0.n_steps, seed=d0.seed,
                init_salt_node=None if any(s is None for s in salt) else np.concatenate(salt),
                init_temp_node=None if any(t is None for t in temp) else np.concatenate(temp))
    deck.runs = {f"run_{k}_start": np.asarray(v, dtype=np.int32) for k, v in starts.items()}
    deck.meta = dict(members=decks)
    return deck


def split(deck: Deck, name: str, values: np.ndarray) -> list[np.ndarray]:
    """A packed field's values run by run (``name`` as in ``GomCore.get_field``)."""
    from .core import field_kind
    kind = field_kind(name)
    s = deck.runs[f"run_{kind}_start"]
    n_ent = {"cell": deck.n_cells, "face": deck.n_faces, "node": deck.n_nodes, "ob": deck.n_ob}[kind]
    per = values.size // n_ent
    return [values[s[r] * per:s[r + 1] * per] for r in range(len(s) - 1)]


# ----------------------------------------------------------------------------- forcing
def holland_node_wind(storm: Storm, t: float, x: np.ndarray, y: np.ndarray):
    """Surface wind (u, v) and air pressure (Pa) at points (x, y) at time t:
    holland_storm_surge.f90:131-221 with the exponent B of Holland (1980):
    V_c^2 = B dp/rho_a (Rmax/r)^B exp(-(Rmax/r)^B), p = p_far - dp (1 - exp(-(Rmax/r)^B))."""
    xe = storm.x0 + storm.speed * t * math.cos(storm.heading)
    ye = storm.y0 + storm.speed * t * math.sin(storm.heading)
    dxh = x - xe
    dyh = y - ye
    r = np.sqrt(dxh * dxh + dyh * dyh)
    r = np.maximum(r, 1.0)
    a = (storm.rmax / r) ** storm.b
    e = np.exp(-a)
    vc2 = storm.b * storm.dp / AIR_DENSITY * a * e
    vc = np.sqrt(vc2)
    theta = np.arctan2(dyh, dxh) - storm.heading
    vg = vc2 / (r * storm.coriolis)
    with np.errstate(divide="ignore", invalid="ignore"):
        gamma = 0.5 * (storm.speed * np.sin(theta) / vc + vc / vg)
        v = np.where(vc < 1e-3, 0.0, vc * (np.sqrt(gamma * gamma + 1.0) - gamma) * GRADIENT_TO_SURFACE)
    ang = 0.5 * math.pi + theta + storm.heading + math.radians(INFLOW_DEG)
    return v * np.cos(ang), v * np.sin(ang), P_FAR - storm.dp * (1.0 - e)


def face_wind_stress(deck: Deck, un: np.ndarray, vn: np.ndarray, rho_o: float, spin: float):
    """calculate_wind_stress.f90:105-137 (wind_formular 1, Cd <= 0.003) from node winds."""
    g = deck.geo
    n1 = g["nodenum_at_face"][:, 0] - 1
    n2 = g["nodenum_at_face"][:, 1] - 1
    u = (un[n1] + un[n2]) / 2.0
    v = (vn[n1] + vn[n2]) / 2.0
    speed = np.sqrt(u * u + v * v)
    normal = u * g["cos_theta"] + v * g["sin_theta"]
    tangent = -u * g["sin_theta"] + v * g["cos_theta"]
    cda = np.minimum(0.001 * (0.75 + 0.067 * speed), float(np.float32(0.003)))   # a default-REAL 0.003
    gamma_t = cda * (AIR_DENSITY / rho_o) * speed
    return gamma_t * normal * spin, gamma_t * tangent * spin, gamma_t


class StormForcing(HostForcing):
    """Host forcing of one storm run: tide + inverse-barometer set-up at the open boundary,
    Holland wind stress and air pressure, with the run's spin-up."""

    def __init__(self, deck: Deck):
        super().__init__(deck)
        self.storm: Storm = deck.meta["storm"]
        self.gamma_t = np.zeros(deck.n_faces)

    def spin(self, t: float) -> float:
        s = self.storm
        return 1.0 if t >= s.spinup else math.tanh(2.0 * t / s.spinup)

    def ob_elevation(self, t: float) -> np.ndarray:
        s = self.storm
        d = self.deck
        cells = d.ob_cell_id - 1
        x = d.geo["x_cell"][cells]
        y = d.geo["y_cell"][cells]
        _, _, p = holland_node_wind(s, t, x, y)
        ib = (P_FAR - p) / (d.params.rho_o * d.params.gravity)
        return self.spin(t) * (s.tide_amplitude * np.cos(2 * math.pi * t / s.tide_period + s.tide_phase) + ib)

    def step(self, it: int) -> dict:
        d = self.deck
        p = d.params
        t = it * p.dt
        out = super().step(it)
        spin = self.spin(t)
        out["spinup_tide"] = spin
        out["eta_at_ob_old"] = self.ob_elevation(t - p.dt)
        out["eta_at_ob_new"] = self.ob_elevation(t)
        u, v, pa = holland_node_wind(self.storm, t, d.geo["x_node"], d.geo["y_node"])
        wsn, wst, gt = face_wind_stress(d, u, v, p.rho_o, spin)
        out.update(wind_stress_normal=wsn, wind_stress_tangnt=wst, gamma_t=gt, air_p=pa)
        return out


class PackedForcing:
    """Host forcing of a packed deck: each run's forcing, concatenated in run order."""

    def __init__(self, deck: Deck):
        self.deck = deck
        self.parts = [StormForcing(d) if "storm" in d.meta else HostForcing(d) for d in deck.meta["members"]]
        self.first = True

    def step(self, it: int) -> dict:
        outs = [f.step(it) for f in self.parts]
        res = {k: outs[0][k] for k in ("elapsed_time", "spinup_tide", "spinup_baroclinic")}
        for k in outs[0]:
            if isinstance(outs[0][k], np.ndarray):
                if k in ("con_at_ob", "con_at_qb"):
                    res[k] = np.concatenate([o[k] for o in outs], axis=0)
                else:
                    res[k] = np.concatenate([o[k] for o in outs])
        return res

    def full(self, it: int) -> dict:
        return self.step(it)
