"""Known-answer tests of the CPU restatement (the checker of the CUDA library), derived from the
mathematics of the scheme rather than from reference outputs (the reference ships none)."""
import numpy as np
import pytest

from fs_system import apply, assemble
from gom_release_gb300.core import GomCore, GomError, TIME_LOOP, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state, tidal_basin
from gom_release_gb300.driver import Run


def _run(deck, so, state=None, steps=10):
    r = Run(deck, GomCore(deck, lib_path=so), state if state is not None else initial_state(deck))
    r.advance(steps)
    return r


def test_lake_at_rest_stays_at_rest(oracle_so):
    deck = tidal_basin(nx=12, ny=8, closed=True)
    r = _run(deck, oracle_so, steps=15)
    c = r.core
    for f in ("un_face", "vn_face", "wn_cell", "u_node", "v_node", "w_node", "eta_cell", "eta_node"):
        assert np.all(c.get_field(f) == 0.0), f
    assert np.all(r.pcg_iters == [0] * 15)   # zero residual: the initial guess is the solution
    s = c.get_field("salt_cell").reshape(deck.n_cells, deck.n_layers)
    top = c.get_field("top_layer_cell")
    bot = deck.geo["bottom_layer_at_element"]
    for i in range(deck.n_cells):   # implicit vertical diffusion of a uniform column: round-off only
        assert np.abs(s[i, bot[i] - 1:top[i]] - 30.0).max() < 1e-12


def test_uniform_tracers_stay_uniform_under_tide(oracle_so):
    """The TVD update keeps a uniform tracer uniform when the free-surface system is solved
    exactly; with the reference's PCG stop ratio of 1e-10 the deviation is ~1e-4, so the solver
    runs to a ratio of 1e-24 here."""
    deck = tidal_basin(nx=14, ny=10)
    deck.params.error_tolerance = 1e-24
    r = _run(deck, oracle_so, steps=30)
    c = r.core
    top = c.get_field("top_layer_cell")
    bot = deck.geo["bottom_layer_at_element"]
    s = c.get_field("salt_cell").reshape(deck.n_cells, deck.n_layers)
    t = c.get_field("temp_cell").reshape(deck.n_cells, deck.n_layers)
    for i in range(deck.n_cells):
        sl = slice(bot[i] - 1, top[i])
        assert np.abs(s[i, sl] - 30.0).max() < 1e-9
        assert np.abs(t[i, sl] - 20.0).max() < 1e-9
    assert np.abs(c.get_field("eta_cell")).max() > 1e-3   # the tide did move the water


def test_volume_conserved_in_closed_basin(oracle_so):
    """Sum of area*dz over wet layers is conserved up to the free-surface solver's residual: 2e-8
    after 40 steps at the reference's stop ratio 1e-10, round-off at 1e-24."""
    deck = tidal_basin(nx=14, ny=10, closed=True)
    deck.params.error_tolerance = 1e-24
    x = deck.geo["x_cell"]
    eta0 = 0.2 * np.cos(np.pi * x / x.max())
    st = initial_state(deck, eta0)
    r = Run(deck, GomCore(deck, lib_path=oracle_so), st)
    v0, _ = r.core.conservation()
    r.advance(40)
    v1, _ = r.core.conservation()
    assert abs(np.abs(r.core.get_field("un_face")).max()) > 1e-3   # the water sloshes
    assert abs(v1 - v0) / v0 < 1e-12


def test_momentum_matrix_identity(oracle_so):
    """A * AinvDeltaZ = dz for the vertical momentum matrix of each wet face (tridiagonal_solver)."""
    deck = estuary(nx=16, ny=8, dx=100.0, n_layers=10, trans_sub_iter=2)
    r = _run(deck, oracle_so, steps=3)
    c = r.core
    L = deck.n_layers
    p = deck.params
    c.set_forcing(r.forcing.full(r.it + 1))
    for ph in TIME_LOOP[:TIME_LOOP.index("momentum") + 1]:
        c.step(ph)
    top = c.get_field("top_layer_face")
    bot = deck.geo["bottom_layer_at_face"]
    av = c.get_field("av").reshape(-1, L + 1)
    dzh = c.get_field("dzhalf_face").reshape(-1, L + 1)
    dz = c.get_field("dz_face").reshape(-1, L)
    gb = c.get_field("gamma_b")
    adz = c.get_field("ainvdz2").reshape(-1, L)
    checked = 0
    for j in range(0, deck.n_faces, 7):
        t, b = top[j], bot[j]
        if t == 0:
            continue
        n = t - b + 1
        A = np.zeros((n, n))
        for row in range(n):        # row 0 = top layer
            k = t - row
            A[row, row] = dz[j, k - 1]
            if row > 0:             # coupling to the layer above (k+1)
                cu = -p.dt * av[j, k] / dzh[j, k]
                A[row, row - 1] = cu
                A[row, row] -= cu
            if k > b:               # coupling to the layer below (k-1)
                lower = -p.dt * av[j, k - 1] / dzh[j, k - 1]
                A[row, row + 1] = lower
                A[row, row] -= lower
            if k == b:
                A[row, row] += gb[j] * p.dt
        sol = adz[j, :n]
        rhs = np.array([dz[j, t - row - 1] for row in range(n)])
        assert np.allclose(A @ sol, rhs, rtol=1e-12, atol=1e-12), j
        checked += 1
    assert checked > 10


def test_pcg_solution_meets_the_stop_criterion(oracle_so):
    deck = estuary(nx=16, ny=8, dx=100.0, n_layers=10, trans_sub_iter=2)
    r = _run(deck, oracle_so, steps=3)
    c = r.core
    f = r.forcing.full(r.it + 1)
    c.set_forcing(f)
    for ph in TIME_LOOP[:TIME_LOOP.index("free_surface")]:
        c.step(ph)
    snap = c.state()
    x0 = snap["eta_cell_new"]
    iters = c.step("free_surface")
    x = c.get_field("eta_cell_new")
    sp, b = assemble(deck, snap, f["eta_at_ob_new"])
    minv = 1.0 / sp[:, 0]
    r0 = b - apply(deck, sp, x0)
    r1 = b - apply(deck, sp, x)
    d0 = float(r0 @ (minv * r0))
    d1 = float(r1 @ (minv * r1))
    assert 0 < iters < deck.params.max_iteration_pcg
    assert np.sqrt(d1 * d1 / (d0 * d0)) < 10 * deck.params.error_tolerance


def test_uniform_flow_elm_feet(oracle_so):
    """Uniform horizontal flow over squares: the foot of every face midpoint is x - U dt, the
    interpolated velocity is U itself."""
    deck = tidal_basin(nx=10, ny=8, tri_rows=0, closed=True)
    st = initial_state(deck)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, st)
    U, V = 0.3, 0.1
    g = deck.geo
    L = deck.n_layers
    ct, sn = g["cos_theta"], g["sin_theta"]
    un = (U * ct + V * sn)[:, None].repeat(L, 1)
    vn = (-U * sn + V * ct)[:, None].repeat(L, 1)
    c.set_field("un_face", un)
    c.set_field("vn_face", vn)
    c.set_field("u_node", np.full((deck.n_nodes, L + 1), U))
    c.set_field("v_node", np.full((deck.n_nodes, L + 1), V))
    c.set_forcing(HostForcing(deck).full(1))
    c.step("advection")
    foot = c.get_field("elm_foot").reshape(-1, L)
    uel = c.get_field("un_elm").reshape(-1, L)
    top = c.get_field("top_layer_face")
    bot = g["bottom_layer_at_face"]
    dx = deck.meta["dx"]
    nx, ny = deck.meta["nx"], deck.meta["ny"]
    checked = 0
    for j in range(deck.n_faces):
        if g["adj_cellnum_at_face"][j, 1] == 0:
            continue
        xf = g["x_face"][j] - U * deck.params.dt
        yf = g["y_face"][j] - V * deck.params.dt
        ci, cj = int(xf // dx), int(yf // dx)
        if not (0 <= ci < nx and 0 <= cj < ny):
            continue
        expect = cj * nx + ci + 1
        for k in range(bot[j], top[j] + 1):
            assert foot[j, k - 1] == expect, (j, k)
            assert abs(uel[j, k - 1] - un[j, k - 1]) < 1e-12
            checked += 1
    assert checked > 100


def test_unesco_density_check_value(oracle_so):
    deck = estuary(nx=10, ny=6, dx=100.0, n_layers=6)
    deck.init_salt_node[:] = 35.0
    deck.init_temp_node[:] = 5.0
    st = initial_state(deck)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, st)
    rho = c.get_field("rho_node").reshape(-1, deck.n_layers)
    top = c.get_field("top_layer_node")
    bot = deck.geo["bottom_layer_at_node"]
    vals = np.concatenate([rho[i, bot[i] - 1:top[i]] for i in range(deck.n_nodes)])
    # UNESCO (1981) check value at S = 35, T = 5 C, p = 0: 1027.67547 kg/m3
    assert np.abs(vals - 1027.67547).max() < 2e-4


def test_fault_codes(oracle_so):
    deck = estuary(nx=12, ny=6, dx=100.0, n_layers=8, trans_sub_iter=2)
    st = initial_state(deck)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, st)
    c.set_forcing(HostForcing(deck).full(1))
    for ph in TIME_LOOP[:TIME_LOOP.index("free_surface")]:
        c.step(ph)
    bad = c.get_field("ainvdz1")
    bad[:] = -1.0
    c.set_field("ainvdz1", bad)
    with pytest.raises(GomError) as e:
        c.step("free_surface")
    assert e.value.code == 3 and e.value.status.site == 100   # GOM_E_NOT_SPD
    c.status(clear=True)
    # zero pivot: a single-layer column with no thickness, no drag
    c2 = GomCore(deck, lib_path=oracle_so)
    prepare(c2, st)
    c2.set_forcing(HostForcing(deck).full(1))
    dz = c2.get_field("dz_face").reshape(deck.n_faces, deck.n_layers)
    dz[:] = 0.0
    c2.set_field("dz_face", dz)
    with pytest.raises(GomError) as e:
        c2.step("momentum")
    assert e.value.code == 4                                 # GOM_E_ZERO_PIVOT


def test_pcg_iteration_cap_returns(oracle_so):
    deck = estuary(nx=12, ny=6, dx=100.0, n_layers=8, trans_sub_iter=2)
    deck.params.max_iteration_pcg = 2
    r = _run(deck, oracle_so, steps=2)
    assert r.pcg_iters == [2, 2]


# ----------------------------------------------------------------- turbulence closure (A13)
def _closure_core(so, flag, rho_profile, shear):
    """A small estuary column set-up with prescribed face densities and velocity shear."""
    deck = estuary(nx=8, ny=6, dx=100.0, n_layers=8, trans_sub_iter=1, turbulence_flag=flag)
    core = GomCore(deck, lib_path=so)
    prepare(core, initial_state(deck))
    L = deck.n_layers
    nf = deck.n_faces
    k = np.arange(1, L + 1, dtype=float)
    core.set_field("rho_face", np.tile(rho_profile(k), nf))
    core.set_field("un_face_new", np.tile(shear * k, nf))
    core.set_field("vn_face_new", np.zeros(nf * L))
    core.set_field("dzhalf_face_new", core.get_field("dzhalf_face"))
    core.step("turbulence")
    return deck, core


def _wet_interfaces(deck, core):
    top = core.get_field("top_layer_face")
    bot = deck.geo["bottom_layer_at_face"]
    L = deck.n_layers
    av = core.get_field("av").reshape(deck.n_faces, L + 1)
    for j in range(deck.n_faces):
        if top[j]:
            yield j, range(bot[j], top[j] + 1), av[j]


def test_pp_closure_neutral_limit(oracle_so):
    """Uniform density: N^2 = -g^2/c^2 < 0, so Ri = 0 and Av = vmax + vmin at every wet interface
    (depth below h1: vmax = vdmax1); the cell diffusivity is the face value Av + tdmin."""
    deck, core = _closure_core(oracle_so, 2, lambda k: np.full_like(k, 1020.0), 0.0)
    p = deck.params
    want_av = p.pp_vdmax1 / 1.0 + p.pp_vdmin1
    n = 0
    for j, ks, av in _wet_interfaces(deck, core):
        if deck.geo["h_face"][j] <= p.pp_h1:
            for k in ks:
                assert av[k] == want_av
                n += 1
    assert n > 0
    kv = core.get_field("kv").reshape(deck.n_cells, deck.n_layers + 1)
    top = core.get_field("top_layer_cell")
    bot = deck.geo["bottom_layer_at_element"]
    for i in range(deck.n_cells):
        if top[i] and deck.geo["h_cell"][i] < p.pp_h1:
            np.testing.assert_allclose(kv[i, bot[i]:top[i] + 1], want_av + p.pp_tdmin, rtol=1e-15)


def test_pp_closure_strong_stratification_limit(oracle_so):
    """Density decreasing upwards with no shear: Ri = N^2 / 1e-10 is huge, Av -> vmin and the face
    diffusivity -> tdmin below the surface interface (where Ri = 0 by definition)."""
    deck, core = _closure_core(oracle_so, 2, lambda k: 1025.0 - 0.5 * k, 0.0)
    p = deck.params
    for j, ks, av in _wet_interfaces(deck, core):
        ks = list(ks)
        for k in ks[:-1]:
            assert abs(av[k] - p.pp_vdmin1) < 1e-12 * max(1.0, p.pp_vdmax1) or deck.geo["h_face"][j] > p.pp_h1
        assert av[ks[-1]] >= p.pp_vdmin1   # surface interface: Ri = 0


def test_step_closure_switches_at_critical_richardson(oracle_so):
    """Scheme 1: Av = Kv = 1e-3 where Ri < 0.25 and 1e-5 otherwise; strong shear with weak
    stratification is sub-critical, no shear with stable stratification is super-critical."""
    deck, core = _closure_core(oracle_so, 1, lambda k: 1025.0 - 0.01 * k, 0.5)
    for _, ks, av in _wet_interfaces(deck, core):
        assert all(av[k] == 1e-3 for k in ks)
    deck, core = _closure_core(oracle_so, 1, lambda k: 1025.0 - 0.5 * k, 0.0)
    for _, ks, av in _wet_interfaces(deck, core):
        ks = list(ks)
        assert all(av[k] == 1e-5 for k in ks[:-1])
        assert av[ks[-1]] == 1e-3


# ----------------------------------------------------------------- building blocks
import ctypes as _C


def _hooks(so):
    lib = _C.CDLL(str(so))
    D = _C.POINTER(_C.c_double)
    lib.gom_oracle_tridiagonal.argtypes = [_C.c_int32, _C.c_int32, D, D, D, D, D]
    lib.gom_oracle_bilinear.argtypes = [D, D, _C.c_double, _C.c_double, D]
    lib.gom_oracle_check_intersection.argtypes = [D, D]
    return lib, D


def test_tridiagonal_against_dense_solve(oracle_so):
    """tridiagonal_solver.f90 on random diagonally dominant systems with three right-hand sides
    against a dense LU solve."""
    lib, D = _hooks(oracle_so)
    rng = np.random.default_rng(5)
    for n in (1, 2, 7, 40):
        a = rng.uniform(-1, 0, n)
        c = rng.uniform(-1, 0, n)
        b = 2.5 + rng.uniform(0, 1, n)
        rhs = rng.normal(size=(3, n))
        sol = np.zeros((3, n))
        assert lib.gom_oracle_tridiagonal(n, 3, a.ctypes.data_as(D), b.ctypes.data_as(D), c.ctypes.data_as(D),
                                          rhs.ctypes.data_as(D), sol.ctypes.data_as(D)) == 0
        m = np.diag(b) + np.diag(a[1:], -1) + np.diag(c[:-1], 1)
        want = np.linalg.solve(m, rhs.T).T
        np.testing.assert_allclose(sol, want, rtol=1e-12, atol=1e-12)
    # zero pivot is reported, not divided by
    z = np.zeros(3)
    one = np.ones(3)
    out = np.zeros(3)
    assert lib.gom_oracle_tridiagonal(3, 1, one.ctypes.data_as(D), z.ctypes.data_as(D), one.ctypes.data_as(D),
                                      one.ctypes.data_as(D), out.ctypes.data_as(D)) != 0


def test_inverse_bilinear_round_trip(oracle_so):
    """bilinear_interpolation.f90 inverts the bilinear map of random convex quads: shape functions
    at a point mapped from (xi, eta) are those of (xi, eta), and reproduce the point."""
    lib, D = _hooks(oracle_so)
    rng = np.random.default_rng(9)
    for _ in range(200):
        # a convex quad: a perturbed square of side ~100 m, counter-clockwise
        base = np.array([[-50.0, -50.0], [50.0, -50.0], [50.0, 50.0], [-50.0, 50.0]])
        q = base + rng.uniform(-12, 12, size=(4, 2))
        xi, eta = rng.uniform(-0.95, 0.95, 2)
        n = np.array([(1 - xi) * (1 - eta), (1 + xi) * (1 - eta), (1 + xi) * (1 + eta), (1 - xi) * (1 + eta)]) / 4
        x, y = n @ q[:, 0], n @ q[:, 1]
        xq = np.ascontiguousarray(q[:, 0])
        yq = np.ascontiguousarray(q[:, 1])
        sh = np.zeros(4)
        assert lib.gom_oracle_bilinear(xq.ctypes.data_as(D), yq.ctypes.data_as(D), x, y, sh.ctypes.data_as(D)) == 0
        np.testing.assert_allclose(sh, n, atol=1e-9)
        assert abs(sh @ q[:, 0] - x) < 1e-7 and abs(sh @ q[:, 1] - y) < 1e-7


def test_segment_intersection_inclusive(oracle_so):
    """check_intersection.f90: crossing segments meet at the right point; touching at an end point
    counts (inclusive [0, 1]); parallel and disjoint segments do not."""
    lib, D = _hooks(oracle_so)

    def hit(x1, y1, x2, y2, x3, y3, x4, y4):
        seg = np.array([x1, x2, x3, x4, y1, y2, y3, y4], dtype=float)
        xy = np.zeros(2)
        f = lib.gom_oracle_check_intersection(seg.ctypes.data_as(D), xy.ctypes.data_as(D))
        return f, xy

    f, xy = hit(0, 0, 2, 2, 0, 2, 2, 0)
    assert f == 1 and np.allclose(xy, [1, 1])
    f, xy = hit(0, 0, 1, 1, 1, 1, 2, 0)          # touch at an end point
    assert f == 1 and np.allclose(xy, [1, 1])
    assert hit(0, 0, 1, 0, 0, 1, 1, 1)[0] == 0  # parallel
    assert hit(0, 0, 1, 1, 2, 0, 3, -1)[0] == 0  # disjoint


def test_elm_transport_keeps_uniform_tracers(oracle_so):
    """transport_solver = 2 (solve_transport_equation_ELM_v8): with uniform tracers every
    backtracked value, every diffusive difference and every vertical solve returns the uniform
    value (the reference's top-row coefficient -dt + Kv/dzhalf keeps the row sums), so the
    tracers stay uniform under the tide while the walk does move feet."""
    import dataclasses
    deck = tidal_basin(nx=14, ny=10)
    deck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, transport_solver=2))
    r = _run(deck, oracle_so, steps=20)
    c = r.core
    top = c.get_field("top_layer_cell")
    bot = deck.geo["bottom_layer_at_element"]
    s = c.get_field("salt_cell").reshape(deck.n_cells, deck.n_layers)
    t = c.get_field("temp_cell").reshape(deck.n_cells, deck.n_layers)
    for i in range(deck.n_cells):
        sl = slice(bot[i] - 1, top[i])
        assert np.abs(s[i, sl] - 30.0).max() < 1e-9
        assert np.abs(t[i, sl] - 20.0).max() < 1e-9
    assert np.abs(c.get_field("salt_node") - 30.0).max() < 1e-9
    assert np.count_nonzero(c.get_field("elm_foot")) > 0


def test_elm_transport_swaps_the_horizontal_sums(oracle_so):
    """The explicit horizontal step of solve_transport_equation_ELM_v8.f90:137-151 adds the
    salinity differences to temperature and the temperature differences to salinity: with a
    salinity gradient and uniform temperature at rest, temperature changes and salinity does
    not (no advection, no vertical gradient)."""
    import dataclasses
    deck = tidal_basin(nx=10, ny=8, closed=True)
    deck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, transport_solver=2, kh_0=10.0))
    st = initial_state(deck)
    L = deck.n_layers
    x = np.repeat(deck.geo["x_cell"], L)
    st["salt_cell"] = 20.0 + 10.0 * x / x.max()
    core = GomCore(deck, lib_path=oracle_so)
    prepare(core, st)
    core.set_forcing(HostForcing(deck).step(1))
    for ph in TIME_LOOP:
        core.step(ph)
    t_new = core.get_field("temp_cell_new")
    s_new = core.get_field("salt_cell_new")
    top = core.get_field("top_layer_cell")
    bot = deck.geo["bottom_layer_at_element"]
    wet = np.zeros_like(t_new, dtype=bool).reshape(deck.n_cells, L)
    for i in range(deck.n_cells):
        wet[i, bot[i] - 1:top[i]] = True
    wet = wet.ravel()
    assert np.abs(t_new[wet] - 20.0).max() > 1e-6
    assert np.abs(s_new[wet] - st["salt_cell"][wet]).max() < 1e-9


def test_heat_option1_source_heats_each_layer(oracle_so):
    """heat_option 1 (solve_transport_equation_v19.f90:100-131) in a basin at rest with no
    vertical diffusion: each wet layer warms by dt phi_sz / (rho_o cp dz) per step."""
    import dataclasses
    deck = tidal_basin(nx=8, ny=6, closed=True)
    deck = dataclasses.replace(deck, params=dataclasses.replace(deck.params, heat_option=1, kv_0=0.0))
    st = initial_state(deck)
    c = GomCore(deck, lib_path=oracle_so)
    prepare(c, st)
    fr = HostForcing(deck)
    L, nc = deck.n_layers, deck.n_cells
    q = np.full((nc, L), 250.0)
    steps = 4
    for it in range(1, steps + 1):
        f = fr.step(it)
        f["phi_sz"] = q
        c.set_forcing(f)
        c.step_all()
    t = c.get_field("temp_cell").reshape(nc, L)
    dz = c.get_field("dz_cell").reshape(nc, L)
    top = c.get_field("top_layer_cell")
    bot = deck.geo["bottom_layer_at_element"]
    p = deck.params
    for i in range(nc):
        for k in range(bot[i], top[i] + 1):
            expect = 20.0 + steps * p.dt * 250.0 / (p.rho_o * 4186.0 * dz[i, k - 1])
            assert abs(t[i, k - 1] - expect) < 1e-11, (i, k, t[i, k - 1], expect)


def test_packed_status_names_the_failing_run(oracle_so):
    """A packed context reports the first failing entity; gom_get_status maps it to the run that
    holds it, so a server can retire that run alone.  The failure is made on the host: one run's
    elevation is set above the highest level."""
    from gom_release_gb300.ensemble import PackedForcing, pack, storm_run
    runs = [storm_run(41, 300, 1.5, 10, max_layers=12), storm_run(42, 400, 2.0, 12, max_layers=12),
            storm_run(43, 250, 1.0, 10, max_layers=12)]
    pk = pack(runs)
    c = GomCore(pk, lib_path=oracle_so)
    prepare(c, initial_state(pk))
    fp = PackedForcing(pk)
    for it in range(1, 3):
        c.set_forcing(fp.step(it))
        c.step_all()
    eta = c.get_field("eta_cell")
    cs = pk.runs["run_cell_start"]
    eta[cs[1]:cs[2]] = pk.z_level[-1] + 5.0
    c.set_field("eta_cell", eta)
    c.set_field("eta_cell_new", eta)
    c.set_forcing(fp.step(3))
    with pytest.raises(GomError) as info:
        c.step_all()
    st = info.value.status
    assert st.code != 0 and st.entity_kind in (1, 2, 3)
    assert st.run == 1, (st.code, st.site, st.entity, st.entity_kind, st.run)


def wind_basin(coriolis_lat=0.0, theta=1.0):
    """A closed 10 km x 1.5 km basin of 5 m depth, one layer, uniform wind stress 0.1 Pa along x
    (ana_windp.f90: kinematic stress tau / 1000), no advection, no transport."""
    from gom_release_gb300.deck import Params, _finish
    from gom_release_gb300.mesh import RawMesh, square_strip_mesh

    x, y, cells, tq = square_strip_mesh(20, 3, 500.0, 0)
    raw = RawMesh(x=x, y=y, h=np.full(len(x), 5.0), tri_or_quad=tq, cells=cells)
    p = Params(dt=120.0, theta=theta, error_tolerance=1e-12, baroclinic_flag=0, trans_sub_iter=1,
               h_flux_limiter=0, v_flux_limiter=0, advection_flag=0, transport_flag=0, coriolis_lat=coriolis_lat)
    d = _finish("wind_basin", raw, 1, -10.0, 2.0, p, [], [], [],
                tide=dict(amplitude=[], period_h=[], phase=[], nodal=[], eq_arg=[], shift=0.0), wind_stress=(0.1, 0.0))
    d.init_salt_node = np.full((d.n_nodes, 1), 30.0)
    d.init_temp_node = np.full((d.n_nodes, 1), 20.0)
    return d


def test_wind_setup_of_a_closed_basin(oracle_so):
    """Steady wind set-up: with one layer and no net flow the face momentum balance is
    g (h + eta) d eta / dx = tau / rho_o (solve_momentum_equation.f90: wind stress in G1 of the
    top layer, the free-surface gradient in the normal equation), so eta rises along the wind
    with slope tau / (rho_o g (h + eta)); the normal velocities vanish."""
    d = wind_basin()
    c = GomCore(d, lib_path=oracle_so)
    prepare(c, initial_state(d))
    f = HostForcing(d)
    for it in range(1, 3001):
        c.set_forcing(f.full(it) if it == 1 else f.step(it))
        c.step_all()
    eta = c.get_field("eta_cell")
    xc = d.geo["x_cell"]
    tau_k = 0.1 / 1000.0
    # the slope between neighbouring cells of the middle row against the local depth h + eta
    row = np.argsort(xc[(d.geo["y_cell"] > 500) & (d.geo["y_cell"] < 1000)])
    mid = np.nonzero((d.geo["y_cell"] > 500) & (d.geo["y_cell"] < 1000))[0][row]
    slope = np.diff(eta[mid]) / np.diff(xc[mid])
    depth = 5.0 + 0.5 * (eta[mid][1:] + eta[mid][:-1])
    want = tau_k / (d.params.gravity * depth)
    assert np.all(np.abs(slope / want - 1.0) < 2e-3), float(np.abs(slope / want - 1.0).max())
    assert float(np.abs(c.get_field("un_face")).max()) < 1e-6
    # the volume is kept (equal cell areas: the mean elevation stays 0 up to the PCG tolerance
    # accumulated over the 3000 steps)
    assert abs(float(eta.mean())) < 1e-8
