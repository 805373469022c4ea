"""Start-up geometry built on the GPU (gom_geometry_build of the CUDA library) against the oracle's
loop-for-loop restatement: every integer array and every double computed with + - x / and sqrt
bit for bit; the four face-angle arrays (cos and sin of atan2 angles, all within [-1, 1]) within
4e-15 absolute, a few ulps of the angle, from CUDA's atan2 / cos / sin against the C library's;
the same stop, site and entity for meshes the reference rejects; and a run from the GPU-built
geometry tracking a run from the host-built one."""
import time

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, GomError, geometry_build, load_library, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state
from gom_release_gb300.mesh import RawMesh
from test_geometry import decks, deck_inputs, jittered

pytestmark = pytest.mark.gpu

ANGLES = ("cos_theta", "sin_theta", "cos_theta2", "sin_theta2")
ANGLE_ATOL = 4e-15


@pytest.fixture(scope="module")
def oracle(oracle_so):
    return load_library(oracle_so)


def _compare(dev, ref):
    bad = [k for k in ref if k not in ANGLES and not np.array_equal(dev[k], ref[k])]
    assert not bad, bad
    for k in ANGLES:
        err = float(np.abs(dev[k] - ref[k]).max())
        assert err <= ANGLE_ATOL, (k, err)


@pytest.mark.parametrize("name", ["mobile_bay", "estuary", "basin"])
def test_device_geometry_equals_oracle_on_decks(oracle, gpu_lib, name):
    d, vor = next((d, v) for n, d, v in decks() if n == name)
    kw = deck_inputs(d, vor)
    _compare(geometry_build(gpu_lib, **kw), geometry_build(oracle, **kw))


@pytest.mark.parametrize("seed,voronoi", [(1, 0), (2, 1), (3, 1)])
def test_device_geometry_equals_oracle_on_jittered_meshes(oracle, gpu_lib, seed, voronoi):
    kw = jittered(seed, voronoi, nx=60, ny=40, tri_rows=7)
    _compare(geometry_build(gpu_lib, **kw), geometry_build(oracle, **kw))


def test_full_estuary_geometry_and_build_time(oracle, gpu_lib):
    d = estuary()
    kw = deck_inputs(d, 1)
    geometry_build(gpu_lib, **kw)   # context and module load outside the timing
    t0 = time.perf_counter()
    dev = geometry_build(gpu_lib, **kw)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = geometry_build(oracle, **kw)
    t_ref = time.perf_counter() - t0
    _compare(dev, ref)
    errs = {k: float(np.abs(dev[k] - ref[k]).max()) for k in ANGLES}
    print(f"\nangle arrays, largest difference from the C library: {errs}")
    print(f"estuary geometry ({d.n_cells} cells, {d.n_faces} faces): GPU {t_dev * 1e3:.1f} ms, "
          f"serial oracle {t_ref * 1e3:.1f} ms")


def _stop(lib, kw):
    with pytest.raises(GomError) as e:
        geometry_build(lib, **kw)
    st = e.value.status
    return (st.site, st.entity, st.entity_kind) if st is not None else None


def test_same_stops_as_oracle(oracle, gpu_lib):
    base = jittered(5, 1)
    raw = base["raw"]
    nn = len(raw.x)

    def extra(k):
        xs = np.append(raw.x, 1.0e4 + 10.0 * np.arange(k))
        ys = np.append(raw.y, np.full(k, 1.0e4))
        cell = np.zeros((1, 4), np.int32)
        cell[0, :k] = nn + 1 + np.arange(k)
        return dict(base, raw=RawMesh(x=xs, y=ys, h=np.append(raw.h, np.full(k, 5.0)),
                                      tri_or_quad=np.append(raw.tri_or_quad, k).astype(np.int32),
                                      cells=np.vstack([raw.cells, cell]).astype(np.int32)))

    g = geometry_build(oracle, **base)
    bf = int(np.nonzero(g["adj_cellnum_at_face"][:, 1] == 0)[0][0])
    n1, n2 = g["nodenum_at_face"][bf]
    cases = [extra(4), extra(3),
             dict(base, raw=RawMesh(x=np.append(raw.x, 0.0), y=np.append(raw.y, 0.0), h=np.append(raw.h, 5.0),
                                    tri_or_quad=raw.tri_or_quad, cells=raw.cells)),
             dict(base, max_nb=3), dict(base, ob_pairs=[(n2, n1)]), dict(base, q_pairs=[(n1, n2), (n2, n1)]),
             dict(base, z_level=np.linspace(-8.0, 2.0, 6))]
    for kw in cases:
        want = _stop(oracle, kw)
        assert want is not None
        assert _stop(gpu_lib, kw) == want


def test_run_from_device_geometry_tracks_host_geometry(gpu_lib):
    kwargs = dict(nx=30, ny=12, dx=100.0, n_layers=8, trans_sub_iter=2)
    host = estuary(**kwargs)
    dev = estuary(**kwargs, geometry_lib=gpu_lib)
    for k in host.geo:
        if k not in ANGLES:
            assert np.array_equal(np.asarray(host.geo[k]), np.asarray(dev.geo[k])), k
    runs = []
    for d in (host, dev):
        c = GomCore(d, lib=gpu_lib)
        prepare(c, initial_state(d))
        f = HostForcing(d)
        for it in range(1, 21):
            c.set_forcing(f.full(it) if it == 1 else f.step(it))
            c.step_all()
        runs.append({n: c.get_field(n) for n in ("eta_cell", "un_face", "salt_cell")})
    for n in runs[0]:
        a, b = runs[0][n], runs[1][n]
        assert float(np.abs(a - b).max()) <= 1e-9 * max(float(np.abs(a).max()), 1e-30), n
