"""gom_pcg_solve_noalloc: the free-surface PCG for callers that cannot allocate device memory.

Such a caller (a Fortran driver whose arrays live in OpenACC or CUDA Fortran data regions, or a
service whose device memory is fixed at start-up) owns its matrix, right-hand side and solution
in device memory -- here PyTorch tensors stand in for another runtime's arrays -- and hands them
over; the solver's work vectors come from the library's fixed device array.  The test builds the
free-surface system of a real step on the host, in the same operation order as the library's
assembly, solves it twice in a row through the no-allocation entry point, and checks both
solutions against the elevation of the regular entry point (gom_step_free_surface) and of the CPU
oracle for the same state, and that a call leaves the device's free memory unchanged.

Collected last on purpose (file name), so a failure here cannot hide earlier results.
"""
import ctypes as C

import numpy as np
import pytest

from gom_release_gb300.core import GomCore, TIME_LOOP, prepare
from gom_release_gb300.deck import HostForcing, estuary, initial_state

pytestmark = pytest.mark.gpu

ETA_TOL = 1e-10   # same tolerance the other parity tests use for the PCG output (metres)


def _assemble(deck, snap, eta_ob_new):
    """Host restatement of the per-cell row and RHS (solve_free_surface_equation.f90:65-212),
    scalar IEEE double arithmetic in the library's operation order."""
    g = deck.geo
    p = deck.params
    L = deck.n_layers
    nc, nf = deck.n_cells, deck.n_faces
    dz_face = snap["dz_face"].reshape(nf, L)
    ainvdz1 = snap["ainvdz1"].reshape(nf, L)
    ainvg1 = snap["ainvg1"].reshape(nf, L)
    un_face = snap["un_face"].reshape(nf, L)
    top_face = snap["top_layer_face"]
    eta_cell = snap["eta_cell"]
    dt, grav, th = float(p.dt), float(p.gravity), float(p.theta)
    gdt2th2 = grav * (dt * dt) * (th * th)
    sparsem = np.zeros((nc, 5))
    rhs = np.zeros(nc)
    for i in range(nc):
        tq = int(g["tri_or_quad"][i])
        ar = float(g["area"][i])
        diag = ar
        off = [0.0, 0.0, 0.0, 0.0]
        r = ar * float(eta_cell[i])
        for l in range(tq):
            j = int(g["facenum_at_cell"][i, l]) - 1
            tj = int(top_face[j])
            if tj == 0:
                continue
            nvl = tj - int(g["bottom_layer_at_face"][j]) + 1
            sdz = 0.0
            for k in range(1, nvl + 1):
                kk = tj + 1 - k
                sdz = sdz + float(dz_face[j, kk - 1]) * float(ainvdz1[j, k - 1])
            base = gdt2th2 * float(g["face_length"][j]) / float(g["delta_j"][j]) * sdz
            coef = base * float(g["cos_theta2"][j])
            diag = diag + coef
            if g["adj_cellnum_at_cell"][i, l] != 0:
                off[l] = -coef
        for l in range(tq):
            j = int(g["facenum_at_cell"][i, l]) - 1
            tj = int(top_face[j])
            if tj == 0:
                continue
            nvl = tj - int(g["bottom_layer_at_face"][j]) + 1
            c1 = 0.0
            c2 = 0.0
            for k in range(1, nvl + 1):
                kk = tj + 1 - k
                dz = float(dz_face[j, kk - 1])
                c1 = c1 + dz * float(un_face[j, kk - 1])
                c2 = c2 + dz * float(ainvg1[j, k - 1])
            sgn = float(g["sign_in_outflow"][i, l])
            fl = float(g["face_length"][j])
            r = r - (1.0 - th) * dt * sgn * fl * c1 - th * dt * sgn * fl * c2
        obf = int(g["ob_element_flag"][i])
        if obf > 0:
            for l in range(tq):
                j = int(g["facenum_at_cell"][i, l]) - 1
                tj = int(top_face[j])
                if g["boundary_type_of_face"][j] > 0 and tj != 0:
                    nvl = tj - int(g["bottom_layer_at_face"][j]) + 1
                    sdz = 0.0
                    for k in range(1, nvl + 1):
                        sdz = sdz + float(dz_face[j, tj - k]) * float(ainvdz1[j, k - 1])
                    base = gdt2th2 * float(g["face_length"][j]) / float(g["delta_j"][j]) * sdz
                    r = r + base * float(eta_ob_new[obf - 1])
        sparsem[i, 0] = diag
        sparsem[i, 1:] = off
        rhs[i] = r
    return sparsem, rhs


def _bind(lib):
    lib.gom_pcg_solve_noalloc.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_int32, C.c_double, C.c_void_p, C.POINTER(C.c_int32), C.c_void_p]
    lib.gom_pcg_solve_noalloc.restype = C.c_int
    return lib


def test_noalloc_pcg_matches_free_surface_entry_and_oracle(gpu_lib, oracle_so):
    import torch

    lib = _bind(gpu_lib)
    deck = estuary(nx=30, ny=14, dx=100.0, n_layers=12, trans_sub_iter=3)
    st = initial_state(deck)
    ref = GomCore(deck, lib_path=oracle_so)
    prepare(ref, st)
    fr = HostForcing(deck)
    for it in range(1, 4):
        ref.set_forcing(fr.step(it))
        ref.step_all()
    f = fr.full(4)
    ref.set_forcing(f)
    for ph in TIME_LOOP[:TIME_LOOP.index("free_surface")]:
        ref.step(ph)
    snap = ref.state()
    # the oracle's own solve of the same system
    ref.step("free_surface")
    eta_oracle = ref.get_field("eta_cell_new")
    # the regular entry point on the same state
    gpu = GomCore(deck, lib=lib)
    gpu.load_state(snap)
    gpu.set_forcing(f)
    gpu.step("free_surface")
    eta_regular = gpu.get_field("eta_cell_new")
    gpu.close()
    assert float(np.abs(eta_regular - eta_oracle).max()) < ETA_TOL
    # the caller's own device arrays
    sparsem, rhs = _assemble(deck, snap, f["eta_at_ob_new"])
    dev = torch.device("cuda:0")
    t_tq = torch.tensor(deck.geo["tri_or_quad"], dtype=torch.int32, device=dev)
    t_adj = torch.tensor(np.ascontiguousarray(deck.geo["adj_cellnum_at_cell"]), dtype=torch.int32, device=dev)
    t_sp = torch.tensor(sparsem, dtype=torch.float64, device=dev)
    t_rhs = torch.tensor(rhs, dtype=torch.float64, device=dev)
    t_x = [torch.tensor(snap["eta_cell_new"], dtype=torch.float64, device=dev) for _ in range(2)]
    t_res = torch.full((2,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    for call in range(2):   # two calls in a row share (and must clear) the library's scratch
        free_before = torch.cuda.mem_get_info(dev)[0]
        iters = C.c_int32(-1)
        rc = lib.gom_pcg_solve_noalloc(deck.n_cells, t_tq.data_ptr(), t_adj.data_ptr(), t_sp.data_ptr(),
                                       t_rhs.data_ptr(), t_x[call].data_ptr(), deck.params.max_iteration_pcg,
                                       deck.params.error_tolerance, C.c_void_p(stream.cuda_stream), C.byref(iters),
                                       C.c_void_p(t_res.data_ptr()))
        torch.cuda.synchronize(dev)
        free_after = torch.cuda.mem_get_info(dev)[0]
        assert rc == 0, f"call {call}: status {rc}"
        assert 0 < iters.value < deck.params.max_iteration_pcg
        assert t_res.cpu().tolist() == [0, iters.value], "device-side status and iteration count"
        if call == 1:
            # the first call may load the library's device code; after that a call holds no memory
            assert free_after == free_before, f"free device memory changed by {free_before - free_after} bytes"
        x = t_x[call].cpu().numpy()
        err = float(np.abs(x - eta_regular).max())
        assert err < ETA_TOL, f"call {call}: differs from gom_step_free_surface by {err:.3e} m"
        err = float(np.abs(x - eta_oracle).max())
        assert err < ETA_TOL, f"call {call}: differs from the oracle by {err:.3e} m"


def test_noalloc_reports_a_failure_to_an_asynchronous_caller(gpu_lib):
    """A system whose diagonal is not positive: the call returns after the launch (no
    iterations pointer) and the caller reads GOM_E_NOT_SPD from its own device memory; the next
    call starts clean."""
    import torch

    lib = _bind(gpu_lib)
    dev = torch.device("cuda:0")
    n = 64
    tq = torch.full((n,), 4, dtype=torch.int32, device=dev)
    adj = torch.zeros((n, 4), dtype=torch.int32, device=dev)
    sp = torch.zeros((n, 5), dtype=torch.float64, device=dev)
    sp[:, 0] = 1.0
    sp[17, 0] = 0.0
    rhs = torch.ones(n, dtype=torch.float64, device=dev)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    res = torch.full((2,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.gom_pcg_solve_noalloc(n, tq.data_ptr(), adj.data_ptr(), sp.data_ptr(), rhs.data_ptr(), x.data_ptr(),
                                   100, 1e-10, C.c_void_p(stream.cuda_stream), None, C.c_void_p(res.data_ptr()))
    assert rc == 0   # asynchronous: launched
    torch.cuda.synchronize(dev)
    assert res.cpu().tolist()[0] == 3   # GOM_E_NOT_SPD
    sp[17, 0] = 2.0
    iters = C.c_int32(-1)
    rc = lib.gom_pcg_solve_noalloc(n, tq.data_ptr(), adj.data_ptr(), sp.data_ptr(), rhs.data_ptr(), x.data_ptr(),
                                   100, 1e-10, C.c_void_p(stream.cuda_stream), C.byref(iters), None)
    assert rc == 0 and iters.value >= 1
    expect = np.ones(n)
    expect[17] = 0.5
    assert np.allclose(x.cpu().numpy(), expect, rtol=0, atol=1e-12)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    lib = _bind(gpu_lib)
    rc = lib.gom_pcg_solve_noalloc(C.c_int32(262145), C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), C.c_void_p(8),
                                   C.c_void_p(8), C.c_int32(10), C.c_double(1e-10), C.c_void_p(None),
                                   C.POINTER(C.c_int32)(), None)
    assert rc == 1   # GOM_E_ARG, before any device work
