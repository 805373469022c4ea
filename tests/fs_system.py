"""Host restatement of the free-surface row assembly (solve_free_surface_equation.f90:65-212)
shared by tests: scalar IEEE double arithmetic in the reference's operation order."""
import numpy as np


def assemble(deck, snap, eta_ob_new):
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
            c1 = 0.0
            c2 = 0.0
            for k in range(1, nvl + 1):
                kk = tj + 1 - k
                dz = float(dz_face[j, kk - 1])
                sdz = sdz + dz * float(ainvdz1[j, k - 1])
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


def apply(deck, sparsem, x):
    """A x for the 5-point rows (diagonal, then neighbours in local-face order)."""
    g = deck.geo
    y = sparsem[:, 0] * x
    for l in range(4):
        nb = g["adj_cellnum_at_cell"][:, l]
        m = nb > 0
        y[m] += sparsem[m, l + 1] * x[nb[m] - 1]
    return y
