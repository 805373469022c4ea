"""Synthetic orthogonal meshes and the static geometry GOM derives from them.

GOM reads ``node.inp`` / ``cell.inp`` (read_node_inp.f90, read_cell_inp.f90) and derives the
connectivity, face geometry and Voronoi centres once at start-up (set_geometry_1.f90,
calculate_voronoi_center.f90, set_geometry_2.f90).  That derivation is host work that stays
on the Fortran side of the C ABI; this module restates it in numpy so that synthetic meshes
produce exactly the arrays the reference would hold in ``mod_global_variables`` and pass to
``gom_create``.

Array layout: a Fortran array declared ``(a, N)`` is stored here as a C-contiguous numpy
array of shape ``(N, a)`` (the same bytes).  Connectivity is 1-based with 0 = none.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


# ----------------------------------------------------------------------------- mesh shapes
@dataclass
class RawMesh:
    """Nodes and cells as cell.inp / node.inp hold them (counter-clockwise nodes)."""

    x: np.ndarray            # (N_n,)
    y: np.ndarray            # (N_n,)
    h: np.ndarray            # (N_n,) depth below MSL, positive down
    tri_or_quad: np.ndarray  # (N_c,) int32 3 or 4
    cells: np.ndarray        # (N_c, 4) int32, 1-based, 4th = 0 for triangles
    meta: dict = field(default_factory=dict)


def square_strip_mesh(nx: int, ny: int, dx: float, tri_rows: int) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """``nx`` x ``ny`` axis-aligned squares of side ``dx`` plus ``tri_rows`` rows of equilateral
    triangles (side ``dx``) along the north edge.

    Squares are numbered row by row from the south-west corner; triangle rows follow, west to
    east.  Triangle circumcentres sit on the perpendicular bisectors of the shared square edges,
    so the mesh is orthogonal in GOM's sense (voronoi = 1).
    """
    hgt = dx * math.sqrt(3.0) / 2.0
    gx, gy = np.meshgrid(np.arange(nx + 1) * dx, np.arange(ny + 1) * dx)
    xs = [gx.ravel()]
    ys = [gy.ravel()]
    nid = np.arange((nx + 1) * (ny + 1), dtype=np.int64).reshape(ny + 1, nx + 1) + 1
    # squares, CCW: SW, SE, NE, NW
    sw = nid[:-1, :-1].ravel()
    se = nid[:-1, 1:].ravel()
    ne = nid[1:, 1:].ravel()
    nw = nid[1:, :-1].ravel()
    cells = [np.stack([sw, se, ne, nw], axis=1)]
    tq = [np.full(nx * ny, 4, dtype=np.int32)]

    lines = [nid[-1, :]]          # line 0: the north row of grid nodes (even line)
    next_id = (nx + 1) * (ny + 1) + 1
    y0 = ny * dx
    for r in range(1, tri_rows + 1):
        if r % 2 == 1:            # odd line: nx nodes, offset dx/2
            cnt = nx
            lx = dx * 0.5 + np.arange(cnt) * dx
        else:
            cnt = nx + 1
            lx = np.arange(cnt) * dx
        ids = np.arange(next_id, next_id + cnt, dtype=np.int64)
        next_id += cnt
        xs.append(lx)
        ys.append(np.full(cnt, y0 + r * hgt))
        lines.append(ids)
    tris = []
    for r in range(tri_rows):
        lo, hi = lines[r], lines[r + 1]
        row = []
        if r % 2 == 0:            # even lower (nx+1), odd upper (nx)
            for i in range(nx):
                row.append((lo[i], lo[i + 1], hi[i]))
                if i < nx - 1:
                    row.append((hi[i], lo[i + 1], hi[i + 1]))
        else:                     # odd lower (nx), even upper (nx+1)
            for i in range(nx):
                row.append((lo[i], hi[i + 1], hi[i]))
                if i < nx - 1:
                    row.append((lo[i], lo[i + 1], hi[i + 1]))
        tris.extend(row)
    if tris:
        t = np.asarray(tris, dtype=np.int64)
        cells.append(np.concatenate([t, np.zeros((len(t), 1), dtype=np.int64)], axis=1))
        tq.append(np.full(len(t), 3, dtype=np.int32))
    x = np.concatenate(xs).astype(np.float64)
    y = np.concatenate(ys).astype(np.float64)
    return x, y, np.concatenate(cells).astype(np.int32), np.concatenate(tq)


def coastal_strip(x: np.ndarray, y: np.ndarray, y0: float, strip: float, coast) -> np.ndarray:
    """The strip nodes (y > y0) of ``square_strip_mesh`` moved so that the strip's north edge
    follows ``coast(x)`` instead of the straight line y0 + strip: each node keeps its fraction of
    the strip height.  With coast(x) - y0 between 0.7 and 1.3 strip heights and varying slowly
    over one cell, every triangle stays acute, so its circumcentre stays inside it and the
    centres of neighbouring cells stay on the perpendicular bisector of their shared side."""
    out = y.copy()
    m = y > y0 + 1e-9
    frac = (y[m] - y0) / strip
    out[m] = y0 + frac * (coast(x[m]) - y0)
    return out


def fourier_noise(x: np.ndarray, y: np.ndarray, rng: np.random.Generator, n_modes: int = 8,
                  lam_min: float = 2000.0, lam_max: float = 15000.0, amplitude: float = 1.0) -> np.ndarray:
    """Seeded smooth noise: ``n_modes`` plane waves with wavelengths in [lam_min, lam_max] whose
    absolute amplitudes sum to ``amplitude``."""
    lam = rng.uniform(lam_min, lam_max, n_modes)
    ang = rng.uniform(0.0, 2.0 * math.pi, n_modes)
    ph = rng.uniform(0.0, 2.0 * math.pi, n_modes)
    w = rng.uniform(0.5, 1.0, n_modes)
    w = w / w.sum() * amplitude
    out = np.zeros_like(x)
    for m in range(n_modes):
        k = 2.0 * math.pi / lam[m]
        out += w[m] * np.sin(k * (x * math.cos(ang[m]) + y * math.sin(ang[m])) + ph[m])
    return out


# ----------------------------------------------------------------------------- geometry
def calculate_area(x1, x2, x3, y1, y2, y3):
    """mod_function_library.f90:49-60."""
    return np.abs((x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3)) / 2.0


def start_end_node() -> np.ndarray:
    """set_geometry_1.f90:48-63: start_end_node(k,i,j) = i+j wrapped into 1..k; returned as
    a (5, 5, 4) int array indexed [k, i, j] (1-based, unused entries 0)."""
    se = np.zeros((5, 5, 4), dtype=np.int32)
    for k in (3, 4):
        for i in range(1, k + 1):
            for j in range(1, k):
                v = i + j
                if v > k:
                    v -= k
                se[k, i, j] = v
    return se


@dataclass
class Geometry:
    n_nodes: int
    n_cells: int
    n_faces: int
    max_nb: int
    arrays: dict


def build_geometry(raw: RawMesh, max_nb: int = 12, voronoi: int = 1) -> Geometry:
    """read_cell_inp.f90:37-65 (areas) + set_geometry_1.f90 + calculate_voronoi_center.f90."""
    x, y, hn = raw.x, raw.y, raw.h
    tq = raw.tri_or_quad.astype(np.int32)
    cells = raw.cells.astype(np.int64)
    nc = len(tq)
    nn = len(x)
    se = start_end_node()
    c0 = cells - 1  # 0-based nodes (4th = -1 for triangles)

    # --- areas (read_cell_inp.f90:39-64); quads: sum of triangles (1,2,3) and (1,3,4)
    n1, n2, n3, n4 = c0[:, 0], c0[:, 1], c0[:, 2], c0[:, 3]
    a123 = calculate_area(x[n1], x[n2], x[n3], y[n1], y[n2], y[n3])
    quad = tq == 4
    n4q = np.where(quad, n4, n1)
    a134 = calculate_area(x[n1], x[n3], x[n4q], y[n1], y[n3], y[n4q])
    a124 = calculate_area(x[n1], x[n2], x[n4q], y[n1], y[n2], y[n4q])
    a234 = calculate_area(x[n2], x[n3], x[n4q], y[n2], y[n3], y[n4q])
    if np.any(quad & ((a123 <= 0) | (a134 <= 0) | (a124 <= 0) | (a234 <= 0))):
        raise ValueError("concave quadrangle (read_cell_inp.f90:55-58)")
    area = np.where(quad, a123 + a134, a123)
    if np.any(area <= 0):
        raise ValueError("negative area (read_cell_inp.f90:61-64)")

    # --- adj_cellnum_at_node / node_count_each_element (set_geometry_1.f90:71-88):
    # traversal order is cell ascending, local node ascending.
    li = np.tile(np.arange(1, 5), nc)
    ci = np.repeat(np.arange(1, nc + 1), 4)
    nd = cells.ravel()
    valid = li <= np.repeat(tq, 4)
    li, ci, nd = li[valid], ci[valid], nd[valid]
    order = np.argsort(nd, kind="stable")
    nd_s, ci_s, li_s = nd[order], ci[order], li[order]
    counts = np.bincount(nd_s, minlength=nn + 1)[1:]
    if np.any(counts == 0):
        raise ValueError("hanging node (set_geometry_1.f90:83-88)")
    if counts.max() > max_nb:
        raise ValueError("too many neighbours at a node (set_geometry_1.f90:75-78)")
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    pos = np.arange(len(nd_s)) - starts[nd_s - 1]
    adj_cells_at_node = counts.astype(np.int32)
    adj_cellnum_at_node = np.zeros((nn, max_nb), dtype=np.int32)
    node_count_each_element = np.zeros((nn, max_nb), dtype=np.int32)
    adj_cellnum_at_node[nd_s - 1, pos] = ci_s
    node_count_each_element[nd_s - 1, pos] = li_s

    # --- adj_nodenum_at_node (set_geometry_1.f90:160-184): for each node, the other nodes of
    # its cells in discovery order (adjacent cell order, then local node order), no repeats.
    # The reference tests nd == i inside its loop over the list, so a node that is the first
    # local node of its first cell lists itself first; that is kept.
    rows_node, rows_seq, rows_nb = [], [], []
    for j in range(max_nb):
        cj = adj_cellnum_at_node[:, j]
        has = cj > 0
        for k in range(4):
            nbk = np.where(has, cells[np.maximum(cj, 1) - 1, k], 0)
            okk = has & (k < tq[np.maximum(cj, 1) - 1]) & ((nbk != np.arange(1, nn + 1)) | (j == 0 and k == 0))
            idx = np.nonzero(okk)[0]
            rows_node.append(idx)
            rows_seq.append(np.full(len(idx), j * 4 + k))
            rows_nb.append(nbk[idx])
    rn = np.concatenate(rows_node)
    rs = np.concatenate(rows_seq)
    rb = np.concatenate(rows_nb)
    o = np.lexsort((rs, rb, rn))          # by node, neighbour, seq
    rn, rs, rb = rn[o], rs[o], rb[o]
    first = np.ones(len(rn), dtype=bool)
    first[1:] = (rn[1:] != rn[:-1]) | (rb[1:] != rb[:-1])
    rn, rs, rb = rn[first], rs[first], rb[first]
    o = np.lexsort((rs, rn))
    rn, rs, rb = rn[o], rs[o], rb[o]
    ncount = np.bincount(rn, minlength=nn)
    if ncount.max() > max_nb:
        raise ValueError("too many surrounding nodes (set_geometry_1.f90:123-126)")
    nstart = np.concatenate([[0], np.cumsum(ncount)[:-1]])
    npos = np.arange(len(rn)) - nstart[rn] + 1
    adj_nodes_at_node = ncount.astype(np.int32)
    adj_nodenum_at_node = np.zeros((nn, max_nb + 1), dtype=np.int32)
    adj_nodenum_at_node[rn, npos] = rb

    # --- edges of each cell: edge l joins local nodes start_end_node(tq,l,1..2)
    e1 = np.zeros((nc, 4), dtype=np.int64)
    e2 = np.zeros((nc, 4), dtype=np.int64)
    for l in range(1, 5):
        for k in (3, 4):
            m = tq == k
            if l > k:
                continue
            e1[m, l - 1] = cells[m, se[k, l, 1] - 1]
            e2[m, l - 1] = cells[m, se[k, l, 2] - 1]
    # --- adj_cellnum_at_cell (set_geometry_1.f90:146-163): the other cell holding both nodes
    key_a = np.minimum(e1, e2)
    key_b = np.maximum(e1, e2)
    ev = np.zeros((nc, 4), dtype=bool)
    for l in range(4):
        ev[:, l] = l < tq
    keys = key_a * (nn + 1) + key_b
    flat_c = np.repeat(np.arange(1, nc + 1), 4).reshape(nc, 4)
    kk = keys[ev]
    cc = flat_c[ev]
    order = np.argsort(kk, kind="stable")
    kk_s, cc_s = kk[order], cc[order]
    if len(kk_s) > 2 and np.any((kk_s[2:] == kk_s[:-2])):
        raise ValueError("non-conforming mesh: an edge is shared by more than two cells")
    partner = np.zeros(len(kk_s), dtype=np.int64)
    same_next = np.zeros(len(kk_s), dtype=bool)
    same_next[:-1] = kk_s[:-1] == kk_s[1:]
    partner[:-1][same_next[:-1]] = cc_s[1:][same_next[:-1]]
    same_prev = np.zeros(len(kk_s), dtype=bool)
    same_prev[1:] = kk_s[1:] == kk_s[:-1]
    partner[1:][same_prev[1:]] = cc_s[:-1][same_prev[1:]]
    adj_flat = np.zeros(len(kk_s), dtype=np.int64)
    adj_flat[order] = partner
    adj_cellnum_at_cell = np.zeros((nc, 4), dtype=np.int32)
    adj_cellnum_at_cell[ev] = adj_flat

    # --- faces (set_geometry_1.f90:171-256): numbered in cell order, local edge order, when
    # the edge is a boundary or the cell has the smaller index.
    newface = ev & ((adj_cellnum_at_cell == 0) | (flat_c < adj_cellnum_at_cell))
    nf = int(newface.sum())
    if nf < nc or nf < nn:
        raise ValueError("weird grid with maxface < maxele or maxface < maxnod (set_geometry_1.f90:181-184)")
    facenum_at_cell = np.zeros((nc, 4), dtype=np.int32)
    facenum_at_cell[newface] = np.arange(1, nf + 1)
    fc = flat_c[newface]
    fl = np.nonzero(newface)[1] + 1
    fn1 = e1[newface]
    fn2 = e2[newface]
    fadj2 = adj_cellnum_at_cell[newface].astype(np.int64)
    # neighbour's local index of this face: first l2 with adj_cellnum_at_cell(l2,nb) == i
    nbm = fadj2 > 0
    nbc = fadj2[nbm]
    own = fc[nbm]
    idx1 = np.zeros(len(nbc), dtype=np.int64)
    found = np.zeros(len(nbc), dtype=bool)
    for l2 in range(4):
        hit = (~found) & (adj_cellnum_at_cell[nbc - 1, l2] == own)
        idx1[hit] = l2
        found |= hit
    if not np.all(found):
        raise ValueError("wrong ball info (set_geometry_1.f90:248-251)")
    facenum_at_cell[nbc - 1, idx1] = np.nonzero(nbm)[0] + 1
    adj_cellnum_at_face = np.stack([fc, fadj2], axis=1).astype(np.int32)
    nodenum_at_face = np.stack([fn1, fn2], axis=1).astype(np.int32)
    xn1, yn1 = x[fn1 - 1], y[fn1 - 1]
    xn2, yn2 = x[fn2 - 1], y[fn2 - 1]
    x_face = (xn1 + xn2) * 0.5
    y_face = (yn1 + yn2) * 0.5
    h_face = (hn[fn1 - 1] + hn[fn2 - 1]) * 0.5
    face_length = np.sqrt((xn2 - xn1) ** 2 + (yn2 - yn1) ** 2)
    if np.any(face_length == 0):
        raise ValueError("zero face_length (set_geometry_1.f90:234-237)")

    # --- sign_in_outflow (set_geometry_1.f90:278-284), integer division truncating to zero
    sign_in_outflow = np.zeros((nc, 4), dtype=np.int32)
    f = facenum_at_cell
    a1 = np.where(ev, adj_cellnum_at_face[np.maximum(f, 1) - 1, 0], 0).astype(np.int64)
    a2 = np.where(ev, adj_cellnum_at_face[np.maximum(f, 1) - 1, 1], 0).astype(np.int64)
    num = a2 - 2 * flat_c + a1
    den = a2 - a1
    den_safe = np.where(ev, den, 1)
    q = np.abs(num) // np.abs(den_safe) * np.sign(num) * np.sign(den_safe)
    sign_in_outflow[ev] = q[ev]

    # --- cell centres and h_cell (set_geometry_1.f90:298-310)
    x_sum = np.zeros(nc)
    y_sum = np.zeros(nc)
    h_cell = np.zeros(nc)
    for l in range(4):
        m = l < tq
        x_sum[m] = x_sum[m] + x[cells[m, l] - 1]
        y_sum[m] = y_sum[m] + y[cells[m, l] - 1]
        hf = h_face[facenum_at_cell[m, l] - 1]
        h_cell[m] = np.where(hf > h_cell[m], hf, h_cell[m])
    x_cell = x_sum / tq
    y_cell = y_sum / tq

    # --- Voronoi centres (calculate_voronoi_center.f90:36-96, 170-207) or centroids
    delta_j = np.zeros(nf)
    if voronoi == 1:
        tri = tq == 3
        xi, yi = x[c0[:, 0]], y[c0[:, 0]]
        xj, yj = x[c0[:, 1]], y[c0[:, 1]]
        xk, yk = x[c0[:, 2]], y[c0[:, 2]]
        xij = 0.5 * (xi + xj)
        yij = 0.5 * (yi + yj)
        xjk = 0.5 * (xj + xk)
        yjk = 0.5 * (yj + yk)
        numer = (xij - xjk) * (xj - xi) + (yij - yjk) * (yj - yi)
        denom = (xj - xi) * (yk - yj) - (xk - xj) * (yj - yi)
        if np.any(tri & (denom == 0.0)):
            raise ValueError("denominator of voronoi is zero (calculate_voronoi_center.f90:58-64)")
        dsafe = np.where(denom == 0.0, 1.0, denom)
        vx_t = xjk + numer / dsafe * (yk - yj)
        vy_t = yjk - numer / dsafe * (xk - xj)
        tx = np.zeros(nc)
        ty = np.zeros(nc)
        for l in range(4):
            m = l < tq
            tx[m] = tx[m] + x[cells[m, l] - 1]
            ty[m] = ty[m] + y[cells[m, l] - 1]
        vx = np.where(tri, vx_t, tx / 4.0)
        vy = np.where(tri, vy_t, ty / 4.0)
        x_cell, y_cell = vx, vy
    inner = adj_cellnum_at_face[:, 1] != 0
    ia = adj_cellnum_at_face[:, 0] - 1
    ib = np.maximum(adj_cellnum_at_face[:, 1], 1) - 1
    d_in = np.sqrt((x_cell[ib] - x_cell[ia]) ** 2 + (y_cell[ib] - y_cell[ia]) ** 2)
    if np.any(inner & (d_in == 0)):
        raise ValueError("zero distance between centres")
    d_bd = np.sqrt((x_cell[ia] - x_face) ** 2 + (y_cell[ia] - y_face) ** 2) * 2.0
    delta_j = np.where(inner, d_in, d_bd)

    # --- face angles (set_geometry_1.f90:352-368); glibc trig, as gfortran calls it
    cos_theta = np.empty(nf)
    sin_theta = np.empty(nf)
    cos_theta2 = np.empty(nf)
    sin_theta2 = np.empty(nf)
    for j in range(nf):
        t0 = math.atan2(xn1[j] - xn2[j], yn2[j] - yn1[j])
        cos_theta[j] = math.cos(t0)
        sin_theta[j] = math.sin(t0)
        if adj_cellnum_at_face[j, 1] == 0:
            t1 = t0
        else:
            c1 = adj_cellnum_at_face[j, 0] - 1
            c2 = adj_cellnum_at_face[j, 1] - 1
            t1 = math.atan2(y_cell[c2] - y_cell[c1], x_cell[c2] - x_cell[c1])
        t2 = t1 - t0
        cos_theta2[j] = math.cos(t2)
        sin_theta2[j] = math.sin(t2)

    arrays = dict(
        x_node=x, y_node=y, h_node=hn,
        adj_cells_at_node=adj_cells_at_node,
        adj_cellnum_at_node=adj_cellnum_at_node,
        node_count_each_element=node_count_each_element,
        adj_nodes_at_node=adj_nodes_at_node,
        adj_nodenum_at_node=adj_nodenum_at_node,
        x_cell=x_cell, y_cell=y_cell, h_cell=h_cell, area=area,
        tri_or_quad=tq, nodenum_at_cell=raw.cells.astype(np.int32),
        facenum_at_cell=facenum_at_cell, adj_cellnum_at_cell=adj_cellnum_at_cell,
        sign_in_outflow=sign_in_outflow,
        x_face=x_face, y_face=y_face, h_face=h_face, face_length=face_length, delta_j=delta_j,
        cos_theta=cos_theta, sin_theta=sin_theta, cos_theta2=cos_theta2, sin_theta2=sin_theta2,
        adj_cellnum_at_face=adj_cellnum_at_face, nodenum_at_face=nodenum_at_face,
    )
    return Geometry(n_nodes=nn, n_cells=nc, n_faces=nf, max_nb=max_nb, arrays=arrays)


def find_element_and_face(geo: Geometry, n1: int, n2: int) -> tuple[int, int]:
    """find_element_and_face.f90:9-67: the cell whose CCW node list holds (n1, n2)
    consecutively, and the face stored as (n1, n2).  Returns 1-based ids, 0 if absent."""
    a = geo.arrays
    cells = a["nodenum_at_cell"]
    element_id = 0
    nxt = np.roll(cells, -1, axis=1)
    nxt[:, 3] = np.where(cells[:, 3] == 0, 0, cells[:, 0])
    nxt_tri = cells.copy()
    # consecutive pairs (j1, j2) with j2 = j1+1 wrapping to 1, and the triangle wrap 3 -> 1
    for j1 in range(4):
        nod1 = cells[:, j1]
        nod2 = cells[:, (j1 + 1) % 4]
        nod2 = np.where(nod2 != 0, nod2, cells[:, 0])
        hit = np.nonzero((nod1 == n1) & (nod2 == n2))[0]
        if len(hit):
            cand = int(hit[0]) + 1
            element_id = cand if element_id == 0 else min(element_id, cand)
    del nxt, nxt_tri
    fnodes = a["nodenum_at_face"]
    hit = np.nonzero((fnodes[:, 0] == n1) & (fnodes[:, 1] == n2))[0]
    face_id = int(hit[0]) + 1 if len(hit) else 0
    return element_id, face_id


def find_elements_and_faces(geo: Geometry, pairs) -> tuple[np.ndarray, np.ndarray]:
    """find_element_and_face.f90:9-67 for many node pairs at once: for each (n1, n2), the lowest
    cell id whose CCW node list holds n1 then n2 consecutively, and the lowest face stored as
    (n1, n2); 1-based ids, 0 if absent."""
    a = geo.arrays
    cells = a["nodenum_at_cell"]
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    base = np.int64(geo.n_nodes + 1)
    keys, ids = [], []
    cell_ids = np.arange(1, cells.shape[0] + 1, dtype=np.int64)
    for j1 in range(4):
        nod1 = cells[:, j1].astype(np.int64)
        nod2 = cells[:, (j1 + 1) % 4].astype(np.int64)
        nod2 = np.where(nod2 != 0, nod2, cells[:, 0])
        m = nod1 != 0
        keys.append(nod1[m] * base + nod2[m])
        ids.append(cell_ids[m])

    def lookup(k_all, id_all, q):
        order = np.lexsort((id_all, k_all))
        ks, vs = k_all[order], id_all[order]
        first = np.ones(len(ks), bool)
        first[1:] = ks[1:] != ks[:-1]
        ks, vs = ks[first], vs[first]
        pos = np.searchsorted(ks, q)
        pos = np.minimum(pos, len(ks) - 1)
        return np.where(ks[pos] == q, vs[pos], 0).astype(np.int32)

    q = pairs[:, 0] * base + pairs[:, 1]
    elem = lookup(np.concatenate(keys), np.concatenate(ids), q)
    fn = a["nodenum_at_face"].astype(np.int64)
    face = lookup(fn[:, 0] * base + fn[:, 1], np.arange(1, fn.shape[0] + 1, dtype=np.int64), q)
    return elem, face


def bottom_layers(h: np.ndarray, msl: float, z_level: np.ndarray) -> np.ndarray:
    """set_geometry_2.f90:101-189: first k with z_level(k) <= MSL-h < z_level(k+1), plus 1."""
    L = len(z_level) - 1
    b = np.zeros(len(h), dtype=np.int32)
    z = msl - h
    for k in range(L - 1, -1, -1):
        m = (z >= z_level[k]) & (z < z_level[k + 1])
        b = np.where(m, k + 1, b)
    if np.any(b == 0):
        raise ValueError("either MSL < depth or land height above the highest level (set_geometry_2.f90)")
    return b
