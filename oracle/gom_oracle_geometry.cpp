// gom_oracle_geometry.cpp -- TEST INFRASTRUCTURE: the CPU oracle of gom_geometry_build.
//
// A serial restatement of GOM's start-up geometry, loop for loop as the reference writes it:
// the cell areas of read_cell_inp.f90:54-87, set_geometry_1.f90 (start_end_node :78-93,
// node-cell adjacency :109-135, node-node adjacency :160-184, cell-cell adjacency :206-225,
// face count :241-257, faces :268-345, sign_in_outflow :375-384, centres :395-411, delta_j
// :446-477, angles :495-515), calculate_voronoi_center.f90:36-208, set_geometry_2.f90 (boundary
// cells and faces :17-66, bottom layers :101-189), the river cells and faces of
// read_main_inp.f90:810-829 with find_element_and_face.f90:9-67, and initial_wetdry_node of
// read_node_inp.f90:79-81.  Only the tests call it, to check the CUDA build and the host mesh
// builder.  Built with the rest of the oracle (-ffp-contract=off: no fused multiply-add).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/gom_core.h"

namespace {

struct Fail {
    int site = 0, entity = 0, kind = GOM_ENTITY_OTHER;
    bool set(int s, int e, int k = GOM_ENTITY_OTHER) {
        if (site == 0) {
            site = s;
            entity = e;
            kind = k;
        }
        return false;
    }
};

// mod_function_library.f90:49-60
double calculate_area(double x1, double x2, double x3, double y1, double y2, double y3) {
    return std::fabs((x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3)) * 0.5;
}

bool build(const gom_mesh &m, gom_mesh_geometry &o, Fail &f) {
    const int NN = m.n_nodes, NC = m.n_cells, NB = m.max_nb, L = m.n_layers;
    auto x_node = [&](int i) { return m.x_node[i - 1]; };
    auto y_node = [&](int i) { return m.y_node[i - 1]; };
    auto h_node = [&](int i) { return m.h_node[i - 1]; };
    auto tq = [&](int i) { return m.tri_or_quad[i - 1]; };
    auto cnode = [&](int l, int i) { return m.nodenum_at_cell[(size_t)(i - 1) * 4 + l - 1]; };
    auto z_level = [&](int k) { return m.z_level[k]; };

    // read_cell_inp.f90:54-87
    std::vector<double> area(NC + 1, 0.0);
    for (int i = 1; i <= NC; ++i) {
        const int n1 = cnode(1, i), n2 = cnode(2, i), n3 = cnode(3, i);
        if (tq(i) == 3) {
            area[i] = calculate_area(x_node(n1), x_node(n2), x_node(n3), y_node(n1), y_node(n2), y_node(n3));
        } else {
            const int n4 = cnode(4, i);
            const double t1 = calculate_area(x_node(n1), x_node(n2), x_node(n3), y_node(n1), y_node(n2), y_node(n3));
            const double t2 = calculate_area(x_node(n1), x_node(n3), x_node(n4), y_node(n1), y_node(n3), y_node(n4));
            const double t3 = calculate_area(x_node(n1), x_node(n2), x_node(n4), y_node(n1), y_node(n2), y_node(n4));
            const double t4 = calculate_area(x_node(n2), x_node(n3), x_node(n4), y_node(n2), y_node(n3), y_node(n4));
            if (t1 <= 0.0 || t2 <= 0.0 || t3 <= 0.0 || t4 <= 0.0) return f.set(GOM_GEO_CONCAVE, i, GOM_ENTITY_CELL);
            area[i] = t1 + t2;
        }
        if (area[i] <= 0.0) return f.set(GOM_GEO_AREA, i, GOM_ENTITY_CELL);
    }

    // set_geometry_1.f90:78-93
    int start_end_node[5][5][4] = {};
    for (int k = 3; k <= 4; ++k)
        for (int i = 1; i <= k; ++i)
            for (int j = 1; j <= k - 1; ++j) {
                int v = i + j;
                if (v > k) v = v - k;
                start_end_node[k][i][j] = v;
            }

    // set_geometry_1.f90:109-135; a node past max_nb is counted on, then reported
    std::vector<int> adj_cells_at_node(NN + 1, 0), adj_cellnum_at_node((size_t)(NN + 1) * NB, 0),
        node_count_each_element((size_t)(NN + 1) * NB, 0);
    auto acn = [&](int j, int i) -> int & { return adj_cellnum_at_node[(size_t)(i - 1) * NB + j - 1]; };
    auto ncee = [&](int j, int i) -> int & { return node_count_each_element[(size_t)(i - 1) * NB + j - 1]; };
    int over = 0;
    for (int i = 1; i <= NC; ++i)
        for (int l = 1; l <= tq(i); ++l) {
            const int nd = cnode(l, i);
            adj_cells_at_node[nd] = adj_cells_at_node[nd] + 1;
            if (adj_cells_at_node[nd] > NB) {
                if (over == 0 || nd < over) over = nd;
                continue;
            }
            acn(adj_cells_at_node[nd], nd) = i;
            ncee(adj_cells_at_node[nd], nd) = l;
        }
    if (over) return f.set(GOM_GEO_MAX_NB, over, GOM_ENTITY_NODE);
    for (int i = 1; i <= NN; ++i)
        if (adj_cells_at_node[i] == 0) return f.set(GOM_GEO_HANGING, i, GOM_ENTITY_NODE);

    // set_geometry_1.f90:160-184
    std::vector<int> adj_nodes_at_node(NN + 1, 0), adj_nodenum_at_node((size_t)(NN + 1) * (NB + 1), 0);
    auto ann = [&](int j, int i) -> int & { return adj_nodenum_at_node[(size_t)(i - 1) * (NB + 1) + j]; };
    for (int i = 1; i <= NN; ++i)
        for (int j = 1; j <= adj_cells_at_node[i]; ++j) {
            const int ie = acn(j, i);
            for (int k = 1; k <= tq(ie); ++k) {
                const int nd = cnode(k, ie);
                bool skip = false;
                for (int l = 1; l <= adj_nodes_at_node[i]; ++l)
                    if (nd == i || nd == ann(l, i)) {
                        skip = true;
                        break;
                    }
                if (skip) continue;
                adj_nodes_at_node[i] = adj_nodes_at_node[i] + 1;
                if (adj_nodes_at_node[i] > NB) return f.set(GOM_GEO_SURROUNDING, i, GOM_ENTITY_NODE);
                ann(adj_nodes_at_node[i], i) = nd;
            }
        }

    // set_geometry_1.f90:206-225: the last cell around nd1 (other than i) that holds nd2
    std::vector<int> adj_cellnum_at_cell((size_t)(NC + 1) * 4, 0);
    auto acc = [&](int l, int i) -> int & { return adj_cellnum_at_cell[(size_t)(i - 1) * 4 + l - 1]; };
    for (int i = 1; i <= NC; ++i)
        for (int l = 1; l <= tq(i); ++l) {
            acc(l, i) = 0;
            const int nd1 = cnode(start_end_node[tq(i)][l][1], i);
            const int nd2 = cnode(start_end_node[tq(i)][l][2], i);
            for (int k = 1; k <= adj_cells_at_node[nd1]; ++k) {
                const int nd = acn(k, nd1);
                if (nd != i && (cnode(1, nd) == nd2 || cnode(2, nd) == nd2 || cnode(3, nd) == nd2 ||
                                (tq(nd) == 4 && cnode(4, nd) == nd2)))
                    acc(l, i) = nd;
            }
        }

    // set_geometry_1.f90:241-257
    int maxface = 0;
    for (int i = 1; i <= NC; ++i)
        for (int l = 1; l <= tq(i); ++l)
            if (acc(l, i) == 0 || i < acc(l, i)) maxface = maxface + 1;
    if (maxface < NC || maxface < NN) return f.set(GOM_GEO_FACE_COUNT, maxface);
    if (maxface > o.face_capacity) return f.set(GOM_GEO_FACE_COUNT, maxface);
    const int NF = maxface;

    // set_geometry_1.f90:268-345
    std::vector<int> facenum_at_cell((size_t)(NC + 1) * 4, 0), adj_cellnum_at_face((size_t)(NF + 1) * 2, 0),
        nodenum_at_face((size_t)(NF + 1) * 2, 0);
    auto fac = [&](int l, int i) -> int & { return facenum_at_cell[(size_t)(i - 1) * 4 + l - 1]; };
    auto acf = [&](int k, int j) -> int & { return adj_cellnum_at_face[(size_t)(j - 1) * 2 + k - 1]; };
    auto nof = [&](int k, int j) -> int & { return nodenum_at_face[(size_t)(j - 1) * 2 + k - 1]; };
    std::vector<double> xn1(NF + 1), xn2(NF + 1), yn1(NF + 1), yn2(NF + 1), x_face(NF + 1), y_face(NF + 1),
        h_face(NF + 1), face_length(NF + 1);
    maxface = 0;
    for (int i = 1; i <= NC; ++i)
        for (int l = 1; l <= tq(i); ++l) {
            const int nd1 = cnode(start_end_node[tq(i)][l][1], i);
            const int nd2 = cnode(start_end_node[tq(i)][l][2], i);
            if (!(acc(l, i) == 0 || i < acc(l, i))) continue;
            maxface = maxface + 1;
            const int j = maxface;
            fac(l, i) = j;
            acf(1, j) = i;
            nof(1, j) = nd1;
            nof(2, j) = nd2;
            xn1[j] = x_node(nd1);
            yn1[j] = y_node(nd1);
            xn2[j] = x_node(nd2);
            yn2[j] = y_node(nd2);
            x_face[j] = (xn1[j] + xn2[j]) * 0.5;
            y_face[j] = (yn1[j] + yn2[j]) * 0.5;
            h_face[j] = (h_node(nd1) + h_node(nd2)) * 0.5;
            face_length[j] = std::sqrt((xn2[j] - xn1[j]) * (xn2[j] - xn1[j]) + (yn2[j] - yn1[j]) * (yn2[j] - yn1[j]));
            if (face_length[j] == 0) return f.set(GOM_GEO_FACE_LENGTH, j, GOM_ENTITY_FACE);
            acf(2, j) = acc(l, i);
            if (acc(l, i) != 0) {
                const int t = acc(l, i);
                int index1 = 0;
                for (int l2 = 1; l2 <= tq(t); ++l2)
                    if (acc(l2, t) == i) {
                        index1 = l2;
                        break;
                    }
                if (index1 == 0) return f.set(GOM_GEO_BALL, i, GOM_ENTITY_CELL);
                fac(index1, t) = j;
            }
        }

    // set_geometry_1.f90:375-384 (integer division truncates toward zero in both languages)
    std::vector<int> sign_in_outflow((size_t)(NC + 1) * 4, 0);
    for (int i = 1; i <= NC; ++i)
        for (int l = 1; l <= tq(i); ++l) {
            const int jsj = fac(l, i);
            sign_in_outflow[(size_t)(i - 1) * 4 + l - 1] = (acf(2, jsj) - 2 * i + acf(1, jsj)) / (acf(2, jsj) - acf(1, jsj));
        }

    // set_geometry_1.f90:397-411
    std::vector<double> x_cell(NC + 1, 0.0), y_cell(NC + 1, 0.0), h_cell(NC + 1, 0.0);
    for (int i = 1; i <= NC; ++i) {
        double x_sum = 0.0, y_sum = 0.0;
        for (int l = 1; l <= tq(i); ++l) {
            x_sum = x_sum + x_node(cnode(l, i));
            y_sum = y_sum + y_node(cnode(l, i));
            if (h_face[fac(l, i)] > h_cell[i]) h_cell[i] = h_face[fac(l, i)];
        }
        x_cell[i] = x_sum / tq(i);
        y_cell[i] = y_sum / tq(i);
    }

    // calculate_voronoi_center.f90:36-208 or set_geometry_1.f90:446-477
    std::vector<double> delta_j(NF + 1, 0.0);
    if (m.voronoi == 1) {
        std::vector<double> vx(NC + 1, 0.0), vy(NC + 1, 0.0);
        for (int i = 1; i <= NC; ++i) {
            if (tq(i) == 3) {
                const double xi = x_node(cnode(1, i)), yi = y_node(cnode(1, i));
                const double xj = x_node(cnode(2, i)), yj = y_node(cnode(2, i));
                const double xk = x_node(cnode(3, i)), yk = y_node(cnode(3, i));
                const double xij = 0.5 * (xi + xj), yij = 0.5 * (yi + yj);
                const double xjk = 0.5 * (xj + xk), yjk = 0.5 * (yj + yk);
                const double numerator = (xij - xjk) * (xj - xi) + (yij - yjk) * (yj - yi);
                const double denominator = (xj - xi) * (yk - yj) - (xk - xj) * (yj - yi);
                if (denominator != 0.0) {
                    vx[i] = xjk + numerator / denominator * (yk - yj);
                    vy[i] = yjk - numerator / denominator * (xk - xj);
                } else {
                    return f.set(GOM_GEO_VORONOI, i, GOM_ENTITY_CELL);
                }
            } else if (tq(i) == 4) {
                double tx = 0.0, ty = 0.0;
                for (int l = 1; l <= tq(i); ++l) {
                    tx = tx + x_node(cnode(l, i));
                    ty = ty + y_node(cnode(l, i));
                }
                vx[i] = tx / 4.0;
                vy[i] = ty / 4.0;
            }
        }
        std::vector<double> dv(NF + 1, 0.0);
        for (int j = 1; j <= NF; ++j)
            if (acf(2, j) != 0) {
                const double dx = vx[acf(2, j)] - vx[acf(1, j)], dy = vy[acf(2, j)] - vy[acf(1, j)];
                dv[j] = std::sqrt(dx * dx + dy * dy);
                if (dv[j] == 0.0) return f.set(GOM_GEO_CENTRES, j, GOM_ENTITY_FACE);
            }
        for (int i = 1; i <= NC; ++i) {
            x_cell[i] = vx[i];
            y_cell[i] = vy[i];
        }
        for (int j = 1; j <= NF; ++j) {
            if (acf(2, j) != 0) {
                delta_j[j] = dv[j];
            } else {
                const double dx = x_cell[acf(1, j)] - x_face[j], dy = y_cell[acf(1, j)] - y_face[j];
                delta_j[j] = std::sqrt(dx * dx + dy * dy) * 2.0;
            }
        }
    } else {
        for (int j = 1; j <= NF; ++j) {
            if (acf(2, j) != 0) {
                const double dx = x_cell[acf(2, j)] - x_cell[acf(1, j)], dy = y_cell[acf(2, j)] - y_cell[acf(1, j)];
                delta_j[j] = std::sqrt(dx * dx + dy * dy);
                if (delta_j[j] == 0) return f.set(GOM_GEO_CENTRES, j, GOM_ENTITY_FACE);
            }
            if (acf(2, j) == 0) {
                const double dx = x_cell[acf(1, j)] - x_face[j], dy = y_cell[acf(1, j)] - y_face[j];
                delta_j[j] = std::sqrt(dx * dx + dy * dy) * 2.0;
            }
        }
    }

    // set_geometry_1.f90:495-515 (the C library's atan2 / cos / sin, as gfortran calls them)
    std::vector<double> cos_t(NF + 1), sin_t(NF + 1), cos_t2(NF + 1), sin_t2(NF + 1);
    for (int j = 1; j <= NF; ++j) {
        const double t0 = std::atan2(xn1[j] - xn2[j], yn2[j] - yn1[j]);
        cos_t[j] = std::cos(t0);
        sin_t[j] = std::sin(t0);
        double t1;
        if (acf(2, j) == 0) {
            t1 = t0;
        } else {
            const double x1 = x_cell[acf(1, j)], y1 = y_cell[acf(1, j)];
            const double x2 = x_cell[acf(2, j)], y2 = y_cell[acf(2, j)];
            t1 = std::atan2(y2 - y1, x2 - x1);
        }
        const double t2 = (t1 - t0);
        cos_t2[j] = std::cos(t2);
        sin_t2[j] = std::sin(t2);
    }

    // find_element_and_face.f90:9-67
    auto find = [&](int n1, int n2, int &element_id, int &face_id) {
        face_id = 0;
        element_id = 0;
        for (int i = 1; i <= NC && element_id == 0; ++i)
            for (int j1 = 1; j1 <= 4; ++j1) {
                const int nod1 = cnode(j1, i);
                int j2 = j1 + 1;
                if (j2 > 4) j2 = 1;
                int nod2 = cnode(j2, i);
                if (nod2 == 0) nod2 = cnode(1, i);
                if (nod1 == n1 && nod2 == n2) {
                    element_id = i;
                    break;
                }
            }
        for (int j = 1; j <= NF; ++j)
            if (n1 == nof(1, j) && n2 == nof(2, j)) {
                face_id = j;
                break;
            }
    };
    // set_geometry_2.f90:17-66 and read_main_inp.f90:810-829
    std::vector<int> ob_cell(m.n_ob + 1, 0), ob_face(m.n_ob + 1, 0), q_cell(m.n_qb + 1, 0), q_face(m.n_qb + 1, 0);
    for (int i = 1; i <= m.n_ob; ++i) {
        find(m.ob_nodes[(size_t)(i - 1) * 2], m.ob_nodes[(size_t)(i - 1) * 2 + 1], ob_cell[i], ob_face[i]);
        if (ob_cell[i] == 0 || ob_face[i] == 0) return f.set(GOM_GEO_BOUNDARY, i);
    }
    for (int i = 1; i <= m.n_qb; ++i) {
        find(m.qb_nodes[(size_t)(i - 1) * 2], m.qb_nodes[(size_t)(i - 1) * 2 + 1], q_cell[i], q_face[i]);
        if (q_cell[i] == 0 || q_face[i] == 0) return f.set(GOM_GEO_BOUNDARY, m.n_ob + i);
    }
    std::vector<int> ob_element_flag(NC + 1, 0), boundary_type_of_face(NF + 1, 0), qb_element_flag(NC + 1, 0),
        isflowside3(NF + 1, 0);
    for (int i = 1; i <= m.n_ob; ++i) {
        ob_element_flag[ob_cell[i]] = i;
        boundary_type_of_face[ob_face[i]] = i;
    }
    for (int j = 1; j <= NF; ++j)
        if (acf(2, j) == 0 && boundary_type_of_face[j] == 0) boundary_type_of_face[j] = -1;
    for (int i = 1; i <= m.n_qb; ++i) {
        isflowside3[q_face[i]] = i;
        qb_element_flag[q_cell[i]] = i;
    }

    // set_geometry_2.f90:101-189: first k with z_level(k) <= MSL - h < z_level(k + 1), plus 1
    auto bottom = [&](double h) {
        for (int k = 0; k <= L - 1; ++k)
            if ((m.msl - h) >= z_level(k) && (m.msl - h) < z_level(k + 1)) return k + 1;
        return 0;
    };
    std::vector<int> b_cell(NC + 1), b_face(NF + 1), b_node(NN + 1);
    for (int i = 1; i <= NC; ++i)
        if ((b_cell[i] = bottom(h_cell[i])) == 0) return f.set(GOM_GEO_VERTICAL, i, GOM_ENTITY_CELL);
    for (int j = 1; j <= NF; ++j)
        if ((b_face[j] = bottom(h_face[j])) == 0) return f.set(GOM_GEO_VERTICAL, j, GOM_ENTITY_FACE);
    for (int i = 1; i <= NN; ++i)
        if ((b_node[i] = bottom(h_node(i))) == 0) return f.set(GOM_GEO_VERTICAL, i, GOM_ENTITY_NODE);

    // the outputs, 0-based
    o.n_faces = NF;
    auto put_i = [](int32_t *dst, const std::vector<int> &src, size_t n, size_t off) {
        if (dst)
            for (size_t q = 0; q < n; ++q) dst[q] = src[q + off];
    };
    auto put_d = [](double *dst, const std::vector<double> &src, size_t n) {
        if (dst)
            for (size_t q = 0; q < n; ++q) dst[q] = src[q + 1];
    };
    put_i(o.adj_cells_at_node, adj_cells_at_node, NN, 1);
    put_i(o.adj_cellnum_at_node, adj_cellnum_at_node, (size_t)NN * NB, 0);
    put_i(o.node_count_each_element, node_count_each_element, (size_t)NN * NB, 0);
    put_i(o.adj_nodes_at_node, adj_nodes_at_node, NN, 1);
    put_i(o.adj_nodenum_at_node, adj_nodenum_at_node, (size_t)NN * (NB + 1), 0);
    put_i(o.bottom_layer_at_node, b_node, NN, 1);
    if (o.initial_wetdry_node)
        for (int i = 1; i <= NN; ++i) o.initial_wetdry_node[i - 1] = h_node(i) <= 0.0 ? 1 : 0;
    put_d(o.x_cell, x_cell, NC);
    put_d(o.y_cell, y_cell, NC);
    put_d(o.h_cell, h_cell, NC);
    put_d(o.area, area, NC);
    put_i(o.facenum_at_cell, facenum_at_cell, (size_t)NC * 4, 0);
    put_i(o.adj_cellnum_at_cell, adj_cellnum_at_cell, (size_t)NC * 4, 0);
    put_i(o.sign_in_outflow, sign_in_outflow, (size_t)NC * 4, 0);
    put_i(o.bottom_layer_at_element, b_cell, NC, 1);
    put_i(o.ob_element_flag, ob_element_flag, NC, 1);
    put_i(o.qb_element_flag, qb_element_flag, NC, 1);
    put_d(o.x_face, x_face, NF);
    put_d(o.y_face, y_face, NF);
    put_d(o.h_face, h_face, NF);
    put_d(o.face_length, face_length, NF);
    put_d(o.delta_j, delta_j, NF);
    put_d(o.cos_theta, cos_t, NF);
    put_d(o.sin_theta, sin_t, NF);
    put_d(o.cos_theta2, cos_t2, NF);
    put_d(o.sin_theta2, sin_t2, NF);
    put_i(o.adj_cellnum_at_face, adj_cellnum_at_face, (size_t)NF * 2, 0);
    put_i(o.nodenum_at_face, nodenum_at_face, (size_t)NF * 2, 0);
    put_i(o.bottom_layer_at_face, b_face, NF, 1);
    put_i(o.boundary_type_of_face, boundary_type_of_face, NF, 1);
    put_i(o.isflowside3, isflowside3, NF, 1);
    put_i(o.ob_cell_id, ob_cell, m.n_ob, 1);
    put_i(o.ob_face_id, ob_face, m.n_ob, 1);
    put_i(o.qb_cell, q_cell, m.n_qb, 1);
    put_i(o.qb_face, q_face, m.n_qb, 1);
    return true;
}

}  // namespace

extern "C" int gom_geometry_build(const gom_mesh *mesh, gom_mesh_geometry *out, gom_status *failure) {
    if (failure) std::memset(failure, 0, sizeof(*failure));
    if (!mesh || !out || mesh->n_nodes <= 0 || mesh->n_cells <= 0 || mesh->max_nb <= 0 || mesh->n_layers <= 0 ||
        mesh->n_ob < 0 || mesh->n_qb < 0 || !mesh->x_node || !mesh->y_node || !mesh->h_node || !mesh->tri_or_quad ||
        !mesh->nodenum_at_cell || !mesh->z_level || (mesh->n_ob > 0 && !mesh->ob_nodes) ||
        (mesh->n_qb > 0 && !mesh->qb_nodes) || out->face_capacity <= 0)
        return GOM_E_ARG;
    for (int i = 0; i < mesh->n_cells; ++i) {
        const int k = mesh->tri_or_quad[i];
        if (k != 3 && k != 4) return GOM_E_ARG;
        for (int l = 0; l < 4; ++l) {
            const int nd = mesh->nodenum_at_cell[(size_t)i * 4 + l];
            if (l < k ? (nd < 1 || nd > mesh->n_nodes) : nd != 0) return GOM_E_ARG;
        }
    }
    for (int i = 0; i < 2 * (mesh->n_ob + mesh->n_qb); ++i) {
        const int nd = i < 2 * mesh->n_ob ? mesh->ob_nodes[i] : mesh->qb_nodes[i - 2 * mesh->n_ob];
        if (nd < 1 || nd > mesh->n_nodes) return GOM_E_ARG;
    }
    Fail f;
    out->n_faces = 0;
    if (build(*mesh, *out, f)) return GOM_OK;
    if (failure) {
        failure->code = GOM_E_ARG;
        failure->site = f.site;
        failure->entity = f.entity;
        failure->entity_kind = f.kind;
    }
    return GOM_E_ARG;
}
