// ORACLE — test infrastructure only (see oracle_core.hpp).
#include "oracle_core.hpp"

#include <cstdio>
#include <fstream>
#include <sstream>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

// ======================= grid input =========================================

ElemType elem_type_from_vtk(size_t t) {  // grid_io.cpp:28-48
    switch (t) {
        case 3: return ElemType::Line;
        case 5: return ElemType::Tri;
        case 9: return ElemType::Quad;
        case 10: return ElemType::Tetra;
        case 12: return ElemType::Hex;
        case 13: return ElemType::Wedge;
        case 14: return ElemType::Pyramid;
        default: throw std::runtime_error("unknown su2 element type");
    }
}

size_t vertices_of(ElemType t) {  // grid_io.cpp:72-91
    switch (t) {
        case ElemType::Line: return 2;
        case ElemType::Tri: return 3;
        case ElemType::Quad: return 4;
        case ElemType::Tetra: return 4;
        case ElemType::Hex: return 8;
        case ElemType::Wedge: return 6;
        case ElemType::Pyramid: return 5;
    }
    return 0;
}

std::vector<ElemIO> vtk_face_order(const std::vector<size_t>& v, ElemType type) {
    // grid_io.cpp:298-348
    using E = ElemType;
    switch (type) {
        case E::Line: return {{{v[0], v[1]}, E::Line}};
        case E::Tri: return {{{v[0], v[1]}, E::Line}, {{v[1], v[2]}, E::Line}, {{v[2], v[0]}, E::Line}};
        case E::Quad:
            return {{{v[0], v[1]}, E::Line}, {{v[1], v[2]}, E::Line},
                    {{v[2], v[3]}, E::Line}, {{v[3], v[0]}, E::Line}};
        case E::Tetra:
            return {{{v[0], v[1], v[2]}, E::Tri}, {{v[0], v[1], v[3]}, E::Tri},
                    {{v[1], v[2], v[3]}, E::Tri}, {{v[0], v[2], v[3]}, E::Tri}};
        case E::Hex:
            return {{{v[0], v[1], v[2], v[3]}, E::Quad}, {{v[0], v[1], v[5], v[4]}, E::Quad},
                    {{v[4], v[5], v[6], v[7]}, E::Quad}, {{v[2], v[3], v[7], v[6]}, E::Quad},
                    {{v[0], v[4], v[7], v[3]}, E::Quad}, {{v[1], v[5], v[6], v[2]}, E::Quad}};
        case E::Wedge:
            return {{{v[0], v[1], v[2]}, E::Tri}, {{v[3], v[5], v[4]}, E::Tri},
                    {{v[1], v[4], v[5], v[2]}, E::Quad}, {{v[0], v[2], v[5], v[3]}, E::Quad},
                    {{v[0], v[3], v[4], v[1]}, E::Quad}};
        case E::Pyramid:
            return {{{v[0], v[3], v[2], v[1]}, E::Quad}, {{v[2], v[3], v[4]}, E::Tri},
                    {{v[0], v[4], v[3]}, E::Tri}, {{v[0], v[1], v[4]}, E::Tri},
                    {{v[1], v[2], v[4]}, E::Tri}};
    }
    throw std::runtime_error("unreachable");
}

static void trim(std::string& s) {  // grid_io.cpp:119-125 (spaces only)
    size_t a = s.find_first_not_of(' ');
    s = (a == std::string::npos) ? "" : s.substr(a);
    size_t b = s.find_last_not_of(' ');
    s = (b == std::string::npos) ? "" : s.substr(0, b + 1);
}

static bool next_line(std::istream& f, std::string& line) {  // grid_io.cpp:145-155
    std::getline(f, line);
    if (f) { trim(line); return true; }
    return false;
}

static std::string read_string(std::string s) {  // grid_io.cpp:131-137
    s = s.substr(s.find('=') + 1);
    trim(s);
    return s;
}

static ElemIO read_element(std::string line) {  // grid_io.cpp:157-173
    size_t pos = line.find(' ');
    ElemType type = elem_type_from_vtk((size_t)std::stoi(line.substr(0, pos)));
    size_t nv = vertices_of(type);
    line = line.substr(pos + 1);
    trim(line);
    std::vector<size_t> ids;
    for (size_t i = 0; i < nv; i++) {
        pos = line.find(' ');
        ids.push_back((size_t)std::stoi(line.substr(0, pos)));
        line = (pos == std::string::npos) ? "" : line.substr(pos + 1);
        trim(line);
    }
    return {ids, type};
}

void GridIO::read_su2(const std::string& path) {  // grid_io.cpp:218-268
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::string line;
    while (next_line(f, line)) {
        if (line.rfind("NDIME", 0) == 0) {
            dim = (size_t)std::stoi(read_string(line));
        } else if (line.rfind("NPOIN", 0) == 0) {
            size_t n = (size_t)std::stoi(read_string(line));
            for (size_t i = 0; i < n; i++) {
                next_line(f, line);
                std::istringstream ss(line);
                double x = 0, y = 0, z = 0;
                ss >> x >> y;
                if (dim == 3) ss >> z;
                vertices.push_back({x, y, z});
            }
        } else if (line.rfind("NELEM", 0) == 0) {
            size_t n = (size_t)std::stoi(read_string(line));
            for (size_t i = 0; i < n; i++) {
                next_line(f, line);
                cells.push_back(read_element(line));
            }
        } else if (line.rfind("NMARK", 0) == 0) {
            size_t nm = (size_t)std::stoi(read_string(line));
            for (size_t m = 0; m < nm; m++) {
                next_line(f, line);
                std::string tag = read_string(line);
                next_line(f, line);
                size_t ne = (size_t)std::stoi(read_string(line));
                std::vector<ElemIO> elems;
                for (size_t e = 0; e < ne; e++) {
                    next_line(f, line);
                    elems.push_back(read_element(line));
                }
                auto& dst = markers[tag];
                dst.insert(dst.end(), elems.begin(), elems.end());
            }
        }
    }
}

// ======================= grid block =========================================

// interface.cpp:38-46 — key of a face = its vertex ids sorted descending
static std::string face_key(std::vector<size_t> ids) {
    std::sort(ids.begin(), ids.end(), std::greater<size_t>());
    std::string h;
    for (size_t v : ids) { h += std::to_string(v); h += ","; }
    return h;
}

template <typename T>
static T distance(const Grid<T>& g, size_t i, size_t j) {  // geom.h:11-26
    T dx = g.vx[j] - g.vx[i];
    T dy = g.vy[j] - g.vy[i];
    T dz = g.vz[j] - g.vz[i];
    return o_sqrt(dx * dx + dy * dy + dz * dz);
}

template <typename T>
static T tri_area(const Grid<T>& g, size_t a, size_t b, size_t c) {  // geom.h:28-49
    T abx = g.vx[b] - g.vx[a], aby = g.vy[b] - g.vy[a], abz = g.vz[b] - g.vz[a];
    T acx = g.vx[c] - g.vx[a], acy = g.vy[c] - g.vy[a], acz = g.vz[c] - g.vz[a];
    T crx = aby * acz - abz * acy;
    T cry = abz * acx - abx * acz;
    T crz = abx * acy - aby * acx;
    return 0.5 * o_sqrt(crx * crx + cry * cry + crz * crz);
}

template <typename T>
void Grid<T>::init(const GridIO& io, const Json& boundaries,
                   const std::map<std::string, PeriodicLink>& periodic) {
    // grid.h:89-167
    dim = io.dim;
    NV = io.vertices.size();
    vx.resize(NV); vy.resize(NV); vz.resize(NV);
    for (size_t i = 0; i < NV; i++) {
        vx[i] = T(io.vertices[i][0]); vy[i] = T(io.vertices[i][1]); vz[i] = T(io.vertices[i][2]);
    }
    std::unordered_map<std::string, size_t> lookup;
    auto lookup_id = [&](const std::vector<size_t>& ids) {
        auto it = lookup.find(face_key(ids));
        return it == lookup.end() ? NONE : it->second;
    };
    N = io.cells.size();
    for (size_t c = 0; c < N; c++) {
        cell_vertices.push_back(io.cells[c].ids);
        cell_shape.push_back(io.cells[c].type);
        std::vector<size_t> fids;
        for (const ElemIO& f : vtk_face_order(io.cells[c].ids, io.cells[c].type)) {
            std::string key = face_key(f.ids);
            auto it = lookup.find(key);
            size_t id;
            if (it == lookup.end()) {
                id = lookup.size();
                lookup.emplace(key, id);
                face_vertices.push_back(f.ids);
                face_shape.push_back(f.type);
            } else {
                id = it->second;
            }
            fids.push_back(id);
        }
        cell_faces.push_back(fids);
    }
    F = face_vertices.size();

    // setup_boundaries, grid.h:406-443 (json object order = sorted tags)
    G = 0;
    std::map<size_t, size_t> ghost_map;
    for (const auto& [tag, bc] : boundaries.items()) {
        boundary_tags.push_back(tag);
        std::vector<ElemIO> marker;
        auto it = io.markers.find(tag);
        if (it != io.markers.end()) marker = it->second;
        std::vector<size_t> ghosts, faces;
        for (const ElemIO& e : marker) {
            size_t fid = lookup_id(e.ids);
            faces.push_back(fid);
            if (bc.at("ghost_cells").as_bool()) {
                size_t gid = N + G;
                G++;
                ghosts.push_back(gid);
                ghost_map.emplace(fid, gid);
            } else {
                ghost_map.emplace(fid, NONE);
            }
        }
        ghost_cells[tag] = ghosts;
        boundary_faces[tag] = faces;
    }

    size_t NT = N + G;
    left.assign(F, NONE); right.assign(F, NONE);
    nx.assign(F, T(0.0)); ny = nx; nz = nx; t1x = nx; t1y = nx; t1z = nx;
    t2x = nx; t2y = nx; t2z = nx; cx = nx; cy = nx; cz = nx; area = nx;
    volume.assign(NT, T(0.0)); ccx = volume; ccy = volume; ccz = volume;

    // Interfaces::compute_centres, interface.h:301-323
    for (size_t f = 0; f < F; f++) {
        T x = 0.0, y = 0.0, z = 0.0;
        size_t n = face_vertices[f].size();
        for (size_t v : face_vertices[f]) { x += vx[v]; y += vy[v]; z += vz[v]; }
        cx[f] = x / (double)n; cy[f] = y / (double)n; cz[f] = z / (double)n;
    }
    // Interfaces::compute_areas, interface.h:253-299
    for (size_t f = 0; f < F; f++) {
        const auto& v = face_vertices[f];
        switch (face_shape[f]) {
            case ElemType::Line: area[f] = distance(*this, v[0], v[1]); break;
            case ElemType::Tri: area[f] = tri_area(*this, v[0], v[1], v[2]); break;
            case ElemType::Quad:
                area[f] = tri_area(*this, v[0], v[1], v[2]) + tri_area(*this, v[0], v[2], v[3]);
                break;
            default: throw std::runtime_error("invalid interface shape");
        }
    }
    // Interfaces::compute_orientations, interface.h:180-251 (+ cross, vector3.h:153-160)
    for (size_t f = 0; f < F; f++) {
        const auto& v = face_vertices[f];
        T x0 = vx[v[0]], x1 = vx[v[1]], y0 = vy[v[0]], y1 = vy[v[1]], z0 = vz[v[0]], z1 = vz[v[1]];
        T il = 1. / o_sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0) + (z1 - z0) * (z1 - z0));
        t1x[f] = il * (x1 - x0); t1y[f] = il * (y1 - y0); t1z[f] = il * (z1 - z0);
        if (face_shape[f] == ElemType::Line) {
            t2x[f] = 0.0; t2y[f] = 0.0; t2z[f] = 1.0;
        } else {
            T sx = vx[v[2]] - vx[v[0]], sy = vy[v[2]] - vy[v[0]], sz = vz[v[2]] - vz[v[0]];
            T proj = t1x[f] * sx + t1y[f] * sy + t1z[f] * sz;
            T ax = sx - proj * t1x[f], ay = sy - proj * t1y[f], az = sz - proj * t1z[f];
            T il2 = 1.0 / o_sqrt(ax * ax + ay * ay + az * az);
            t2x[f] = il2 * ax; t2y[f] = il2 * ay; t2z[f] = il2 * az;
        }
        nx[f] = t1y[f] * t2z[f] - t1z[f] * t2y[f];
        ny[f] = t1z[f] * t2x[f] - t1x[f] * t2z[f];
        nz[f] = t1x[f] * t2y[f] - t1y[f] * t2x[f];
    }
    // Cells::compute_centroids, cell.h:228-255
    for (size_t c = 0; c < N; c++) {
        T x = 0.0, y = 0.0, z = 0.0;
        size_t n = cell_vertices[c].size();
        for (size_t v : cell_vertices[c]) { x += vx[v]; y += vy[v]; z += vz[v]; }
        ccx[c] = x / (double)n; ccy[c] = y / (double)n; ccz[c] = z / (double)n;
    }
    // compute_interface_connectivity, grid.h:180-232
    outsigns.assign(N, {});
    for (size_t c = 0; c < N; c++) {
        outsigns[c].assign(cell_faces[c].size(), 0);
        for (size_t k = 0; k < cell_faces[c].size(); k++) {
            size_t f = cell_faces[c][k];
            T dx = cx[f] - ccx[c], dy = cy[f] - ccy[c], dz = cz[f] - ccz[c];
            T dot = dx * nx[f] + dy * ny[f] + dz * nz[f];
            if (dot > 0.0) { left[f] = c; outsigns[c][k] = 1; }
            else { right[f] = c; outsigns[c][k] = -1; }
        }
    }
    for (const auto& [fid, gid] : ghost_map) {
        if (fid == NONE) continue;
        if (left[fid] == NONE) left[fid] = gid; else right[fid] = gid;
    }
    // Cells::compute_volumes, cell.h:257-300 (+ geom.h:66-83)
    for (size_t c = 0; c < N; c++) {
        const auto& v = cell_vertices[c];
        switch (cell_shape[c]) {
            case ElemType::Tri: volume[c] = tri_area(*this, v[0], v[1], v[2]); break;
            case ElemType::Quad:
                volume[c] = tri_area(*this, v[0], v[1], v[2]) + tri_area(*this, v[0], v[2], v[3]);
                break;
            case ElemType::Line: throw std::runtime_error("invalid cell shape");
            default: {
                T vol = 0.0;
                for (size_t k = 0; k < cell_faces[c].size(); k++) {
                    size_t f = cell_faces[c][k];
                    double out = (double)outsigns[c][k];
                    T dot = cx[f] * out * nx[f] + cy[f] * out * ny[f] + cz[f] * out * nz[f];
                    vol += dot * area[f];
                }
                volume[c] = vol / 3.0;
            }
        }
    }
    // compute_cell_neighbours, grid.h:340-358
    cell_nbrs.assign(N, {});
    for (size_t c = 0; c < N; c++) {
        for (size_t f : cell_faces[c]) cell_nbrs[c].push_back(left[f] == c ? right[f] : left[f]);
    }
    // compute_ghost_cell_centres, grid.h:364-403
    for (const auto& [tag, faces] : boundary_faces) {
        for (size_t f : faces) {
            size_t l = left[f], r = right[f];
            size_t valid = l < N ? l : r, ghost = l < N ? r : l;
            if (ghost == NONE) continue;
            T dx = cx[f] - ccx[valid], dy = cy[f] - ccy[valid], dz = cz[f] - ccz[valid];
            ccx[ghost] = cx[f] + dx; ccy[ghost] = cy[f] + dy; ccz[ghost] = cz[f] + dz;
        }
    }

    // periodic extension: the donor of a ghost on tag A is the valid cell next to
    // the face of the partner tag whose centre equals this face centre + offset
    ghost_donor.assign(G, NONE);
    for (const auto& [tag, link] : periodic) {
        const auto& faces = boundary_faces.at(tag);
        const auto& pfaces = boundary_faces.at(link.partner);
        std::map<std::array<long long, 3>, size_t> partner_at;
        auto q = [](double v) { return (long long)std::llround(v * 1e9); };
        for (size_t f : pfaces) {
            partner_at[{q(real_part(cx[f])), q(real_part(cy[f])), q(real_part(cz[f]))}] = f;
        }
        for (size_t f : faces) {
            std::array<long long, 3> key = {q(real_part(cx[f]) + link.offset[0]),
                                            q(real_part(cy[f]) + link.offset[1]),
                                            q(real_part(cz[f]) + link.offset[2])};
            auto it = partner_at.find(key);
            if (it == partner_at.end()) throw std::runtime_error("periodic: no partner face for " + tag);
            size_t pf = it->second;
            size_t donor = left[pf] < N ? left[pf] : right[pf];
            size_t ghost = left[f] < N ? right[f] : left[f];
            ghost_donor[ghost - N] = donor;
        }
    }
}

template <typename T>
void Grid<T>::compute_gradient_weights() {  // gradient.h:119-162
    r.assign(N, {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)});
#pragma omp parallel for schedule(static)
    for (long long ci = 0; ci < (long long)N; ci++) {
        size_t i = (size_t)ci;
        T sxx = 0.0, sxy = 0.0, sxz = 0.0, syy = 0.0, syz = 0.0, szz = 0.0;
        T xi = ccx[i], yi = ccy[i], zi = ccz[i];
        for (size_t nb : cell_nbrs[i]) {
            T dx = ccx[nb] - xi, dy = ccy[nb] - yi, dz = ccz[nb] - zi;
            sxx += dx * dx; sxy += dx * dy; sxz += dx * dz;
            syy += dy * dy; syz += dy * dz; szz += dz * dz;
        }
        T r11 = o_sqrt(sxx);
        T r12 = 1.0 / r11 * sxy;
        T r22 = o_sqrt(syy - r12 * r12);
        T r13 = 1.0 / r11 * sxz;
        T r23 = 1.0 / r22 * (syz - r12 / r11 * sxz);
        T r33 = o_sqrt(szz - (r13 * r13 + r23 * r23));
        r[i][0] = r11; r[i][1] = r12; r[i][2] = r22;
        if (dim == 3) { r[i][3] = r13; r[i][4] = r23; r[i][5] = r33; }
    }
}

// WLSGradient::compute_gradients, gradient.h:65-116
template <typename T>
static void lsq_gradient(const Grid<T>& g, const std::vector<T>& values,
                         std::vector<std::array<T, 3>>& grad) {
    int dim = (int)g.dim;
#pragma omp parallel for schedule(static)
    for (long long ci = 0; ci < (long long)g.N; ci++) {
        size_t i = (size_t)ci;
        T gx = 0.0, gy = 0.0, gz = 0.0;
        T ui = values[i];
        T r11 = g.r[i][0], r12 = g.r[i][1], r22 = g.r[i][2];
        T r13 = 0.0, r23 = 0.0, r33 = 0.0;
        if (dim == 3) { r13 = g.r[i][3]; r23 = g.r[i][4]; r33 = g.r[i][5]; }
        T beta = (r12 * r23 - r13 * r23) / (r11 * r22);
        T xi = g.ccx[i], yi = g.ccy[i], zi = g.ccz[i];
        for (size_t nb : g.cell_nbrs[i]) {
            T du = values[nb] - ui;
            T dx = g.ccx[nb] - xi, dy = g.ccy[nb] - yi, dz = g.ccz[nb] - zi;
            T a1 = dx / (r11 * r11);
            T a2 = 1.0 / (r22 * r22) * (dy - r12 / r11 * dx);
            T a3 = 0.0;
            if (dim == 3) a3 = 1.0 / (r33 * r33) * (dz - r23 / r22 * dy + beta * dx);
            T w1 = a1 - r12 / r11 * a2 + beta * a3;
            T w2 = a2 - r23 / r22 * a3;
            T w3 = a3;
            gx += w1 * du; gy += w2 * du; gz += w3 * du;
        }
        grad[i] = {gx, gy, gz};
    }
}

// BarthJespersen::calculate_limiters, limiter.cpp:23-63
template <typename T>
static void barth_jespersen(const Grid<T>& g, const std::vector<T>& values,
                            const std::vector<std::array<T, 3>>& grad, double eps,
                            std::vector<T>& phi_out, BranchCode* branches, size_t stride,
                            size_t slot) {
#pragma omp parallel for schedule(static)
    for (long long ci = 0; ci < (long long)g.N; ci++) {
        size_t i = (size_t)ci;
        T Ui = values[i], Umin = Ui, Umax = Ui;
        for (size_t nb : g.cell_nbrs[i]) {
            Umin = o_min(Umin, values[nb]);
            Umax = o_max(Umax, values[nb]);
        }
        T phi = 1.0;
        BranchCode code = 0;
        T x = g.ccx[i], y = g.ccy[i], z = g.ccz[i];
        const auto& faces = g.cell_faces[i];
        for (size_t j = 0; j < faces.size(); j++) {
            size_t f = faces[j];
            T dx = g.cx[f] - x, dy = g.cy[f] - y, dz = g.cz[f] - z;
            T d2 = grad[i][0] * dx + grad[i][1] * dy + grad[i][2] * dz;
            int s = (d2 > 0.0) - (d2 < 0.0);
            d2 = (double)s * (o_abs(d2) + eps);
            T ratio;
            if (s > 0) ratio = (Umax - Ui) / d2;
            else if (s < 0) ratio = (Umin - Ui) / d2;
            if (s != 0) {
                code |= (BranchCode)(s > 0 ? 1 : 2) << (2 * j);
                // the selected operand of min(phi, ratio): ties pick ratio
                if (!(phi < ratio)) code = (code & 0xFFFFu) | ((BranchCode)(j + 1) << 16);
                phi = o_min(phi, ratio);
            }
        }
        phi_out[i] = phi;
        if (branches) branches[i * stride + slot] = code;
    }
}

// ======================= finite volume ======================================

template <typename T>
void FiniteVolume<T>::setup(const Grid<T>& grid, const FvConfig& c,
                            const std::vector<BoundaryCondition>& b) {
    cfg = c;
    dim = grid.dim;
    bcs = b;
    bc_faces.clear();
    for (const auto& tag : grid.boundary_tags) bc_faces.push_back(grid.boundary_faces.at(tag));
    flux = Conserved<T>(grid.F, dim);
    left.resize(grid.F); right.resize(grid.F); face_fs.resize(grid.F);
    std::array<T, 3> z = {T(0.0), T(0.0), T(0.0)};
    g_p.assign(grid.N, z); g_rho = g_p; g_u = g_p; g_temp = g_p; g_vx = g_p; g_vy = g_p; g_vz = g_p;
    l_p.assign(grid.N, T(0.0)); l_rho = l_p; l_u = l_p; l_temp = l_p; l_vx = l_p; l_vy = l_p; l_vz = l_p;
    branches.assign(grid.N * 5, 0);
}

template <typename T>
void FiniteVolume<T>::apply_ghost_actions(const std::vector<Action>& acts, FlowStates<T>& fs,
                                          const Grid<T>& g, const std::vector<size_t>& faces,
                                          const IdealGas& gas) {
    size_t N = g.N;
    for (const Action& a : acts) {
        for (size_t i = 0; i < faces.size(); i++) {
            size_t f = faces[i];
            size_t l = g.left[f], r = g.right[f];
            size_t ghost = l < N ? r : l;
            size_t valid = l < N ? l : r;
            switch (a.kind) {
                case ActionKind::FlowStateCopy:  // boundary.cpp:14-46
                    fs.temp[ghost] = fs_value<T>(a, 0); fs.p[ghost] = fs_value<T>(a, 1);
                    fs.rho[ghost] = fs_value<T>(a, 2); fs.e[ghost] = fs_value<T>(a, 3);
                    fs.vx[ghost] = fs_value<T>(a, 4); fs.vy[ghost] = fs_value<T>(a, 5);
                    fs.vz[ghost] = fs_value<T>(a, 6);
                    break;
                case ActionKind::InternalCopy:  // boundary.cpp:99-137
                    fs.temp[ghost] = fs.temp[valid]; fs.p[ghost] = fs.p[valid];
                    fs.rho[ghost] = fs.rho[valid]; fs.e[ghost] = fs.e[valid];
                    fs.vx[ghost] = fs.vx[valid]; fs.vy[ghost] = fs.vy[valid]; fs.vz[ghost] = fs.vz[valid];
                    break;
                case ActionKind::PeriodicCopy: {  // extension: copy from the periodic donor
                    size_t d = g.ghost_donor[ghost - N];
                    fs.temp[ghost] = fs.temp[d]; fs.p[ghost] = fs.p[d];
                    fs.rho[ghost] = fs.rho[d]; fs.e[ghost] = fs.e[d];
                    fs.vx[ghost] = fs.vx[d]; fs.vy[ghost] = fs.vy[d]; fs.vz[ghost] = fs.vz[d];
                    break;
                }
                case ActionKind::InternalCopyReflectNormal: {  // boundary.cpp:141-206
                    fs.temp[ghost] = fs.temp[valid]; fs.p[ghost] = fs.p[valid];
                    fs.rho[ghost] = fs.rho[valid]; fs.e[ghost] = fs.e[valid];
                    T x = fs.vx[valid], y = fs.vy[valid], z = fs.vz[valid];
                    T xs = -(x * g.nx[f] + y * g.ny[f] + z * g.nz[f]);
                    T ys = x * g.t1x[f] + y * g.t1y[f] + z * g.t1z[f];
                    T zs = x * g.t2x[f] + y * g.t2y[f] + z * g.t2z[f];
                    fs.vx[ghost] = xs * g.nx[f] + ys * g.t1x[f] + zs * g.t2x[f];
                    fs.vy[ghost] = xs * g.ny[f] + ys * g.t1y[f] + zs * g.t2y[f];
                    fs.vz[ghost] = xs * g.nz[f] + ys * g.t1z[f] + zs * g.t2z[f];
                    break;
                }
                case ActionKind::InternalVelCopyReflect:  // boundary.cpp:208-241
                    fs.vx[ghost] = -fs.vx[valid]; fs.vy[ghost] = -fs.vy[valid]; fs.vz[ghost] = -fs.vz[valid];
                    break;
                case ActionKind::FixTemperature:  // boundary.cpp:243-277
                    fs.temp[ghost] = 2 * T(a.value) - fs.temp[valid];
                    break;
                case ActionKind::BoundaryLayerProfile: {  // boundary.cpp:59-94
                    // the profile at the ghost centroid's height; p, T -> rho, e
                    double pos = real_part(g.ccy[ghost]);
                    T tp = a.spline_T.eval(pos);
                    fs.p[ghost] = a.value;
                    fs.temp[ghost] = tp;
                    fs.rho[ghost] = fs.p[ghost] / (gas.R * fs.temp[ghost]);
                    fs.e[ghost] = gas.Cv * fs.temp[ghost];
                    fs.vx[ghost] = a.spline_v.eval(pos);
                    fs.vy[ghost] = 0.0;
                    fs.vz[ghost] = 0.0;
                    break;
                }
                case ActionKind::SubsonicInflow: {  // boundary.cpp:284-343
                    T nxf = g.nx[f], nyf = g.ny[f], nzf = g.nz[f];
                    const T fvx = fs_value<T>(a, 4), fvy = fs_value<T>(a, 5), fvz = fs_value<T>(a, 6);
                    T vc = nxf * (fvx - fs.vx[valid]) + nyf * (fvy - fs.vy[valid]) + nzf * (fvz - fs.vz[valid]);
                    T sos = o_sqrt(gas.gamma * gas.R * fs.temp[valid]);
                    T rho_ref = fs.rho[valid];
                    T p_in = fs_value<T>(a, 1);
                    T p_face = 0.5 * (p_in + fs.p[valid] - rho_ref * sos * vc);
                    T rho_face = fs_value<T>(a, 2) + (p_face - p_in) / sos / sos;
                    T vxf = fvx - nxf * (p_in - p_face) / (rho_ref * sos);
                    T vyf = fvy - nyf * (p_in - p_face) / (rho_ref * sos);
                    T vzf = fvz - nzf * (p_in - p_face) / (rho_ref * sos);
                    fs.p[ghost] = 2 * p_face - fs.p[valid];
                    fs.rho[ghost] = 2 * rho_face - fs.rho[valid];
                    fs.temp[ghost] = fs.p[ghost] / (fs.rho[ghost] * gas.R);
                    fs.e[ghost] = gas.Cv * fs.temp[ghost];
                    fs.vx[ghost] = 2 * vxf - fs.vx[valid];
                    fs.vy[ghost] = 2 * vyf - fs.vy[valid];
                    fs.vz[ghost] = 2 * vzf - fs.vz[valid];
                    break;
                }
                case ActionKind::SubsonicOutflow: {  // boundary.cpp:347-400
                    T nxf = g.nx[f], nyf = g.ny[f], nzf = g.nz[f];
                    T p_face = a.value;
                    T rho_ref = fs.rho[valid];
                    T p_ref = fs.p[valid];
                    T sos = o_sqrt(gas.gamma * gas.R * fs.temp[valid]);
                    T rho_face = fs.rho[valid] + (p_face - p_ref) / sos / sos;
                    T vxf = fs.vx[valid] + nxf * (p_ref - p_face) / (rho_ref * sos);
                    T vyf = fs.vy[valid] + nyf * (p_ref - p_face) / (rho_ref * sos);
                    T vzf = fs.vz[valid] + nzf * (p_ref - p_face) / (rho_ref * sos);
                    fs.p[ghost] = 2 * p_face - fs.p[valid];
                    fs.rho[ghost] = 2 * rho_face - fs.rho[valid];
                    fs.temp[ghost] = fs.p[ghost] / (fs.rho[ghost] * gas.R);
                    fs.e[ghost] = gas.Cv * fs.temp[ghost];
                    fs.vx[ghost] = 2 * vxf - fs.vx[valid];
                    fs.vy[ghost] = 2 * vyf - fs.vy[valid];
                    fs.vz[ghost] = 2 * vzf - fs.vz[valid];
                    break;
                }
                case ActionKind::ConstantFlux:
                    break;  // a flux action, applied after the convective flux
            }
        }
    }
}

// linear_interpolate, convective_flux.cpp:242-255
template <typename T>
static inline T lin_interp(T value, const std::array<T, 3>& grad, T dx, T dy, T dz, T limiter,
                           bool valid) {
    T gx = 0.0, gy = 0.0, gz = 0.0;
    if (valid) { gx = grad[0]; gy = grad[1]; gz = grad[2]; }
    return value + limiter * (gx * dx + gy * dy + gz * dz);
}

// Flux calculators in the face-normal frame (flux_calculators/*.cpp)
template <typename T>
struct FaceState {
    T r, p, temp, u, v, w;
};

template <typename T>
static void hanel(const FaceState<T>& L, const FaceState<T>& R, const IdealGas& gm, T* F,
                  bool three_d) {  // hanel.cpp:7-65
    T rL = L.r, pL = L.p, eL = gm.Cv * L.temp, aL = o_sqrt(gm.gamma * gm.R * L.temp);
    T uL = L.u, vL = L.v, wL = L.w;
    T keL = 0.5 * (uL * uL + vL * vL + wL * wL);
    T pLrL = pL / rL;
    T HL = eL + pLrL + keL;
    T rR = R.r, pR = R.p, eR = gm.Cv * R.temp, aR = o_sqrt(gm.gamma * gm.R * R.temp);
    T uR = R.u, vR = R.v, wR = R.w;
    T keR = 0.5 * (uR * uR + vR * vR + wR * wR);
    T pRrR = pR / rR;
    T HR = eR + pRrR + keR;
    T pLplus, uLplus;
    if (o_abs(uL) <= aL) {
        uLplus = 1.0 / (4.0 * aL) * (uL + aL) * (uL + aL);
        pLplus = pL * uLplus * (1.0 / aL * (2.0 - uL / aL));
    } else {
        uLplus = 0.5 * (uL + o_abs(uL));
        pLplus = pL * uLplus * (1.0 / uL);
    }
    T pRminus, uRminus;
    if (o_abs(uR) <= aR) {
        uRminus = -1.0 / (4.0 * aR) * (uR - aR) * (uR - aR);
        pRminus = pR * uRminus * (1.0 / aR * (-2.0 - uR / aR));
    } else {
        uRminus = 0.5 * (uR - o_abs(uR));
        pRminus = pR * uRminus * (1.0 / uR);
    }
    T p_half = pLplus + pRminus;
    F[0] = uLplus * rL + uRminus * rR;
    F[1] = uLplus * rL * uL + uRminus * rR * uR + p_half;
    F[2] = uLplus * rL * vL + uRminus * rR * vR;
    if (three_d) F[3] = uLplus * rL * wL + uRminus * rR * wR;
    F[three_d ? 4 : 3] = uLplus * rL * HL + uRminus * rR * HR;
}

template <typename T>
static void ausmdv(const FaceState<T>& L, const FaceState<T>& R, const IdealGas& gm, T* F,
                   bool three_d) {  // ausmdv.cpp:8-132
    T rL = L.r, pL = L.p, pLrL = pL / rL, uL = L.u, vL = L.v, wL = L.w;
    T eL = gm.Cv * L.temp, aL = o_sqrt(gm.gamma * gm.R * L.temp);
    T keL = 0.5 * (uL * uL + vL * vL + wL * wL);
    T HL = eL + pLrL + keL;
    T rR = R.r, pR = R.p, pRrR = pR / rR, uR = R.u, vR = R.v, wR = R.w;
    T eR = gm.Cv * R.temp, aR = o_sqrt(gm.gamma * gm.R * R.temp);
    T keR = 0.5 * (uR * uR + vR * vR + wR * wR);
    T HR = eR + pRrR + keR;
    T alphaL = 2.0 * pLrL / (pLrL + pRrR);
    T alphaR = 2.0 * pRrR / (pLrL + pRrR);
    T am = o_max(aL, aR);
    T ML = uL / am, MR = uR / am;
    T pLplus, uLplus;
    T duL = 0.5 * (uL + o_abs(uL));
    if (o_abs(ML) <= 1.0) {
        pLplus = pL * (ML + 1.0) * (ML + 1.0) * (2.0 - ML) * 0.25;
        uLplus = alphaL * ((uL + am) * (uL + am) / (4.0 * am) - duL) + duL;
    } else {
        pLplus = pL * duL / uL;
        uLplus = duL;
    }
    T pRminus, uRminus;
    T duR = 0.5 * (uR - o_abs(uR));
    if (o_abs(MR) <= 1.0) {
        pRminus = pR * (MR - 1.0) * (MR - 1.0) * (2.0 + MR) * 0.25;
        uRminus = alphaR * (-(uR - am) * (uR - am) / (4.0 * am) - duR) + duR;
    } else {
        pRminus = pR * duR / uR;
        uRminus = duR;
    }
    T ru_half = uLplus * rL + uRminus * rR;
    T p_half = pLplus + pRminus;
    T dp = pL - pR;
    const double K_SWITCH = 10.0;
    dp = K_SWITCH * o_abs(dp) / o_min(pL, pR);
    T s = 0.5 * o_min(1.0, dp);
    T ru2_AUSMV = uLplus * rL * uL + uRminus * rR * uR;
    T ru2_AUSMD = 0.5 * (ru_half * (uL + uR) - o_abs(ru_half) * (uR - uL));
    T ru2_half = (0.5 + s) * ru2_AUSMV + (0.5 - s) * ru2_AUSMD;
    const size_t ie = three_d ? 4 : 3;
    F[0] = ru_half;
    if (ru_half >= 0.0) {
        F[1] = (ru2_half + p_half);
        F[2] = (ru_half * vL);
        if (three_d) F[3] = (ru_half * wL);
        F[ie] = ru_half * HL;
    } else {
        F[1] = (ru2_half + p_half);
        F[2] = (ru_half * vR);
        if (three_d) F[3] = (ru_half * wR);
        F[ie] = ru_half * HR;
    }
    const double C_EFIX = 0.125;
    bool caseA = ((uL - aL) < 0.0) && ((uR - aR) > 0.0);
    bool caseB = ((uL + aL) < 0.0) && ((uR + aR) > 0.0);
    T d_ua = 0.0;
    if (caseA && !caseB) d_ua = C_EFIX * ((uR - aR) - (uL - aL));
    if (caseB && !caseA) d_ua = C_EFIX * ((uR + aR) - (uL + aL));
    if (d_ua != 0.0) {
        F[0] -= d_ua * (rR - rL);
        F[1] -= d_ua * (rR * uR - rL * uL);
        F[2] -= d_ua * (rR * vR - rL * vL);
        if (three_d) F[3] -= d_ua * (rR * wR - rL * wL);
        F[ie] -= d_ua * (rR * HR - rL * HL);
    }
}

template <typename T>
static void ldfss2(const FaceState<T>& L, const FaceState<T>& R, const IdealGas& gm, T* F,
                   bool three_d, double delta) {  // ldfss2.cpp:9-90
    T rL = L.r, pL = L.p, pLrL = pL / rL, uL = L.u, vL = L.v, wL = L.w;
    T eL = gm.Cv * L.temp, aL = o_sqrt(gm.gamma * gm.R * L.temp);
    T keL = 0.5 * (uL * uL + vL * vL + wL * wL);
    T HL = eL + pLrL + keL;
    T rR = R.r, pR = R.p, pRrR = pR / rR, uR = R.u, vR = R.v, wR = R.w;
    T eR = gm.Cv * R.temp, aR = o_sqrt(gm.gamma * gm.R * R.temp);
    T keR = 0.5 * (uR * uR + vR * vR + wR * wR);
    T HR = eR + pRrR + keR;
    T am = 0.5 * (aL + aR);
    T ML = uL / am, MR = uR / am;
    T MpL = 0.25 * (ML + 1.0) * (ML + 1.0);
    T MmR = -0.25 * (MR - 1.0) * (MR - 1.0);
    T alphaL = 0.5 * (1.0 + o_copysign(T(1.0), ML));
    T alphaR = 0.5 * (1.0 - o_copysign(T(1.0), MR));
    T betaL = -o_max(0.0, 1.0 - o_floor(o_abs(ML)));
    T betaR = -o_max(0.0, 1.0 - o_floor(o_abs(MR)));
    T PL = 0.25 * (ML + 1.0) * (ML + 1.0) * (2.0 - ML);
    T PR = 0.25 * (MR - 1.0) * (MR - 1.0) * (2.0 + MR);
    T DL = alphaL * (1.0 + betaL) - betaL * PL;
    T DR = alphaR * (1.0 + betaR) - betaR * PR;
    T Mhalf = 0.25 * betaL * betaR * o_pow((o_sqrt(0.5 * (ML * ML + MR * MR)) - 1.0), T(2.0));
    T MhalfL = Mhalf * (1.0 - ((pL - pR) / (pL + pR) + delta * (o_abs(pL - pR) / pL)));
    T MhalfR = Mhalf * (1.0 + ((pL - pR) / (pL + pR) - delta * (o_abs(pL - pR) / pR)));
    T CL = alphaL * (1.0 + betaL) * ML - betaL * MpL - MhalfL;
    T CR = alphaR * (1.0 + betaR) * MR - betaR * MmR + MhalfR;
    T ru_half = am * rL * CL + am * rR * CR;
    T ru2_half = am * rL * CL * uL + am * rR * CR * uR;
    T p_half = DL * pL + DR * pR;
    F[0] = ru_half;
    F[1] = ru2_half + p_half;
    F[2] = am * rL * CL * vL + am * rR * CR * vR;
    if (three_d) F[3] = am * rL * CL * wL + am * rR * CR * wR;
    F[three_d ? 4 : 3] = am * rL * CL * HL + am * rR * CR * HR;
}

template <typename T>
static void rusanov(const FaceState<T>& L, const FaceState<T>& R, const IdealGas& gm, T* F,
                    bool three_d) {  // rusanov.cpp:9-53
    T rL = L.r, eL = gm.Cv * L.temp, pL = L.p, uL = L.u, vL = L.v, wL = L.w;
    T ruL = rL * uL;
    T keL = 0.5 * (uL * uL + vL * vL + wL * wL);
    T HL = eL + pL / rL + keL;
    T aL = o_sqrt(gm.gamma * gm.R * L.temp);
    T rR = R.r, eR = gm.Cv * R.temp, pR = R.p, uR = R.u, vR = R.v, wR = R.w;
    T ruR = rR * uR;
    T keR = 0.5 * (uR * uR + vR * vR + wR * wR);
    T HR = eR + pR / rR + keR;
    T aR = o_sqrt(gm.gamma * gm.R * R.temp);
    T S = o_max(o_abs(uL - aL), o_abs(uR - aR));
    S = o_max(S, o_abs(uL + aL));
    S = o_max(S, o_abs(uR + aR));
    F[0] = 0.5 * (ruL + ruR) - 0.5 * S * (rR - rL);
    F[1] = 0.5 * (ruL * uL + pL + ruR * uR + pR) - 0.5 * S * (rR * uR - rL * uL);
    F[2] = 0.5 * (ruL * vL + ruR * vR) - 0.5 * S * (rR * vR - rL * vL);
    if (three_d) F[3] = 0.5 * (ruL * wL + ruR * wR) - 0.5 * S * (rR * wR - rL * wL);
    F[three_d ? 4 : 3] = 0.5 * (ruL * HL + ruR * HR) - 0.5 * S * (rR * HR - rL * HL);
}

// IdealGas thermo closures, gas_model.h:11-116
template <typename T>
static void thermo_update(Thermo th, const IdealGas& gm, T& rho, T& p, T& temp, T& e) {
    switch (th) {
        case Thermo::rho_p: temp = p / (rho * gm.R); e = gm.Cv * temp; break;
        case Thermo::rho_u: temp = e / gm.Cv; p = rho * gm.R * temp; break;
        case Thermo::rho_T: p = rho * gm.R * temp; e = gm.Cv * temp; break;
        case Thermo::p_T: rho = p / (gm.R * temp); e = gm.Cv * temp; break;
    }
}

template <typename T>
void FiniteVolume<T>::convective_flux(const FlowStates<T>& fs, const Grid<T>& g,
                                      const IdealGas& gm, bool allow_reconstruction) {
    // convective_flux.cpp:84-178
    const size_t N = g.N;
    const int order = allow_reconstruction ? cfg.order : 1;
    if (order == 2) {
        // compute_convective_gradient, convective_flux.cpp:180-209
        switch (cfg.thermo) {
            case Thermo::rho_p: lsq_gradient(g, fs.p, g_p); lsq_gradient(g, fs.rho, g_rho); break;
            case Thermo::rho_u: lsq_gradient(g, fs.rho, g_rho); lsq_gradient(g, fs.e, g_u); break;
            case Thermo::rho_T: lsq_gradient(g, fs.rho, g_rho); lsq_gradient(g, fs.temp, g_temp); break;
            case Thermo::p_T: lsq_gradient(g, fs.p, g_p); lsq_gradient(g, fs.temp, g_temp); break;
        }
        lsq_gradient(g, fs.vx, g_vx);
        lsq_gradient(g, fs.vy, g_vy);
        if (dim == 3) lsq_gradient(g, fs.vz, g_vz);
        // compute_limiters, convective_flux.cpp:422-462
        if (cfg.limiter_enabled) {
            BranchCode* br = record_branches ? branches.data() : nullptr;
            double eps = cfg.epsilon;
            switch (cfg.thermo) {
                case Thermo::rho_p:
                    barth_jespersen(g, fs.p, g_p, eps, l_p, br, 5, 0);
                    barth_jespersen(g, fs.rho, g_rho, eps, l_rho, br, 5, 1);
                    break;
                case Thermo::rho_u:
                    barth_jespersen(g, fs.rho, g_rho, eps, l_rho, br, 5, 0);
                    barth_jespersen(g, fs.e, g_u, eps, l_u, br, 5, 1);
                    break;
                case Thermo::rho_T:
                    barth_jespersen(g, fs.rho, g_rho, eps, l_rho, br, 5, 0);
                    barth_jespersen(g, fs.temp, g_temp, eps, l_temp, br, 5, 1);
                    break;
                case Thermo::p_T:
                    barth_jespersen(g, fs.p, g_p, eps, l_p, br, 5, 0);
                    barth_jespersen(g, fs.temp, g_temp, eps, l_temp, br, 5, 1);
                    break;
            }
            barth_jespersen(g, fs.vx, g_vx, eps, l_vx, br, 5, 2);
            barth_jespersen(g, fs.vy, g_vy, eps, l_vy, br, 5, 3);
            barth_jespersen(g, fs.vz, g_vz, eps, l_vz, br, 5, 4);
        }
    }

    const bool lim = cfg.limiter_enabled;
    const bool three_d = dim == 3;
#pragma omp parallel for schedule(static)
    for (long long fi = 0; fi < (long long)g.F; fi++) {
        size_t f = (size_t)fi;
        FaceState<T> S[2];
        size_t cells[2] = {g.left[f], g.right[f]};
        for (int side = 0; side < 2; side++) {
            size_t c = cells[side];
            T rho, p, temp, e, vx, vy, vz;
            if (order == 1) {  // copy_reconstruct, convective_flux.cpp:211-240
                rho = fs.rho[c]; p = fs.p[c]; temp = fs.temp[c]; e = fs.e[c];
                vx = fs.vx[c]; vy = fs.vy[c]; vz = fs.vz[c];
            } else {  // linear_reconstruct, convective_flux.cpp:257-420
                bool valid = c < N;
                bool limit = lim && valid;
                T dx = g.cx[f] - g.ccx[c], dy = g.cy[f] - g.ccy[c], dz = g.cz[f] - g.ccz[c];
                T one = 1.0;
                auto L = [&](const std::vector<T>& l) { return limit ? l[c] : one; };
                static const std::array<T, 3> zero3 = {T(0.0), T(0.0), T(0.0)};
                auto G = [&](const std::vector<std::array<T, 3>>& gr) -> const std::array<T, 3>& {
                    return valid ? gr[c] : zero3;
                };
                rho = fs.rho[c]; p = fs.p[c]; temp = fs.temp[c]; e = fs.e[c];
                switch (cfg.thermo) {
                    case Thermo::rho_p:
                        p = lin_interp(fs.p[c], G(g_p), dx, dy, dz, L(l_p), valid);
                        rho = lin_interp(fs.rho[c], G(g_rho), dx, dy, dz, L(l_rho), valid);
                        break;
                    case Thermo::rho_u:
                        rho = lin_interp(fs.rho[c], G(g_rho), dx, dy, dz, L(l_rho), valid);
                        e = lin_interp(fs.e[c], G(g_u), dx, dy, dz, L(l_u), valid);
                        break;
                    case Thermo::rho_T:
                        rho = lin_interp(fs.rho[c], G(g_rho), dx, dy, dz, L(l_rho), valid);
                        temp = lin_interp(fs.temp[c], G(g_temp), dx, dy, dz, L(l_temp), valid);
                        break;
                    case Thermo::p_T:
                        p = lin_interp(fs.p[c], G(g_p), dx, dy, dz, L(l_p), valid);
                        temp = lin_interp(fs.temp[c], G(g_temp), dx, dy, dz, L(l_temp), valid);
                        break;
                }
                thermo_update(cfg.thermo, gm, rho, p, temp, e);
                vx = lin_interp(fs.vx[c], G(g_vx), dx, dy, dz, L(l_vx), valid);
                vy = lin_interp(fs.vy[c], G(g_vy), dx, dy, dz, L(l_vy), valid);
                vz = lin_interp(fs.vz[c], G(g_vz), dx, dy, dz, L(l_vz), valid);
            }
            FlowStates<T>& dst = side == 0 ? left : right;
            dst.rho[f] = rho; dst.p[f] = p; dst.temp[f] = temp; dst.e[f] = e;
            dst.vx[f] = vx; dst.vy[f] = vy; dst.vz[f] = vz;
            // transform_to_local_frame, vector3.cpp:141-153
            S[side].r = rho; S[side].p = p; S[side].temp = temp;
            S[side].u = vx * g.nx[f] + vy * g.ny[f] + vz * g.nz[f];
            S[side].v = vx * g.t1x[f] + vy * g.t1y[f] + vz * g.t1z[f];
            S[side].w = vx * g.t2x[f] + vy * g.t2y[f] + vz * g.t2z[f];
        }
        T Fl[5] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
        switch (cfg.flux) {
            case FluxKind::Hanel: hanel(S[0], S[1], gm, Fl, three_d); break;
            case FluxKind::Ausmdv: ausmdv(S[0], S[1], gm, Fl, three_d); break;
            case FluxKind::Ldfss2: ldfss2(S[0], S[1], gm, Fl, three_d, cfg.ldfss_delta); break;
            case FluxKind::Rusanov: rusanov(S[0], S[1], gm, Fl, three_d); break;
        }
        // transform_to_global, convective_flux.cpp:145-177
        T px = Fl[1], py = Fl[2], pz = 0.0;
        if (three_d) pz = Fl[3];
        T x = px * g.nx[f] + py * g.t1x[f] + pz * g.t2x[f];
        T y = px * g.ny[f] + py * g.t1y[f] + pz * g.t2y[f];
        T z = px * g.nz[f] + py * g.t1z[f] + pz * g.t2z[f];
        flux.mass(f) = Fl[0];
        flux.mx(f) = x;
        flux.my(f) = y;
        if (three_d) flux.mz(f) = z;
        flux.energy(f) = Fl[three_d ? 4 : 3];
    }
}

template <typename T>
static T sutherland(const Transport& tp, T temp) {  // transport_properties.h:28-42
    return tp.mu0 * o_pow(temp / tp.T0, T(3.0 / 2.0)) * (T(tp.T0) + T(tp.Ts)) / (temp + tp.Ts);
}

template <typename T>
void FiniteVolume<T>::viscous_flux(const FlowStates<T>& fs, const Grid<T>& g,
                                   const IdealGas& gm, const Transport& tp) {
    // compute_viscous_gradient, viscous_flux.cpp:169-178
    lsq_gradient(g, fs.temp, g_temp);
    lsq_gradient(g, fs.vx, g_vx);
    lsq_gradient(g, fs.vy, g_vy);
    lsq_gradient(g, fs.vz, g_vz);
    const size_t N = g.N;
    // compute_viscous_flux, viscous_flux.cpp:180-232
#pragma omp parallel for schedule(static)
    for (long long fi = 0; fi < (long long)g.F; fi++) {
        size_t f = (size_t)fi;
        size_t l = g.left[f], r = g.right[f];
        bool lv = l < N, rv = r < N;
        std::array<T, 3> gT, gx, gy, gz;
        if (!lv || !rv) {  // copy_gradients_to_face, viscous_flux.cpp:63-82
            size_t in = lv ? l : r;
            gT = g_temp[in]; gx = g_vx[in]; gy = g_vy[in]; gz = g_vz[in];
        } else {  // hasselbacher_average, viscous_flux.cpp:84-128
            T ex = g.ccx[r] - g.ccx[l], ey = g.ccy[r] - g.ccy[l], ez = g.ccz[r] - g.ccz[l];
            T len_e = o_sqrt(ex * ex + ey * ey + ez * ez);
            T ehx = ex / len_e, ehy = ey / len_e, ehz = ez / len_e;
            T nxf = g.nx[f], nyf = g.ny[f], nzf = g.nz[f];
            T edn = ehx * nxf + ehy * nyf + ehz * nzf;
            auto avg = [&](const std::vector<std::array<T, 3>>& gr, T vl, T vr) {
                T ax = 0.5 * (gr[l][0] + gr[r][0]);
                T ay = 0.5 * (gr[l][1] + gr[r][1]);
                T az = 0.5 * (gr[l][2] + gr[r][2]);
                T ade = ax * ehx + ay * ehy + az * ehz;
                T corr = ade - (vr - vl) / len_e;
                return std::array<T, 3>{ax - corr * nxf / edn, ay - corr * nyf / edn,
                                        az - corr * nzf / edn};
            };
            gx = avg(g_vx, fs.vx[l], fs.vx[r]);
            gy = avg(g_vy, fs.vy[l], fs.vy[r]);
            gz = avg(g_vz, fs.vz[l], fs.vz[r]);
            gT = avg(g_temp, fs.temp[l], fs.temp[r]);
        }
        // average_flow_states_pT + update_thermo_from_pT (flow_state.h:88-91, gas_state.h:219-225)
        T p = 0.5 * (fs.p[l] + fs.p[r]);
        T temp = 0.5 * (fs.temp[l] + fs.temp[r]);
        T rho = p / (gm.R * temp);
        T e = gm.Cv * temp;
        T vx = 0.5 * (fs.vx[l] + fs.vx[r]);
        T vy = 0.5 * (fs.vy[l] + fs.vy[r]);
        T vz = 0.5 * (fs.vz[l] + fs.vz[r]);
        face_fs.rho[f] = rho; face_fs.p[f] = p; face_fs.temp[f] = temp; face_fs.e[f] = e;
        face_fs.vx[f] = vx; face_fs.vy[f] = vy; face_fs.vz[f] = vz;
        T mu = sutherland(tp, temp);
        T k = gm.Cp * mu / tp.Pr;
        T lambda = -2.0 / 3.0 * mu;
        T bulk = lambda * (gx[0] + gy[1] + gz[2]);
        T txx = 2.0 * mu * gx[0] + bulk;
        T tyy = 2.0 * mu * gy[1] + bulk;
        T tzz = 2.0 * mu * gz[2] + bulk;
        T txy = mu * (gx[1] + gy[0]);
        T txz = mu * (gx[2] + gz[0]);
        T tyz = mu * (gy[2] + gz[1]);
        T thx = vx * txx + vy * txy + vz * txz + k * gT[0];
        T thy = vx * txy + vy * tyy + vz * tyz + k * gT[1];
        T thz = vx * txz + vy * tyz + vz * tzz + k * gT[2];
        T nxf = g.nx[f], nyf = g.ny[f], nzf = g.nz[f];
        flux.mx(f) -= nxf * txx + nyf * txy + nzf * txz;
        flux.my(f) -= nxf * txy + nyf * tyy + nzf * tyz;
        if (dim == 3) flux.mz(f) -= nxf * txz + nyf * tyz + nzf * tzz;
        flux.energy(f) -= nxf * thx + nyf * thy + nzf * thz;
    }
}

template <typename T>
void FiniteVolume<T>::surface_integral(const Grid<T>& g, Conserved<T>& dudt) {
    // flux_surface_integral, finite_volume.cpp:220-255
    const bool three_d = dim == 3;
#pragma omp parallel for schedule(static)
    for (long long ci = 0; ci < (long long)g.N; ci++) {
        size_t c = (size_t)ci;
        T dm = 0.0, dx = 0.0, dy = 0.0, dz = 0.0, de = 0.0;
        for (size_t k = 0; k < g.cell_faces[c].size(); k++) {
            size_t f = g.cell_faces[c][k];
            T a = -g.area[f] * (double)g.outsigns[c][k];
            dm += flux.mass(f) * a;
            dx += flux.mx(f) * a;
            dy += flux.my(f) * a;
            if (three_d) dz += flux.mz(f) * a;
            de += flux.energy(f) * a;
        }
        dudt.mass(c) = dm / g.volume[c];
        dudt.mx(c) = dx / g.volume[c];
        dudt.my(c) = dy / g.volume[c];
        if (three_d) dudt.mz(c) = dz / g.volume[c];
        dudt.energy(c) = de / g.volume[c];
    }
}

template <typename T>
void FiniteVolume<T>::compute_dudt(FlowStates<T>& fs, const Grid<T>& g, Conserved<T>& dudt,
                                   const IdealGas& gm, const Transport& tp,
                                   bool allow_reconstruction) {
    // finite_volume.cpp:56-85
    for (size_t i = 0; i < bcs.size(); i++) apply_ghost_actions(bcs[i].pre_reconstruction, fs, g, bc_faces[i], gm);
    convective_flux(fs, g, gm, allow_reconstruction);
    // apply_post_convective_flux_bc: ConstantFlux, boundary.cpp:404-444 (vy*n.x quirk kept)
    for (size_t i = 0; i < bcs.size(); i++) {
        for (const Action& a : bcs[i].post_convective_flux) {
            if (a.kind != ActionKind::ConstantFlux) continue;
            for (size_t f : bc_faces[i]) {
                T nxf = g.nx[f], nyf = g.ny[f], nzf = g.nz[f];
                const T fvx = fs_value<T>(a, 4), fvy = fs_value<T>(a, 5), fvz = fs_value<T>(a, 6);
                T u = gm.Cv * fs_value<T>(a, 0);
                T rvx = fvx - 0.0, rvy = fvy - 0.0, rvz = fvz - 0.0;
                T mass = fs_value<T>(a, 2) * (rvx * nxf + rvy * nyf + rvz * nzf);
                T p = fs_value<T>(a, 1);
                flux.mass(f) = mass;
                flux.mx(f) = p * nxf + fvx * mass;
                flux.my(f) = p * nyf + fvy * mass;
                if (dim == 3) flux.mz(f) = p * nzf + fvz * mass;
                flux.energy(f) = mass * (u + 0.5 * (fvx * fvx + fvy * fvy + fvz * fvz)) +
                                 p * (fvx * nxf + fvy * nxf + fvz * nzf);
            }
        }
    }
    if (cfg.viscous) {
        for (size_t i = 0; i < bcs.size(); i++) apply_ghost_actions(bcs[i].pre_viscous_grad, fs, g, bc_faces[i], gm);
        viscous_flux(fs, g, gm, tp);
    }
    surface_integral(g, dudt);
}

template <typename T>
double FiniteVolume<T>::estimate_dt(const FlowStates<T>& fs, const Grid<T>& g,
                                    const IdealGas& gm, const Transport& tp) {
    // finite_volume.cpp:130-184
    double dt = std::numeric_limits<double>::max();
    const bool visc = cfg.viscous;
    const double sf = cfg.signal_factor;
#pragma omp parallel for reduction(min : dt) schedule(static)
    for (long long ci = 0; ci < (long long)g.N; ci++) {
        size_t c = (size_t)ci;
        T vx = fs.vx[c], vy = fs.vy[c], vz = fs.vz[c];
        T src = 0.0, srv = 0.0;
        T vol = g.volume[c];
        for (size_t f : g.cell_faces[c]) {
            T a = g.area[f];
            T dot = vx * g.nx[f] + vy * g.ny[f] + vz * g.nz[f];
            T sig = o_abs(dot) + o_sqrt(gm.gamma * gm.R * fs.temp[c]);
            src += sig * a;
            if (visc) {
                T gamma = gm.gamma;
                T mu = sutherland(tp, face_fs.temp[f]);
                T k = gm.Cp * sutherland(tp, face_fs.temp[f]) / tp.Pr;
                T rho = face_fs.rho[f];
                T Pr = mu * gm.Cp / k;
                T tmp = (gamma / rho) * (mu / Pr) * a * a;
                srv += tmp / vol;
            }
        }
        T local = vol / (src + sf * srv);
        double l = real_part(local);
        dt = (l < dt) ? l : dt;
    }
    return dt;
}

template <typename T>
size_t FiniteVolume<T>::count_bad_cells(const FlowStates<T>& fs, size_t n) {
    size_t bad = 0;  // finite_volume.cpp:257-270
    for (size_t i = 0; i < n; i++) {
        if (fs.temp[i] < 0.0 || fs.rho[i] < 0.0 || o_isnan(fs.rho[i]) || o_isinf(fs.rho[i])) bad++;
    }
    return bad;
}

template <typename T>
void conserved_to_primatives(const Conserved<T>& cq, FlowStates<T>& fs, const IdealGas& gm) {
    // primative_conserved_conversion.cpp:4-23
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)fs.size(); ii++) {
        size_t i = (size_t)ii;
        T rho = cq.mass(i);
        T vx = cq.mx(i) / rho;
        T vy = cq.my(i) / rho;
        T vz = (cq.dim == 3) ? cq.mz(i) / rho : T(0.0);
        T ke = 0.5 * (vx * vx + vy * vy + vz * vz);
        T u = cq.energy(i) / rho - ke;
        fs.rho[i] = rho; fs.vx[i] = vx; fs.vy[i] = vy; fs.vz[i] = vz; fs.e[i] = u;
        fs.temp[i] = u / gm.Cv;
        fs.p[i] = rho * gm.R * fs.temp[i];
    }
}

template <typename T>
void primatives_to_conserved(Conserved<T>& cq, const FlowStates<T>& fs) {
    // primative_conserved_conversion.cpp:31-51
    for (size_t i = 0; i < fs.size(); i++) {
        T vx = fs.vx[i], vy = fs.vy[i], vz = fs.vz[i], rho = fs.rho[i];
        cq.mass(i) = fs.rho[i];
        cq.mx(i) = rho * vx;
        cq.my(i) = rho * vy;
        if (cq.dim == 3) cq.mz(i) = rho * vz;
        T ke = 0.5 * (vx * vx + vy * vy + vz * vz);
        cq.energy(i) = rho * (ke + fs.e[i]);
    }
}

template <typename T>
Norms l2_norms(const Conserved<T>& cq) {  // conserved_quantities.cpp:40-69
    Norms n;
    for (size_t i = 0; i < cq.n; i++) {
        double m = real_part(cq.mass(i)), x = real_part(cq.mx(i)), y = real_part(cq.my(i));
        double z = cq.dim == 3 ? real_part(cq.mz(i)) : 0.0, e = real_part(cq.energy(i));
        n.mass += m * m; n.mx += x * x; n.my += y * y; n.mz += z * z; n.energy += e * e;
        n.global += m * m + x * x + y * y + z * z + e * e;
    }
    n.global = std::sqrt(n.global); n.mass = std::sqrt(n.mass); n.mx = std::sqrt(n.mx);
    n.my = std::sqrt(n.my); n.mz = std::sqrt(n.mz); n.energy = std::sqrt(n.energy);
    return n;
}

// apply_time_derivative(U0, U1, dUdt, dt), conserved_quantities.cpp:79-94
template <typename T>
static void axpy_into(const Conserved<T>& U0, Conserved<T>& U1, const Conserved<T>& k, double dt) {
    for (size_t i = 0; i < U0.q.size(); i++) U1.q[i] = U0.q[i] + k.q[i] * dt;
}
// ConservedQuantities::apply_time_derivative, conserved_quantities.cpp:25-38
template <typename T>
static void axpy_inplace(Conserved<T>& U, const Conserved<T>& k, double dt) {
    for (size_t i = 0; i < U.q.size(); i++) U.q[i] += k.q[i] * dt;
}

// ======================= configuration ======================================

FvConfig parse_fv_config(const Json& config) {
    FvConfig c;  // finite_volume.cpp:13-54, convective_flux.cpp:60-82, flux_calc.cpp:8-23
    const Json& cf = config.at("convective_flux");
    std::string ft = cf.at("flux_calculator").at("type").as_string();
    if (ft == "hanel") c.flux = FluxKind::Hanel;
    else if (ft == "ausmdv") c.flux = FluxKind::Ausmdv;
    else if (ft == "ldfss2") { c.flux = FluxKind::Ldfss2; c.ldfss_delta = cf.at("flux_calculator").at("delta").as_double(); }
    else if (ft == "rusanov") c.flux = FluxKind::Rusanov;
    else throw std::runtime_error("Unknown flux calculator " + ft);
    c.order = (int)cf.at("reconstruction_order").as_int();
    if (c.order > 1) {
        std::string th = cf.at("thermo_interpolator").as_string();
        if (th == "rho_p") c.thermo = Thermo::rho_p;
        else if (th == "rho_T") c.thermo = Thermo::rho_T;
        else if (th == "rho_u") c.thermo = Thermo::rho_u;
        else if (th == "p_T") c.thermo = Thermo::p_T;
        else throw std::runtime_error("Unknown thermo interpolator " + th);
        std::string lt = cf.at("limiter").at("type").as_string();
        if (lt == "barth_jespersen") { c.limiter_enabled = true; c.epsilon = cf.at("limiter").at("epsilon").as_double(); }
        else if (lt == "unlimited") c.limiter_enabled = false;
        else throw std::runtime_error("Unknown limiter " + lt);
    } else if (c.order != 1) {
        throw std::runtime_error("Invalid reconstruction order");
    }
    const Json& vf = config.at("viscous_flux");
    c.viscous = vf.at("enabled").as_bool();
    c.signal_factor = vf.at("signal_factor").as_double();
    return c;
}

void CubicSpline::fit(const std::vector<double>& xs, const std::vector<double>& ys) {
    const size_t n = xs.size();
    if (n < 4) throw std::runtime_error("Insufficient points for cubic spline");
    if (ys.size() != n) throw std::runtime_error("Cubic spline has different number of x and y points");
    x = xs;
    y = ys;
    const size_t ne = n - 2;  // one equation per interior knot
    std::vector<double> diag(ne, 0.0), upper(ne, 0.0), rhs(ne, 0.0);
    for (size_t i = 0; i <= ne; i++) {
        double dx = x[i + 1] - x[i];
        double dy = y[i + 1] - y[i];
        if (i != ne) {
            diag[i] += dx;
            rhs[i] -= dy / dx;
        }
        if (i == 0) continue;
        rhs[i - 1] += dy / dx;
        diag[i - 1] += dx;
        if (i - 1 < ne - 1) upper[i - 1] += dx;
    }
    for (size_t i = 0; i < ne; i++) {
        rhs[i] *= 6;
        diag[i] *= 2;
    }
    for (size_t i = 1; i < ne; i++) {
        double w = upper[i - 1] / diag[i - 1];
        diag[i] = diag[i] - w * upper[i - 1];
        rhs[i] = rhs[i] - w * rhs[i - 1];
    }
    m.assign(n, 0.0);
    m[n - 2] = rhs[ne - 1] / diag[ne - 1];
    for (long i = (long)ne - 2; i >= 0; i--) m[i + 1] = (rhs[i] - upper[i] * m[i + 2]) / diag[i];
}

double CubicSpline::eval(double t) const {
    if (t <= x.front()) return y.front();
    if (t >= x.back()) return y.back();
    size_t idx = 0;
    for (size_t i = 0; i < x.size(); i++) {
        if (x[i] >= t) {
            idx = i - 1;
            break;
        }
    }
    double dp = x[idx + 1] - t;
    double dm = t - x[idx];
    double dxi = x[idx + 1] - x[idx];
    double a = (m[idx] * dp * dp * dp + m[idx + 1] * dm * dm * dm) / (6 * dxi);
    double b = (y[idx] / dxi - m[idx] * dxi / 6) * dp;
    double c = (y[idx + 1] / dxi - m[idx + 1] * dxi / 6) * dm;
    return a + b + c;
}

static Action parse_action(const Json& a) {  // boundary.cpp:448-492
    Action out;
    std::string t = a.at("type").as_string();
    auto read_fs = [&](const Json& fs) {
        out.fs[0] = fs.at("T").as_double(); out.fs[1] = fs.at("p").as_double();
        out.fs[2] = fs.at("rho").as_double(); out.fs[3] = fs.at("energy").as_double();
        out.fs[4] = fs.at("vx").as_double(); out.fs[5] = fs.at("vy").as_double();
        out.fs[6] = fs.at("vz").as_double();
    };
    if (t == "flow_state_copy") { out.kind = ActionKind::FlowStateCopy; read_fs(a.at("flow_state")); }
    else if (t == "internal_copy") out.kind = ActionKind::InternalCopy;
    else if (t == "internal_copy_reflect_normal") out.kind = ActionKind::InternalCopyReflectNormal;
    else if (t == "internal_vel_copy_reflect") out.kind = ActionKind::InternalVelCopyReflect;
    else if (t == "fix_temperature") { out.kind = ActionKind::FixTemperature; out.value = a.at("temperature").as_double(); }
    else if (t == "subsonic_inflow") { out.kind = ActionKind::SubsonicInflow; read_fs(a.at("flow_state")); }
    else if (t == "subsonic_outflow") { out.kind = ActionKind::SubsonicOutflow; out.value = a.at("pressure").as_double(); }
    else if (t == "constant_flux") { out.kind = ActionKind::ConstantFlux; read_fs(a.at("flow_state")); }
    else if (t == "periodic_copy") out.kind = ActionKind::PeriodicCopy;
    else if (t == "boundary_layer_profile") {  // BoundaryLayerProfile ctor, boundary.cpp:48-57
        out.kind = ActionKind::BoundaryLayerProfile;
        const Json& pr = a.at("profile");
        std::vector<double> h = pr.at("height").as_doubles();
        out.spline_v.fit(h, pr.at("v").as_doubles());
        out.spline_T.fit(h, pr.at("T").as_doubles());
        out.value = pr.at("p").as_double();
    }
    else throw std::runtime_error("Unknown boundary action " + t);
    return out;
}

template <typename T>
std::unique_ptr<Sim<T>> build_sim(const Json& config, const GridIO& io) {
    auto sim = std::make_unique<Sim<T>>();
    const Json& grid_cfg = config.at("grid");
    const Json& bnds = grid_cfg.at("boundaries");
    std::map<std::string, PeriodicLink> periodic;
    for (const auto& [tag, bc] : bnds.items()) {
        for (const Json& a : bc.at("pre_reconstruction").elements()) {
            if (a.at("type").as_string() == "periodic_copy") {
                PeriodicLink l;
                l.partner = a.at("partner").as_string();
                auto off = a.at("offset").as_doubles();
                for (int d = 0; d < 3; d++) l.offset[d] = off[d];
                periodic[tag] = l;
            }
        }
    }
    sim->grid.init(io, bnds, periodic);
    FvConfig fc = parse_fv_config(config);
    if (fc.viscous || fc.order > 1) sim->grid.compute_gradient_weights();
    std::vector<BoundaryCondition> bcs;
    for (const auto& tag : sim->grid.boundary_tags) {
        const Json& b = bnds.at(tag);
        BoundaryCondition bc;
        for (const Json& a : b.at("pre_reconstruction").elements()) bc.pre_reconstruction.push_back(parse_action(a));
        for (const Json& a : b.at("post_convective_flux").elements()) bc.post_convective_flux.push_back(parse_action(a));
        for (const Json& a : b.at("pre_viscous_grad").elements()) bc.pre_viscous_grad.push_back(parse_action(a));
        bcs.push_back(bc);
    }
    sim->fv.setup(sim->grid, fc, bcs);
    const Json& gm = config.at("gas_model");  // gas_model.h:58-62
    sim->gas.R = gm.at("R").as_double(); sim->gas.Cv = gm.at("Cv").as_double();
    sim->gas.Cp = gm.at("Cp").as_double(); sim->gas.gamma = gm.at("gamma").as_double();
    if (config.contains("transport_properties")) {  // transport_properties.h:91-109
        const Json& tpc = config.at("transport_properties");
        sim->tp.mu0 = tpc.at("viscosity").at("mu_0").as_double();
        sim->tp.T0 = tpc.at("viscosity").at("T_0").as_double();
        sim->tp.Ts = tpc.at("viscosity").at("T_s").as_double();
        sim->tp.Pr = tpc.at("thermal_conductivity").at("Pr").as_double();
    }
    size_t NT = sim->grid.N + sim->grid.G;
    sim->fs = FlowStates<T>(NT);
    sim->U = Conserved<T>(NT, sim->grid.dim);
    return sim;
}

template <typename T>
void Sim<T>::init_rk(const Json& sc) {  // runge_kutta.cpp:21-80
    const Json& bt = sc.at("butcher_tableau");
    rk.tab.a.clear();
    for (const Json& row : bt.at("a").elements()) rk.tab.a.push_back(row.as_doubles());
    rk.tab.b = bt.at("b").as_doubles();
    rk.tab.c = bt.at("c").as_doubles();
    const Json& cfl = sc.at("cfl");
    std::string ct = cfl.at("type").as_string();
    if (ct == "constant") rk.cfl = cfl.at("value").as_double();
    else if (ct == "linear_interpolate") { rk.cfl_times = cfl.at("times").as_doubles(); rk.cfl_values = cfl.at("cfls").as_doubles(); }
    else throw std::runtime_error("unsupported cfl schedule for runge_kutta: " + ct);
    rk.max_time = sc.at("max_time").as_double();
    rk.plot_frequency = sc.at("plot_frequency").as_double();
    rk.dt_init = sc.at("dt_init").as_double();
    rk.aliased_stages = sc.contains("stage_derivatives") && sc.at("stage_derivatives").as_string() == "aliased";
    size_t NT = grid.N + grid.G;
    k.assign(rk.tab.stages(), Conserved<T>(NT, grid.dim));
    k_tmp = Conserved<T>(NT, grid.dim);
    fs_tmp = FlowStates<T>(NT);
}

template <typename T>
double Sim<T>::cfl_eval(double t) const {  // cfl.cpp:94-127
    if (rk.cfl_times.empty()) return rk.cfl;
    const auto& ts = rk.cfl_times;
    const auto& cs = rk.cfl_values;
    if (t <= ts[0]) return cs[0];
    size_t n = ts.size();
    if (t >= ts[n - 1]) return cs[n - 1];
    for (size_t i = 0; i + 1 < n; i++) {
        if (t >= ts[i] && t < ts[i + 1]) {
            double frac = (t - ts[i]) / (ts[i + 1] - ts[i]);
            return cs[i] + frac * (cs[i + 1] - cs[i]);
        }
    }
    throw std::runtime_error("Shouldn't reach here");
}

template <typename T>
void Sim<T>::rk_initialise() {  // runge_kutta.cpp:82-104
    primatives_to_conserved(U, fs);
    rk.dt = (rk.dt_init > 0) ? rk.dt_init : std::numeric_limits<double>::max();
    rk.t = 0.0;
    rk.time_since_last_plot = 0.0;
    fv.compute_dudt(fs, grid, k[0], gas, tp);
}

template <typename T>
void Sim<T>::rk_estimate_dt() {  // runge_kutta.cpp:108-119
    rk.stable_dt = fv.estimate_dt(fs, grid, gas, tp);
    double dt_startup = std::min(cfl_eval(rk.t) * rk.stable_dt, 1.5 * rk.dt);
    rk.dt = std::min(dt_startup, rk.max_time - rk.t);
    if (rk.plot_frequency > 0.0 && rk.time_since_last_plot < rk.plot_frequency) {
        rk.dt = std::min(rk.dt, rk.plot_frequency - rk.time_since_last_plot);
    }
}

template <typename T>
void Sim<T>::rk_take_step() {  // runge_kutta.cpp:131-203
    auto K = [&](size_t i) -> Conserved<T>& { return k[rk.aliased_stages ? 0 : i]; };
    fv.compute_dudt(fs, grid, K(0), gas, tp);
    rk_estimate_dt();
    double dt = rk.dt;
    for (size_t i = 1; i < rk.tab.stages(); i++) {
        axpy_into(U, k_tmp, K(0), rk.tab.A(i, 0) * dt);
        for (size_t j = 1; j < i; j++) {
            if (rk.tab.A(i, j) < 1e-14) continue;
            axpy_inplace(k_tmp, K(j), rk.tab.A(i, j) * dt);
        }
        conserved_to_primatives(k_tmp, fs_tmp, gas);
        fv.compute_dudt(fs_tmp, grid, K(i), gas, tp);
    }
    for (size_t i = 0; i < rk.tab.stages(); i++) axpy_inplace(U, K(i), rk.tab.b[i] * dt);
    conserved_to_primatives(U, fs, gas);
    rk.t += dt;
    rk.time_since_last_plot += dt;
}

// ======================= GMRES / JFNK =======================================

static double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
}

// apply_rotations_to_hessenberg_, gmres.cpp:22-74 (dense (m+1)x(m+1) host matrices)
struct Hess {
    size_t m;
    std::vector<double> H0, H1, Q0, Q1, Om, g0, g1, hr;
    explicit Hess(size_t m_) : m(m_) {
        size_t n = m + 1;
        H0.assign(n * m, 0.0); H1 = H0;
        Q0.assign(n * n, 0.0); Q1 = Q0; Om = Q0;
        g0.assign(n, 0.0); g1 = g0; hr = g0;
        for (size_t i = 0; i < n; i++) { Q0[i * n + i] = 1; Q1[i * n + i] = 1; Om[i * n + i] = 1; }
    }
    double& H(size_t i, size_t j) { return H0[i * m + j]; }
    double& Q(std::vector<double>& A, size_t i, size_t j) { return A[i * (m + 1) + j]; }
    void rotate(size_t j) {
        size_t n = m + 1;
        if (j != 0) {
            for (size_t r = 0; r < j + 1; r++) {
                double d = 0.0;
                for (size_t c = 0; c < j + 1; c++) d += Q0[r * n + c] * H0[c * m + j];
                hr[r] = d;
            }
            for (size_t r = 0; r < j + 1; r++) H0[r * m + j] = hr[r];
        }
        for (size_t i = 0; i < n * n; i++) Om[i] = 0.0;
        for (size_t i = 0; i < n; i++) Om[i * n + i] = 1.0;
        double denom = std::sqrt(H(j, j) * H(j, j) + H(j + 1, j) * H(j + 1, j));
        double si = H(j + 1, j) / denom;
        double ci = H(j, j) / denom;
        Om[j * n + j] = ci; Om[j * n + j + 1] = si; Om[(j + 1) * n + j] = -si; Om[(j + 1) * n + j + 1] = ci;
        size_t k = j + 2;  // sub-matrices of size (j+2)x(j+2)
        // H_new = Omega_sub * H_old  (columns limited to j+2 but H has m columns)
        for (size_t r = 0; r < k; r++) {
            for (size_t c = 0; c < std::min(k, m); c++) {
                double d = 0.0;
                for (size_t i = 0; i < k; i++) d += Om[r * n + i] * H0[i * m + c];
                H1[r * m + c] = d;
            }
        }
        for (size_t r = 0; r < k; r++) {
            double d = 0.0;
            for (size_t i = 0; i < k; i++) d += Om[r * n + i] * g0[i];
            g1[r] = d;
        }
        if (j == 0) {
            for (size_t r = 0; r < k; r++) for (size_t c = 0; c < k; c++) Q1[r * n + c] = Om[r * n + c];
        } else {
            for (size_t r = 0; r < k; r++) {
                for (size_t c = 0; c < k; c++) {
                    double d = 0.0;
                    for (size_t i = 0; i < k; i++) d += Om[r * n + i] * Q0[i * n + c];
                    Q1[r * n + c] = d;
                }
            }
        }
        for (size_t r = 0; r < k; r++) g0[r] = g1[r];
        for (size_t r = 0; r < k; r++) for (size_t c = 0; c < k; c++) Q0[r * n + c] = Q1[r * n + c];
        for (size_t r = 0; r < k; r++) for (size_t c = 0; c < std::min(k, m); c++) H0[r * m + c] = H1[r * m + c];
    }
};

static void finish_solution(Hess& hs, size_t nv, const std::vector<std::vector<double>>& V,
                            std::vector<double>& x) {
    // upper_triangular_solve + gemv + add_scaled_vector, gmres.cpp:170-179
    int n = (int)nv;
    std::vector<double> y(n, 0.0);
    y[n - 1] = hs.g0[n - 1] / hs.H(n - 1, n - 1);
    for (int i = n - 2; i >= 0; i--) {
        double s = hs.g0[i];
        for (int j = i + 1; j < n; j++) s -= hs.H(i, j) * y[j];
        y[i] = s / hs.H(i, i);
    }
    for (size_t r = 0; r < x.size(); r++) {
        double d = 0.0;
        for (int c = 0; c < n; c++) d += V[c][r] * y[c];
        x[r] += d * 1.0;
    }
}

GmresResult gmres_solve(const MatVec& A, const std::vector<double>& rhs, std::vector<double>& x,
                        size_t max_iters_cfg, double tol) {
    size_t nvars = rhs.size();
    size_t m = std::min(nvars, max_iters_cfg);
    Hess hs(m);
    std::vector<double> w(nvars), r0(nvars), v(nvars);
    A(x, w);  // compute_r0_, gmres.cpp:11-20
    for (size_t i = 0; i < nvars; i++) r0[i] = rhs[i] - w[i];
    double beta = std::sqrt(dot(r0, r0));
    if (beta < tol) return {true, 0, tol, beta};
    hs.g0[0] = beta;
    for (size_t i = 0; i < nvars; i++) v[i] = r0[i] * (1.0 / beta);
    std::vector<std::vector<double>> V{v};
    GmresResult res{false, 0, tol, beta};
    for (size_t j = 0; j < m; j++) {
        A(v, w);
        for (size_t i = 0; i < j + 1; i++) {
            hs.H(i, j) = dot(w, V[i]);
            double h = -hs.H(i, j);
            for (size_t q = 0; q < nvars; q++) w[q] += V[i][q] * h;
        }
        hs.H(j + 1, j) = std::sqrt(dot(w, w));
        double s = 1.0 / hs.H(j + 1, j);
        for (size_t q = 0; q < nvars; q++) v[q] = w[q] * s;
        V.push_back(v);
        hs.rotate(j);
        double r = std::fabs(hs.g0[j + 1]);
        res.residual = r / beta;
        res.n_iters = j + 1;
        if (r < tol * beta) { res.success = true; break; }
    }
    finish_solution(hs, res.n_iters, V, x);
    return res;
}

GmresResult fgmres_solve(const MatVec& A, const MatVec& P, std::vector<double>& x,
                         const std::vector<double>& rhs, size_t max_iters_cfg, double tol,
                         size_t max_prec_iters, double prec_tol) {
    // gmres.cpp:234-303
    size_t nvars = rhs.size();
    size_t m = std::min(nvars, max_iters_cfg);
    Hess hs(m);
    std::vector<double> w(nvars), r0(nvars), v(nvars), z(nvars);
    A(x, w);
    for (size_t i = 0; i < nvars; i++) r0[i] = rhs[i] - w[i];
    double beta = std::sqrt(dot(r0, r0));
    if (beta < tol) return {true, 0, tol, beta};
    hs.g0[0] = beta;
    for (size_t i = 0; i < nvars; i++) v[i] = r0[i] * (1.0 / beta);
    std::vector<std::vector<double>> V{v}, Z;
    GmresResult res{false, 0, tol, beta};
    for (size_t j = 0; j < m; j++) {
        std::fill(z.begin(), z.end(), 0.0);
        gmres_solve(P, v, z, max_prec_iters, prec_tol);
        Z.push_back(z);
        A(z, w);
        for (size_t i = 0; i < j + 1; i++) {
            hs.H(i, j) = dot(w, V[i]);
            double h = -hs.H(i, j);
            for (size_t q = 0; q < nvars; q++) w[q] += V[i][q] * h;
        }
        hs.H(j + 1, j) = std::sqrt(dot(w, w));
        double s = 1.0 / hs.H(j + 1, j);
        for (size_t q = 0; q < nvars; q++) v[q] = w[q] * s;
        V.push_back(v);
        hs.rotate(j);
        double r = std::fabs(hs.g0[j + 1]);
        res.residual = r / beta;
        res.n_iters = j + 1;
        if (r < tol * beta) { res.success = true; break; }
    }
    finish_solution(hs, res.n_iters, Z, x);
    return res;
}

void Steady::setup(const Json& config, const GridIO& io) {  // steady_state.cpp:176-221
    sim = build_sim<Dual>(config, io);
    size_t NT = sim->grid.N + sim->grid.G;
    size_t nc = sim->grid.dim + 2;
    n_vars = sim->grid.N * nc;
    residuals = Conserved<Dual>(NT, sim->grid.dim);
    cq_tmp = Conserved<Dual>(NT, sim->grid.dim);
    fs_tmp = FlowStates<Dual>(NT);
    rhs.assign(n_vars, 0.0);
    dU.assign(n_vars, 0.0);
    const Json& sc = config.at("solver");
    const Json& ls = sc.at("linear_solver");
    fgmres = ls.at("type").as_string() == "fgmres";
    if (fgmres) {
        max_iters = (size_t)ls.at("max_iters").as_int();
        gmres_tol = ls.at("tolerance").as_double();
        max_prec_iters = (size_t)ls.at("max_preconditioner_iters").as_int();
        prec_tol = ls.at("preconditioner_tolerance").as_double();
    } else {
        max_iters = (size_t)ls.at("max_iters").as_int();
        gmres_tol = ls.at("tol").as_double();
    }
    const Json& cfl = sc.at("cfl");
    std::string ct = cfl.at("type").as_string();
    if (ct == "constant") cfl_const = cfl.at("value").as_double();
    else if (ct == "linear_interpolate") { cfl_times = cfl.at("times").as_doubles(); cfl_values = cfl.at("cfls").as_doubles(); }
    else if (ct == "residual_based") {
        residual_based = true;
        rb_threshold = cfl.at("growth_threshold").as_double(); rb_power = cfl.at("power").as_double();
        rb_start = cfl.at("start_cfl").as_double(); rb_max = cfl.at("max_cfl").as_double();
        rb_prev_cfl = rb_start; rb_prev_res = 1.0;
    }
}

void Steady::matvec(const std::vector<double>& v, std::vector<double>& out, bool allow_reconstruction) {
    Sim<Dual>& s = *sim;
    size_t nc = s.grid.dim + 2;
    for (size_t c = 0; c < s.grid.N; c++) {
        for (size_t q = 0; q < nc; q++) {
            cq_tmp.q[c * nc + q].re = s.U.q[c * nc + q].re;
            cq_tmp.q[c * nc + q].du = v[c * nc + q];
        }
    }
    conserved_to_primatives(cq_tmp, fs_tmp, s.gas);
    s.fv.compute_dudt(fs_tmp, s.grid, residuals, s.gas, s.tp, allow_reconstruction);
    for (size_t c = 0; c < s.grid.N; c++) {
        for (size_t q = 0; q < nc; q++) {
            out[c * nc + q] = 1 / dt_star * v[c * nc + q] - residuals.q[c * nc + q].du;
        }
    }
}

void Steady::eval_rhs() {
    Sim<Dual>& s = *sim;
    s.fv.compute_dudt(s.fs, s.grid, residuals, s.gas, s.tp, true);
    size_t nc = s.grid.dim + 2;
    for (size_t c = 0; c < s.grid.N; c++)
        for (size_t q = 0; q < nc; q++) rhs[c * nc + q] = residuals.q[c * nc + q].re;
}

void Steady::initialise() {
    primatives_to_conserved(sim->U, sim->fs);
    eval_rhs();
    residual_norms = l2_norms(residuals);
    initial_norms = residual_norms;
}

double Steady::calculate_cfl(size_t step) {  // jfnk.h:39-47, cfl.cpp
    if (residual_based) {
        double t = residual_norms.global / initial_norms.global;
        if (t > rb_threshold) { rb_prev_res = t; return rb_prev_cfl; }
        double ratio = rb_prev_res / t;
        double c = rb_prev_cfl * std::pow(ratio, rb_power);
        c = std::min(c, rb_max);
        c = std::max(rb_start, c);
        rb_prev_res = t;
        rb_prev_cfl = c;
        return c;
    }
    if (cfl_times.empty()) return cfl_const;
    double t = (double)step;
    if (t <= cfl_times[0]) return cfl_values[0];
    size_t n = cfl_times.size();
    if (t >= cfl_times[n - 1]) return cfl_values[n - 1];
    for (size_t i = 0; i + 1 < n; i++) {
        if (t >= cfl_times[i] && t < cfl_times[i + 1]) {
            double frac = (t - cfl_times[i]) / (cfl_times[i + 1] - cfl_times[i]);
            return cfl_values[i] + frac * (cfl_values[i + 1] - cfl_values[i]);
        }
    }
    return cfl_values[n - 1];
}

GmresResult Steady::step(size_t step_index) {
    Sim<Dual>& s = *sim;
    std::fill(dU.begin(), dU.end(), 0.0);
    double stable_dt = s.fv.estimate_dt(s.fs, s.grid, s.gas, s.tp);
    double cfl = calculate_cfl(step_index);
    dt_star = cfl * stable_dt;
    MatVec A = [&](const std::vector<double>& v, std::vector<double>& o) { matvec(v, o, true); };
    if (fgmres) {
        MatVec P = [&](const std::vector<double>& v, std::vector<double>& o) { matvec(v, o, false); };
        last = fgmres_solve(A, P, dU, rhs, max_iters, gmres_tol, max_prec_iters, prec_tol);
    } else {
        last = gmres_solve(A, rhs, dU, max_iters, gmres_tol);
    }
    // apply_update_, jfnk.cpp:63-93
    size_t nc = s.grid.dim + 2;
    for (size_t c = 0; c < s.grid.N; c++) {
        for (size_t q = 0; q < nc; q++) {
            s.U.q[c * nc + q].re += dU[c * nc + q];
            s.U.q[c * nc + q].du = 0.0;
        }
    }
    conserved_to_primatives(s.U, s.fs, s.gas);
    eval_rhs();
    residual_norms = l2_norms(residuals);
    return last;
}

void lsq_gradient_real(const Grid<double>& g, const std::vector<double>& values,
                       std::vector<std::array<double, 3>>& grad) {
    lsq_gradient(g, values, grad);
}

FlopCounts g_flops;

template struct Grid<double>;
template struct Grid<Cnt>;
template struct FiniteVolume<Cnt>;
template struct Sim<Cnt>;
template std::unique_ptr<Sim<Cnt>> build_sim<Cnt>(const Json&, const GridIO&);
template void conserved_to_primatives<Cnt>(const Conserved<Cnt>&, FlowStates<Cnt>&, const IdealGas&);
template void primatives_to_conserved<Cnt>(Conserved<Cnt>&, const FlowStates<Cnt>&);
template Norms l2_norms<Cnt>(const Conserved<Cnt>&);
template struct Grid<Dual>;
template struct FiniteVolume<double>;
template struct FiniteVolume<Dual>;
template struct Sim<double>;
template struct Sim<Dual>;
template std::unique_ptr<Sim<double>> build_sim<double>(const Json&, const GridIO&);
template std::unique_ptr<Sim<Dual>> build_sim<Dual>(const Json&, const GridIO&);
template void conserved_to_primatives<double>(const Conserved<double>&, FlowStates<double>&, const IdealGas&);
template void conserved_to_primatives<Dual>(const Conserved<Dual>&, FlowStates<Dual>&, const IdealGas&);
template void primatives_to_conserved<double>(Conserved<double>&, const FlowStates<double>&);
template void primatives_to_conserved<Dual>(Conserved<Dual>&, const FlowStates<Dual>&);
template Norms l2_norms<double>(const Conserved<double>&);
template Norms l2_norms<Dual>(const Conserved<Dual>&);

}  // namespace oracle
