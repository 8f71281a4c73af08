// Host-side grid preprocessing (see mesh.hpp).  Compile with -ffp-contract=off.
#include "mesh.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

#include "json_lite.hpp"

namespace ibisgb {

ElemKind elem_kind_from_vtk(int code) {
    switch (code) {
        case 3: return kLine;
        case 5: return kTri;
        case 9: return kQuad;
        case 10: return kTetra;
        case 12: return kHex;
        case 13: return kWedge;
        case 14: return kPyramid;
        default: throw std::runtime_error("unknown su2 element type " + std::to_string(code));
    }
}

int vertices_per_elem(ElemKind k) {
    static const int n[] = {2, 3, 4, 4, 8, 6, 5};
    return n[(int)k];
}

// ---------------------------------------------------------------- SU2 reader

namespace {

struct LineReader {
    const char* p;
    const char* end;
    // next line with leading/trailing spaces removed; false at end of input
    bool next(const char*& b, const char*& e) {
        if (p >= end) return false;
        const char* nl = (const char*)std::memchr(p, '\n', (size_t)(end - p));
        const char* le = nl ? nl : end;
        b = p;
        e = le;
        p = nl ? nl + 1 : end;
        while (b < e && (*b == ' ' || *b == '\t')) b++;
        while (e > b && (e[-1] == ' ' || e[-1] == '\r' || e[-1] == '\t')) e--;
        return true;
    }
};

bool starts(const char* b, const char* e, const char* key) {
    size_t n = std::strlen(key);
    return (size_t)(e - b) >= n && std::memcmp(b, key, n) == 0;
}

long long value_after_eq(const char* b, const char* e) {
    const char* q = (const char*)std::memchr(b, '=', (size_t)(e - b));
    if (!q) throw std::runtime_error("su2: expected '=' in header line");
    return std::strtoll(q + 1, nullptr, 10);
}

std::string string_after_eq(const char* b, const char* e) {
    const char* q = (const char*)std::memchr(b, '=', (size_t)(e - b));
    if (!q) throw std::runtime_error("su2: expected '=' in header line");
    q++;
    while (q < e && *q == ' ') q++;
    return std::string(q, e);
}

void read_element(const char* b, const char* e, ElemList& out) {
    char* q;
    long code = std::strtol(b, &q, 10);
    ElemKind k = elem_kind_from_vtk((int)code);
    int n = vertices_per_elem(k);
    int64_t ids[8];
    for (int i = 0; i < n; i++) {
        const char* before = q;
        ids[i] = std::strtoll(q, &q, 10);
        if (q == before || q > e) throw std::runtime_error("su2: short element line");
    }
    out.push(k, ids, n);
}

}  // namespace

GridInput read_su2(const std::string& path) {
    std::string text = read_text_file(path);
    GridInput g;
    LineReader lr{text.data(), text.data() + text.size()};
    const char *b, *e;
    while (lr.next(b, e)) {
        if (starts(b, e, "NDIME")) {
            g.dim = (int)value_after_eq(b, e);
        } else if (starts(b, e, "NPOIN")) {
            long long n = value_after_eq(b, e);
            g.xyz.assign((size_t)n * 3, 0.0);
            for (long long i = 0; i < n; i++) {
                if (!lr.next(b, e)) throw std::runtime_error("su2: missing vertices");
                char* q = (char*)b;
                for (int d = 0; d < g.dim; d++) g.xyz[3 * i + d] = std::strtod(q, &q);
            }
        } else if (starts(b, e, "NELEM")) {
            long long n = value_after_eq(b, e);
            for (long long i = 0; i < n; i++) {
                if (!lr.next(b, e)) throw std::runtime_error("su2: missing elements");
                read_element(b, e, g.cells);
            }
        } else if (starts(b, e, "NMARK")) {
            long long nm = value_after_eq(b, e);
            for (long long m = 0; m < nm; m++) {
                if (!lr.next(b, e)) throw std::runtime_error("su2: missing marker");
                std::string tag = string_after_eq(b, e);
                if (!lr.next(b, e)) throw std::runtime_error("su2: missing marker size");
                long long ne = value_after_eq(b, e);
                ElemList& dst = g.markers[tag];
                for (long long k = 0; k < ne; k++) {
                    if (!lr.next(b, e)) throw std::runtime_error("su2: missing marker element");
                    read_element(b, e, dst);
                }
            }
        }
    }
    if (g.dim != 2 && g.dim != 3) throw std::runtime_error("su2: NDIME must be 2 or 3");
    return g;
}

// ------------------------------------------------------------ face numbering

namespace {

// The faces of a cell in VTK order (grid_io.cpp:298-348): local vertex indices.
struct FaceTemplate {
    int n;
    ElemKind kind;
    int v[4];
};

int cell_face_templates(ElemKind k, FaceTemplate* out) {
    auto set = [&](int i, ElemKind kind, std::initializer_list<int> vs) {
        out[i].n = (int)vs.size();
        out[i].kind = kind;
        int j = 0;
        for (int v : vs) out[i].v[j++] = v;
    };
    switch (k) {
        case kTri:
            set(0, kLine, {0, 1}); set(1, kLine, {1, 2}); set(2, kLine, {2, 0});
            return 3;
        case kQuad:
            set(0, kLine, {0, 1}); set(1, kLine, {1, 2}); set(2, kLine, {2, 3}); set(3, kLine, {3, 0});
            return 4;
        case kTetra:
            set(0, kTri, {0, 1, 2}); set(1, kTri, {0, 1, 3}); set(2, kTri, {1, 2, 3}); set(3, kTri, {0, 2, 3});
            return 4;
        case kHex:
            set(0, kQuad, {0, 1, 2, 3}); set(1, kQuad, {0, 1, 5, 4}); set(2, kQuad, {4, 5, 6, 7});
            set(3, kQuad, {2, 3, 7, 6}); set(4, kQuad, {0, 4, 7, 3}); set(5, kQuad, {1, 5, 6, 2});
            return 6;
        case kWedge:
            set(0, kTri, {0, 1, 2}); set(1, kTri, {3, 5, 4}); set(2, kQuad, {1, 4, 5, 2});
            set(3, kQuad, {0, 2, 5, 3}); set(4, kQuad, {0, 3, 4, 1});
            return 5;
        case kPyramid:
            set(0, kQuad, {0, 3, 2, 1}); set(1, kTri, {2, 3, 4}); set(2, kTri, {0, 4, 3});
            set(3, kTri, {0, 1, 4}); set(4, kTri, {1, 2, 4});
            return 5;
        case kLine:
            throw std::runtime_error("a line is not a valid cell");
    }
    return 0;
}

// Open-addressing table keyed by a face's vertex set (ids sorted descending,
// padded with ~0): the reference keys faces by the same sorted list
// (InterfaceLookup::hash_vertex_ids, interface.cpp:38-46).
struct FaceKey {
    uint64_t a, b;  // four 32-bit vertex ids
    bool operator==(const FaceKey& o) const { return a == o.a && b == o.b; }
};

FaceKey make_key(const int64_t* ids, int n) {
    uint32_t s[4] = {~0u, ~0u, ~0u, ~0u};
    for (int i = 0; i < n; i++) {
        if (ids[i] < 0 || ids[i] >= (int64_t)0xFFFFFFFFu) throw std::runtime_error("vertex id out of range");
        s[i] = (uint32_t)ids[i];
    }
    std::sort(s, s + n, [](uint32_t x, uint32_t y) { return x > y; });
    return {((uint64_t)s[0] << 32) | s[1], ((uint64_t)s[2] << 32) | s[3]};
}

struct FaceTable {
    std::vector<FaceKey> keys;
    std::vector<int64_t> vals;
    uint64_t mask;
    // `slots` bounds the number of distinct faces; load factor stays <= 0.8
    explicit FaceTable(size_t slots) {
        size_t cap = 16;
        while (cap < slots + slots / 4) cap <<= 1;
        keys.assign(cap, FaceKey{~0ull, ~0ull});
        vals.assign(cap, -1);
        mask = cap - 1;
    }
    static uint64_t mix(uint64_t x) {
        x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
        return x;
    }
    // returns the slot of key (existing or empty)
    size_t slot(const FaceKey& k) const {
        size_t h = (size_t)(mix(k.a ^ mix(k.b)) & mask);
        while (vals[h] >= 0 && !(keys[h] == k)) h = (h + 1) & mask;
        return h;
    }
};

}  // namespace

// ---------------------------------------------------------------- geometry

namespace {

// geom.h:28-49
double tri_area(const double* X, int64_t a, int64_t b, int64_t c) {
    double abx = X[3 * b] - X[3 * a], aby = X[3 * b + 1] - X[3 * a + 1], abz = X[3 * b + 2] - X[3 * a + 2];
    double acx = X[3 * c] - X[3 * a], acy = X[3 * c + 1] - X[3 * a + 1], acz = X[3 * c + 2] - X[3 * a + 2];
    double crx = aby * acz - abz * acy;
    double cry = abz * acx - abx * acz;
    double crz = abx * acy - aby * acx;
    return 0.5 * std::sqrt(crx * crx + cry * cry + crz * crz);
}

}  // namespace

void build_mesh(const GridInput& in, const std::vector<BoundarySpec>& bounds_in, bool need_lsq,
                Mesh& m) {
    m.dim = in.dim;
    m.N = (int64_t)in.cells.size();
    const double* X = in.xyz.data();
    const int64_t N = m.N;

    // --- faces by first appearance (grid.h:113-133)
    FaceTemplate ft[6];
    int64_t slots = 0;
    m.MF = 0;
    for (int64_t c = 0; c < N; c++) {
        int nf = cell_face_templates((ElemKind)in.cells.kind[c], ft);
        slots += nf;
        m.MF = std::max(m.MF, nf);
    }
    const int MF = m.MF;
    FaceTable table((size_t)slots + 16);
    m.cell_kind = in.cells.kind;
    m.cell_vtx_off = in.cells.off;
    m.cell_vtx = in.cells.vtx;
    m.nfaces.assign(N, 0);
    m.cell_face.assign(N * MF, -1);
    m.face_vtx_off.assign(1, 0);
    int64_t F = 0;
    for (int64_t c = 0; c < N; c++) {
        const int64_t* cv = &in.cells.vtx[in.cells.off[c]];
        int nf = cell_face_templates((ElemKind)in.cells.kind[c], ft);
        m.nfaces[c] = nf;
        for (int k = 0; k < nf; k++) {
            int64_t ids[4];
            for (int j = 0; j < ft[k].n; j++) ids[j] = cv[ft[k].v[j]];
            FaceKey key = make_key(ids, ft[k].n);
            size_t s = table.slot(key);
            if (table.vals[s] < 0) {
                table.keys[s] = key;
                table.vals[s] = F++;
                m.face_kind.push_back(ft[k].kind);
                m.face_vtx.insert(m.face_vtx.end(), ids, ids + ft[k].n);
                m.face_vtx_off.push_back((int64_t)m.face_vtx.size());
            }
            m.cell_face[c * MF + k] = table.vals[s];
        }
    }
    m.F = F;

    // --- boundaries in sorted tag order (setup_boundaries, grid.h:406-443)
    std::vector<BoundarySpec> bounds = bounds_in;
    std::sort(bounds.begin(), bounds.end(),
              [](const BoundarySpec& a, const BoundarySpec& b) { return a.tag < b.tag; });
    m.bounds = bounds;
    m.bound_faces.assign(bounds.size(), {});
    m.bound_ghosts.assign(bounds.size(), {});
    std::vector<int64_t> ghost_of_face(F, -2);  // -2 unset, -1 boundary without ghost cells
    int64_t G = 0;
    for (size_t bi = 0; bi < bounds.size(); bi++) {
        auto it = in.markers.find(bounds[bi].tag);
        if (it == in.markers.end()) continue;  // GridIO returns an empty marker (grid.h:416)
        const ElemList& mk = it->second;
        for (size_t e = 0; e < mk.size(); e++) {
            const int64_t* ids = &mk.vtx[mk.off[e]];
            int n = (int)(mk.off[e + 1] - mk.off[e]);
            FaceKey key = make_key(ids, n);
            size_t s = table.slot(key);
            if (table.vals[s] < 0)
                throw std::runtime_error("marker '" + bounds[bi].tag + "' has a face that belongs to no cell");
            int64_t f = table.vals[s];
            m.bound_faces[bi].push_back(f);
            if (bounds[bi].ghost_cells) {
                int64_t gid = N + G++;
                m.bound_ghosts[bi].push_back(gid);
                if (ghost_of_face[f] == -2) ghost_of_face[f] = gid;  // std::map::insert keeps the first
                m.ghost_face.push_back(f);
                m.ghost_bound.push_back((int64_t)bi);
            } else if (ghost_of_face[f] == -2) {
                ghost_of_face[f] = -1;
            }
        }
    }
    m.G = G;
    const int64_t NT = N + G;

    // --- face geometry (interface.h:180-323)
    m.left.assign(F, -1); m.right.assign(F, -1);
    auto zF = [&](std::vector<double>& v) { v.assign(F, 0.0); };
    zF(m.nx); zF(m.ny); zF(m.nz); zF(m.t1x); zF(m.t1y); zF(m.t1z); zF(m.t2x); zF(m.t2y); zF(m.t2z);
    zF(m.fcx); zF(m.fcy); zF(m.fcz); zF(m.area);
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < F; f++) {
        const int64_t* v = &m.face_vtx[m.face_vtx_off[f]];
        int n = (int)(m.face_vtx_off[f + 1] - m.face_vtx_off[f]);
        double x = 0.0, y = 0.0, z = 0.0;  // compute_centres
        for (int j = 0; j < n; j++) { x += X[3 * v[j]]; y += X[3 * v[j] + 1]; z += X[3 * v[j] + 2]; }
        m.fcx[f] = x / (double)n; m.fcy[f] = y / (double)n; m.fcz[f] = z / (double)n;
        ElemKind k = (ElemKind)m.face_kind[f];  // compute_areas
        if (k == kLine) {
            double dx = X[3 * v[1]] - X[3 * v[0]], dy = X[3 * v[1] + 1] - X[3 * v[0] + 1],
                   dz = X[3 * v[1] + 2] - X[3 * v[0] + 2];
            m.area[f] = std::sqrt(dx * dx + dy * dy + dz * dz);
        } else if (k == kTri) {
            m.area[f] = tri_area(X, v[0], v[1], v[2]);
        } else {
            m.area[f] = tri_area(X, v[0], v[1], v[2]) + tri_area(X, v[0], v[2], v[3]);
        }
        // compute_orientations
        double x0 = X[3 * v[0]], x1 = X[3 * v[1]], y0 = X[3 * v[0] + 1], y1 = X[3 * v[1] + 1];
        double z0 = X[3 * v[0] + 2], z1 = X[3 * v[1] + 2];
        double il = 1. / std::sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0) + (z1 - z0) * (z1 - z0));
        double a1 = il * (x1 - x0), a2 = il * (y1 - y0), a3 = il * (z1 - z0);
        double b1, b2, b3;
        if (k == kLine) {
            b1 = 0.0; b2 = 0.0; b3 = 1.0;
        } else {
            double sx = X[3 * v[2]] - X[3 * v[0]], sy = X[3 * v[2] + 1] - X[3 * v[0] + 1],
                   sz = X[3 * v[2] + 2] - X[3 * v[0] + 2];
            double proj = a1 * sx + a2 * sy + a3 * sz;
            double px = sx - proj * a1, py = sy - proj * a2, pz = sz - proj * a3;
            double il2 = 1.0 / std::sqrt(px * px + py * py + pz * pz);
            b1 = il2 * px; b2 = il2 * py; b3 = il2 * pz;
        }
        m.t1x[f] = a1; m.t1y[f] = a2; m.t1z[f] = a3;
        m.t2x[f] = b1; m.t2y[f] = b2; m.t2z[f] = b3;
        m.nx[f] = a2 * b3 - a3 * b2;  // cross(t1, t2), vector3.h:153-160
        m.ny[f] = a3 * b1 - a1 * b3;
        m.nz[f] = a1 * b2 - a2 * b1;
    }

    // --- cell centroids (cell.h:228-255)
    m.ccx.assign(NT, 0.0); m.ccy.assign(NT, 0.0); m.ccz.assign(NT, 0.0); m.volume.assign(NT, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < N; c++) {
        const int64_t* v = &in.cells.vtx[in.cells.off[c]];
        int n = (int)(in.cells.off[c + 1] - in.cells.off[c]);
        double x = 0.0, y = 0.0, z = 0.0;
        for (int j = 0; j < n; j++) { x += X[3 * v[j]]; y += X[3 * v[j] + 1]; z += X[3 * v[j] + 2]; }
        m.ccx[c] = x / (double)n; m.ccy[c] = y / (double)n; m.ccz[c] = z / (double)n;
    }

    // --- left/right and outsigns (compute_interface_connectivity, grid.h:180-232)
    m.outsign.assign(N * MF, 0);
    for (int64_t c = 0; c < N; c++) {
        for (int k = 0; k < m.nfaces[c]; k++) {
            int64_t f = m.cell_face[c * MF + k];
            double dx = m.fcx[f] - m.ccx[c], dy = m.fcy[f] - m.ccy[c], dz = m.fcz[f] - m.ccz[c];
            double dot = dx * m.nx[f] + dy * m.ny[f] + dz * m.nz[f];
            if (dot > 0.0) { m.left[f] = c; m.outsign[c * MF + k] = 1; }
            else { m.right[f] = c; m.outsign[c * MF + k] = -1; }
        }
    }
    for (int64_t f = 0; f < F; f++) {  // std::map iteration = increasing face id
        int64_t g = ghost_of_face[f];
        if (g < 0) continue;
        if (m.left[f] < 0) m.left[f] = g; else m.right[f] = g;
    }
    for (int64_t f = 0; f < F; f++) {
        if (m.left[f] < 0 || m.right[f] < 0)
            throw std::runtime_error("face " + std::to_string(f) + " has a missing side (boundary without a marker or ghost cells)");
    }

    // --- volumes (cell.h:257-300, geom.h:66-83)
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < N; c++) {
        const int64_t* v = &in.cells.vtx[in.cells.off[c]];
        ElemKind k = (ElemKind)in.cells.kind[c];
        if (k == kTri) {
            m.volume[c] = tri_area(X, v[0], v[1], v[2]);
        } else if (k == kQuad) {
            m.volume[c] = tri_area(X, v[0], v[1], v[2]) + tri_area(X, v[0], v[2], v[3]);
        } else {
            double vol = 0.0;
            for (int j = 0; j < m.nfaces[c]; j++) {
                int64_t f = m.cell_face[c * MF + j];
                double out = (double)m.outsign[c * MF + j];
                double dot = m.fcx[f] * out * m.nx[f] + m.fcy[f] * out * m.ny[f] + m.fcz[f] * out * m.nz[f];
                vol += dot * m.area[f];
            }
            m.volume[c] = vol / 3.0;
        }
    }

    // --- neighbours (grid.h:340-358)
    m.cell_nbr.assign(N * MF, -1);
    for (int64_t c = 0; c < N; c++) {
        for (int k = 0; k < m.nfaces[c]; k++) {
            int64_t f = m.cell_face[c * MF + k];
            m.cell_nbr[c * MF + k] = m.left[f] == c ? m.right[f] : m.left[f];
        }
    }

    // --- ghost centroids mirrored about the face (grid.h:364-403) and ghost sources
    m.ghost_src.assign(G, -1);
    for (size_t bi = 0; bi < bounds.size(); bi++) {
        for (int64_t f : m.bound_faces[bi]) {
            int64_t l = m.left[f], r = m.right[f];
            int64_t valid = l < N ? l : r, ghost = l < N ? r : l;
            if (ghost < N) continue;
            double dx = m.fcx[f] - m.ccx[valid], dy = m.fcy[f] - m.ccy[valid], dz = m.fcz[f] - m.ccz[valid];
            m.ccx[ghost] = m.fcx[f] + dx; m.ccy[ghost] = m.fcy[f] + dy; m.ccz[ghost] = m.fcz[f] + dz;
        }
    }
    for (int64_t g = 0; g < G; g++) {
        int64_t f = m.ghost_face[g];
        int64_t l = m.left[f], r = m.right[f];
        m.ghost_src[g] = l < N ? l : r;
    }
    // periodic extension: the source of a ghost is the valid cell next to the
    // partner face whose centre is this face centre + offset
    for (size_t bi = 0; bi < bounds.size(); bi++) {
        if (!bounds[bi].periodic) continue;
        size_t pi = 0;
        while (pi < bounds.size() && bounds[pi].tag != bounds[bi].partner) pi++;
        if (pi == bounds.size()) throw std::runtime_error("periodic partner '" + bounds[bi].partner + "' not found");
        auto q = [](double v) { return (long long)std::llround(v * 1e9); };
        std::map<std::array<long long, 3>, int64_t> at;
        for (int64_t f : m.bound_faces[pi]) at[{q(m.fcx[f]), q(m.fcy[f]), q(m.fcz[f])}] = f;
        for (size_t j = 0; j < m.bound_faces[bi].size(); j++) {
            int64_t f = m.bound_faces[bi][j];
            std::array<long long, 3> key = {q(m.fcx[f] + bounds[bi].offset[0]), q(m.fcy[f] + bounds[bi].offset[1]),
                                            q(m.fcz[f] + bounds[bi].offset[2])};
            auto it = at.find(key);
            if (it == at.end()) throw std::runtime_error("periodic: no partner face on '" + bounds[pi].tag + "'");
            int64_t pf = it->second;
            int64_t donor = m.left[pf] < N ? m.left[pf] : m.right[pf];
            int64_t ghost = m.left[f] < N ? m.right[f] : m.left[f];
            m.ghost_src[ghost - N] = donor;
        }
    }

    // --- least-squares QR factors (gradient.h:119-162)
    if (need_lsq) compute_lsq(m);
}

// WLSGradient::compute_weights and the per-neighbour weights of compute_gradients
// (gradient.h:89-162) from the centroids: the r factors per valid cell and the
// weights per neighbour slot.
void compute_lsq(Mesh& m) {
    const int64_t N = m.N;
    const int MF = m.MF;
    m.r.assign(N * 6, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < N; c++) {
        double sxx = 0.0, sxy = 0.0, sxz = 0.0, syy = 0.0, syz = 0.0, szz = 0.0;
        double xi = m.ccx[c], yi = m.ccy[c], zi = m.ccz[c];
        for (int k = 0; k < m.nfaces[c]; k++) {
            int64_t nb = m.cell_nbr[c * MF + k];
            double dx = m.ccx[nb] - xi, dy = m.ccy[nb] - yi, dz = m.ccz[nb] - zi;
            sxx += dx * dx; sxy += dx * dy; sxz += dx * dz;
            syy += dy * dy; syz += dy * dz; szz += dz * dz;
        }
        double r11 = std::sqrt(sxx);
        double r12 = 1.0 / r11 * sxy;
        double r22 = std::sqrt(syy - r12 * r12);
        double r13 = 1.0 / r11 * sxz;
        double r23 = 1.0 / r22 * (syz - r12 / r11 * sxz);
        double r33 = std::sqrt(szz - (r13 * r13 + r23 * r23));
        double* rr = &m.r[c * 6];
        rr[0] = r11; rr[1] = r12; rr[2] = r22;
        if (m.dim == 3) { rr[3] = r13; rr[4] = r23; rr[5] = r33; }
    }
    // the weights WLSGradient::compute_gradients applies to each neighbour
    // difference (gradient.h:89-107), stored per neighbour slot
    m.lsqw.assign(3 * (size_t)MF * N, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < N; c++) {
        const double* rr = &m.r[c * 6];
        double r11 = rr[0], r12 = rr[1], r22 = rr[2], r13 = 0.0, r23 = 0.0, r33 = 0.0;
        if (m.dim == 3) { r13 = rr[3]; r23 = rr[4]; r33 = rr[5]; }
        double beta = (r12 * r23 - r13 * r23) / (r11 * r22);
        for (int k = 0; k < m.nfaces[c]; k++) {
            int64_t nb = m.cell_nbr[c * MF + k];
            double dx = m.ccx[nb] - m.ccx[c], dy = m.ccy[nb] - m.ccy[c], dz = m.ccz[nb] - m.ccz[c];
            double a1 = dx / (r11 * r11);
            double a2 = 1.0 / (r22 * r22) * (dy - r12 / r11 * dx);
            double a3 = 0.0;
            if (m.dim == 3) a3 = 1.0 / (r33 * r33) * (dz - r23 / r22 * dy + beta * dx);
            m.lsqw[(0 * (size_t)MF + k) * N + c] = a1 - r12 / r11 * a2 + beta * a3;
            m.lsqw[(1 * (size_t)MF + k) * N + c] = a2 - r23 / r22 * a3;
            m.lsqw[(2 * (size_t)MF + k) * N + c] = a3;
        }
    }
}

}  // namespace ibisgb

namespace ibisgb {

// Concatenates independent cases into one mesh: valid cells of all cases first
// (case order), then the ghost cells of all cases, faces and boundaries in case
// order.  Ids inside each case are shifted by the case's offsets; element and
// vertex lists are not carried over (the device kernels do not use them).
void merge_meshes(const std::vector<const Mesh*>& parts, Mesh& out, std::vector<int64_t>& cell_off,
                  std::vector<int64_t>& ghost_off, std::vector<int64_t>& face_off,
                  std::vector<int64_t>& bound_off) {
    if (parts.empty()) throw std::runtime_error("no cases to merge");
    const size_t nc = parts.size();
    out = Mesh{};
    out.dim = parts[0]->dim;
    cell_off.assign(nc + 1, 0); ghost_off.assign(nc + 1, 0); face_off.assign(nc + 1, 0);
    bound_off.assign(nc + 1, 0);
    bool lsq = !parts[0]->lsqw.empty();
    for (size_t c = 0; c < nc; c++) {
        const Mesh& m = *parts[c];
        if (m.dim != out.dim) throw std::runtime_error("cases of a batch must have the same dimension");
        if (m.lsqw.empty() != !lsq) throw std::runtime_error("cases of a batch must share the gradient settings");
        cell_off[c + 1] = cell_off[c] + m.N;
        ghost_off[c + 1] = ghost_off[c] + m.G;
        face_off[c + 1] = face_off[c] + m.F;
        bound_off[c + 1] = bound_off[c] + (int64_t)m.bounds.size();
        out.MF = std::max(out.MF, m.MF);
    }
    const int64_t N = cell_off[nc], G = ghost_off[nc], F = face_off[nc], MF = out.MF;
    out.N = N; out.G = G; out.F = F;
    auto cell_id = [&](size_t c, int64_t x) -> int64_t {
        if (x < 0) return -1;
        const Mesh& m = *parts[c];
        return x < m.N ? cell_off[c] + x : N + ghost_off[c] + (x - m.N);
    };
    out.left.resize(F); out.right.resize(F);
    std::vector<double>* fo[13] = {&out.nx, &out.ny, &out.nz, &out.t1x, &out.t1y, &out.t1z, &out.t2x,
                                   &out.t2y, &out.t2z, &out.fcx, &out.fcy, &out.fcz, &out.area};
    for (auto* a : fo) a->reserve(F);
    out.nfaces.resize(N);
    out.cell_face.assign(N * MF, -1); out.cell_nbr.assign(N * MF, -1); out.outsign.assign(N * MF, 0);
    out.ccx.resize(N + G); out.ccy.resize(N + G); out.ccz.resize(N + G); out.volume.resize(N + G);
    if (!parts[0]->r.empty()) out.r.reserve(6 * N);
    if (lsq) out.lsqw.assign(3 * (size_t)MF * N, 0.0);
    out.ghost_face.resize(G); out.ghost_bound.resize(G); out.ghost_src.resize(G);
    for (size_t c = 0; c < nc; c++) {
        const Mesh& m = *parts[c];
        for (int64_t f = 0; f < m.F; f++) {
            out.left[face_off[c] + f] = cell_id(c, m.left[f]);
            out.right[face_off[c] + f] = cell_id(c, m.right[f]);
        }
        const std::vector<double>* fi[13] = {&m.nx, &m.ny, &m.nz, &m.t1x, &m.t1y, &m.t1z, &m.t2x,
                                             &m.t2y, &m.t2z, &m.fcx, &m.fcy, &m.fcz, &m.area};
        for (int q = 0; q < 13; q++) fo[q]->insert(fo[q]->end(), fi[q]->begin(), fi[q]->end());
        for (int64_t i = 0; i < m.N; i++) {
            const int64_t o = cell_off[c] + i;
            out.nfaces[o] = m.nfaces[i];
            for (int k = 0; k < m.MF; k++) {
                const int64_t fk = m.cell_face[i * m.MF + k];
                out.cell_face[o * MF + k] = fk < 0 ? -1 : face_off[c] + fk;
                out.cell_nbr[o * MF + k] = cell_id(c, m.cell_nbr[i * m.MF + k]);
                out.outsign[o * MF + k] = m.outsign[i * m.MF + k];
                if (lsq)
                    for (int d = 0; d < 3; d++)
                        out.lsqw[(d * (size_t)MF + k) * N + o] = m.lsqw[(d * (size_t)m.MF + k) * m.N + i];
            }
        }
        if (!m.r.empty()) out.r.insert(out.r.end(), m.r.begin(), m.r.end());
        for (int64_t x = 0; x < m.N + m.G; x++) {
            const int64_t o = cell_id(c, x);
            out.ccx[o] = m.ccx[x]; out.ccy[o] = m.ccy[x]; out.ccz[o] = m.ccz[x]; out.volume[o] = m.volume[x];
        }
        for (int64_t g = 0; g < m.G; g++) {
            const int64_t o = ghost_off[c] + g;
            out.ghost_face[o] = face_off[c] + m.ghost_face[g];
            out.ghost_bound[o] = bound_off[c] + m.ghost_bound[g];
            out.ghost_src[o] = cell_id(c, m.ghost_src[g]);
        }
        for (size_t b = 0; b < m.bounds.size(); b++) {
            out.bounds.push_back(m.bounds[b]);
            std::vector<int64_t> bf, bg;
            for (int64_t f : m.bound_faces[b]) bf.push_back(face_off[c] + f);
            for (int64_t x : m.bound_ghosts[b]) bg.push_back(cell_id(c, x));
            out.bound_faces.push_back(bf);
            out.bound_ghosts.push_back(bg);
        }
    }
}

}  // namespace ibisgb

namespace ibisgb {

// Reverse Cuthill-McKee order of the valid cells over their interior-face
// graph: each connected component breadth-first from a pseudo-peripheral cell
// (the far end of a breadth-first sweep from a cell of least degree),
// neighbours queued by increasing degree, the whole order reversed.
std::vector<int64_t> rcm_cell_order(const Mesh& m) {
    const int64_t N = m.N;
    const int MF = m.MF;
    std::vector<int32_t> deg(N, 0);
    for (int64_t c = 0; c < N; c++)
        for (int k = 0; k < MF; k++) {
            const int64_t nb = m.cell_nbr[c * MF + k];
            if (nb >= 0 && nb < N) deg[c]++;
        }
    std::vector<int64_t> order;
    order.reserve(N);
    std::vector<char> seen(N, 0);
    std::vector<int64_t> level(N, -1), nbrs;
    auto bfs_far = [&](int64_t s) {  // the last cell of a breadth-first sweep (on a scratch level array)
        std::vector<int64_t> q{s};
        level[s] = 0;
        int64_t last = s;
        for (size_t h = 0; h < q.size(); h++) {
            const int64_t c = q[h];
            last = c;
            for (int k = 0; k < MF; k++) {
                const int64_t nb = m.cell_nbr[c * MF + k];
                if (nb < 0 || nb >= N || level[nb] >= 0) continue;
                level[nb] = level[c] + 1;
                q.push_back(nb);
            }
        }
        for (int64_t c : q) level[c] = -1;
        return last;
    };
    std::vector<int64_t> by_degree(N);
    for (int64_t c = 0; c < N; c++) by_degree[c] = c;
    std::stable_sort(by_degree.begin(), by_degree.end(), [&](int64_t a, int64_t b) { return deg[a] < deg[b]; });
    for (int64_t s0 : by_degree) {
        if (seen[s0]) continue;
        const int64_t s = bfs_far(bfs_far(s0));
        const size_t head0 = order.size();
        order.push_back(s);
        seen[s] = 1;
        for (size_t h = head0; h < order.size(); h++) {
            const int64_t c = order[h];
            nbrs.clear();
            for (int k = 0; k < MF; k++) {
                const int64_t nb = m.cell_nbr[c * MF + k];
                if (nb >= 0 && nb < N && !seen[nb]) {
                    seen[nb] = 1;
                    nbrs.push_back(nb);
                }
            }
            std::stable_sort(nbrs.begin(), nbrs.end(), [&](int64_t a, int64_t b) { return deg[a] < deg[b]; });
            order.insert(order.end(), nbrs.begin(), nbrs.end());
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

// Bandwidth of the valid-cell graph: the largest |i - j| over interior faces.
int64_t cell_bandwidth(const Mesh& m) {
    int64_t b = 0;
    for (int64_t f = 0; f < m.F; f++)
        if (m.left[f] >= 0 && m.left[f] < m.N && m.right[f] >= 0 && m.right[f] < m.N)
            b = std::max<int64_t>(b, std::llabs(m.left[f] - m.right[f]));
    return b;
}

void renumber_mesh(Mesh& m, const std::vector<int64_t>& cell_ref_of_new, MeshNumbering& num) {
    const int64_t N = m.N, F = m.F, G = m.G;
    const int MF = m.MF;
    num.cell_ref_of_new = cell_ref_of_new;
    num.cell_new_of_ref.assign(N, -1);
    for (int64_t c = 0; c < N; c++) num.cell_new_of_ref[cell_ref_of_new[c]] = c;
    auto cnew = [&](int64_t c) { return c >= 0 && c < N ? num.cell_new_of_ref[c] : c; };  // ghosts keep their ids
    // faces by their lower, then higher, new cell id
    std::vector<int64_t> fo(F);
    for (int64_t f = 0; f < F; f++) fo[f] = f;
    auto key = [&](int64_t f) {
        const int64_t a = cnew(m.left[f]), b = cnew(m.right[f]);
        return std::make_pair(std::min(a, b), std::max(a, b));
    };
    std::stable_sort(fo.begin(), fo.end(), [&](int64_t x, int64_t y) { return key(x) < key(y); });
    num.face_ref_of_new = fo;
    num.face_new_of_ref.assign(F, -1);
    for (int64_t f = 0; f < F; f++) num.face_new_of_ref[fo[f]] = f;
    auto fnew = [&](int64_t f) { return f >= 0 ? num.face_new_of_ref[f] : f; };

    // faces
    {
        std::vector<int8_t> kind(F);
        std::vector<int64_t> off(1, 0), vtx, l(F), r(F);
        std::vector<double>* g[13] = {&m.nx, &m.ny, &m.nz, &m.t1x, &m.t1y, &m.t1z, &m.t2x, &m.t2y, &m.t2z,
                                      &m.fcx, &m.fcy, &m.fcz, &m.area};
        std::vector<std::vector<double>> gn(13, std::vector<double>(F));
        for (int64_t f = 0; f < F; f++) {
            const int64_t o = fo[f];
            kind[f] = m.face_kind[o];
            vtx.insert(vtx.end(), m.face_vtx.begin() + m.face_vtx_off[o], m.face_vtx.begin() + m.face_vtx_off[o + 1]);
            off.push_back((int64_t)vtx.size());
            l[f] = cnew(m.left[o]);
            r[f] = cnew(m.right[o]);
            for (int q = 0; q < 13; q++) gn[q][f] = (*g[q])[o];
        }
        m.face_kind.swap(kind); m.face_vtx_off.swap(off); m.face_vtx.swap(vtx); m.left.swap(l); m.right.swap(r);
        for (int q = 0; q < 13; q++) g[q]->swap(gn[q]);
    }
    // cells (slot order within a cell is kept: it is the reference's summation order)
    {
        std::vector<int8_t> kind(N), osg((size_t)N * MF);
        std::vector<int64_t> off(1, 0), vtx, cf((size_t)N * MF), cn((size_t)N * MF);
        std::vector<int32_t> nf(N);
        std::vector<double> cx(m.ccx), cy(m.ccy), cz(m.ccz), vol(m.volume), rr(m.r.size()), w(m.lsqw.size());
        for (int64_t c = 0; c < N; c++) {
            const int64_t o = cell_ref_of_new[c];
            kind[c] = m.cell_kind[o];
            vtx.insert(vtx.end(), m.cell_vtx.begin() + m.cell_vtx_off[o], m.cell_vtx.begin() + m.cell_vtx_off[o + 1]);
            off.push_back((int64_t)vtx.size());
            nf[c] = m.nfaces[o];
            for (int k = 0; k < MF; k++) {
                cf[c * MF + k] = fnew(m.cell_face[o * MF + k]);
                cn[c * MF + k] = cnew(m.cell_nbr[o * MF + k]);
                osg[c * MF + k] = m.outsign[o * MF + k];
            }
            cx[c] = m.ccx[o]; cy[c] = m.ccy[o]; cz[c] = m.ccz[o]; vol[c] = m.volume[o];
            if (!m.r.empty())
                for (int q = 0; q < 6; q++) rr[c * 6 + q] = m.r[o * 6 + q];
            if (!m.lsqw.empty())
                for (int a = 0; a < 3; a++)
                    for (int k = 0; k < MF; k++) w[((size_t)a * MF + k) * N + c] = m.lsqw[((size_t)a * MF + k) * N + o];
        }
        m.cell_kind.swap(kind); m.cell_vtx_off.swap(off); m.cell_vtx.swap(vtx); m.nfaces.swap(nf);
        m.cell_face.swap(cf); m.cell_nbr.swap(cn); m.outsign.swap(osg);
        m.ccx.swap(cx); m.ccy.swap(cy); m.ccz.swap(cz); m.volume.swap(vol);
        m.r.swap(rr); m.lsqw.swap(w);
    }
    // boundaries and ghosts (ghost ids are unchanged)
    for (auto& bf : m.bound_faces)
        for (auto& f : bf) f = fnew(f);
    for (int64_t g = 0; g < G; g++) {
        m.ghost_face[g] = fnew(m.ghost_face[g]);
        m.ghost_src[g] = cnew(m.ghost_src[g]);
    }
}

}  // namespace ibisgb
