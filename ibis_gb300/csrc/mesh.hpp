// Host-side grid preprocessing for the GB300 residual engine.
//
// Turns an SU2 element list into the face/cell connectivity, geometry, ghost
// cells and least-squares factors the device kernels consume.  Numbering and
// geometry reproduce ibis's GridBlock exactly (src/grid/grid/grid.h:89-167):
// faces are numbered by first appearance while scanning cells in file order and
// their VTK faces in order; a face is identified by its vertex set; ghost cells
// get ids N.. while iterating boundary tags in sorted order, marker faces in
// file order.  Floating-point formulas keep the reference's operation order and
// are compiled without FMA contraction, so connectivity, left/right assignment
// and outsigns are bit-identical to the reference's.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace ibisgb {

enum ElemKind : int8_t { kLine = 0, kTri, kTetra, kQuad, kHex, kWedge, kPyramid };

ElemKind elem_kind_from_vtk(int code);  // grid_io.cpp:28-48
int vertices_per_elem(ElemKind k);      // grid_io.cpp:72-91

// One list of elements (cells or the faces of one marker), CSR connectivity.
struct ElemList {
    std::vector<int8_t> kind;
    std::vector<int64_t> off{0};
    std::vector<int64_t> vtx;
    size_t size() const { return kind.size(); }
    void push(ElemKind k, const int64_t* ids, int n) {
        kind.push_back(k);
        vtx.insert(vtx.end(), ids, ids + n);
        off.push_back((int64_t)vtx.size());
    }
};

struct GridInput {
    int dim = 0;
    std::vector<double> xyz;  // 3 per vertex (z = 0 in 2-D)
    ElemList cells;
    std::map<std::string, ElemList> markers;  // repeated tags are appended
    int64_t num_vertices() const { return (int64_t)xyz.size() / 3; }
};

// SU2 reader (reference: GridIO::read_su2_grid, grid_io.cpp:218-268).
GridInput read_su2(const std::string& path);

struct BoundarySpec {
    std::string tag;
    bool ghost_cells = true;
    bool periodic = false;       // extension: ghost copies the matching cell across the domain
    std::string partner;         // periodic partner tag
    double offset[3] = {0, 0, 0};  // partner face centre = this face centre + offset
};

struct Mesh {
    int dim = 0;
    int64_t N = 0, G = 0, F = 0;
    int MF = 0;  // max faces per cell
    int64_t NT() const { return N + G; }

    // faces
    std::vector<int8_t> face_kind;
    std::vector<int64_t> face_vtx_off, face_vtx;
    std::vector<int64_t> left, right;  // -1 when absent
    std::vector<double> nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z, fcx, fcy, fcz, area;

    // cells, slot-major padded to MF (slot k of cell c at c*MF+k; -1 / 0 padding)
    std::vector<int8_t> cell_kind;
    std::vector<int64_t> cell_vtx_off, cell_vtx;
    std::vector<int32_t> nfaces;
    std::vector<int64_t> cell_face, cell_nbr;
    std::vector<int8_t> outsign;
    std::vector<double> ccx, ccy, ccz, volume;  // N+G entries (ghost volume 0)
    std::vector<double> r;                      // 6 per valid cell: r11 r12 r22 r13 r23 r33
    std::vector<double> lsqw;                   // [3][MF][N] gradient weights of each neighbour slot

    // boundaries in sorted tag order
    std::vector<BoundarySpec> bounds;
    std::vector<std::vector<int64_t>> bound_faces, bound_ghosts;
    std::vector<int64_t> ghost_face, ghost_bound, ghost_src;  // per ghost (index g = id - N)
};

// GridBlock::init_grid_block and friends (grid.h:89-167, 180-232, 340-443),
// Interfaces geometry (interface.h:180-323), Cells geometry (cell.h:228-300),
// WLSGradient::compute_weights (gradient.h:119-162).
void build_mesh(const GridInput& in, const std::vector<BoundarySpec>& bounds, bool need_lsq,
                Mesh& m);

// The least-squares factors (r, lsqw) of a built mesh from its centroids
// (WLSGradient::compute_weights / compute_gradients, gradient.h:89-162).
void compute_lsq(Mesh& m);

// An internal numbering of cells and faces and its map to the reference's
// (each vector maps an id of one numbering to the other).
struct MeshNumbering {
    std::vector<int64_t> cell_new_of_ref, cell_ref_of_new, face_new_of_ref, face_ref_of_new;
    bool active() const { return !cell_ref_of_new.empty(); }
};

// Reverse Cuthill-McKee order of the valid cells (their reference ids in the
// new order) and the bandwidth of the valid-cell graph.
std::vector<int64_t> rcm_cell_order(const Mesh& m);
int64_t cell_bandwidth(const Mesh& m);

// Renumbers the valid cells (cell_ref_of_new: the reference id of each new id)
// and the faces (by their lower, then higher, new cell id) of a built mesh in
// place, keeping each cell's face slots in order and the ghost ids; fills num.
void renumber_mesh(Mesh& m, const std::vector<int64_t>& cell_ref_of_new, MeshNumbering& num);

// Concatenation of independent cases (batched ensembles): valid cells of all
// cases first, in case order, then all ghost cells; faces and boundaries in
// case order.  The offset vectors get one entry per case plus the total.
void merge_meshes(const std::vector<const Mesh*>& parts, Mesh& out, std::vector<int64_t>& cell_off,
                  std::vector<int64_t>& ghost_off, std::vector<int64_t>& face_off,
                  std::vector<int64_t>& bound_off);

}  // namespace ibisgb
