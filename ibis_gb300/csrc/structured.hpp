// Structured-block view of a grid for the fused stage kernel.
//
// Grids whose cells are quads (2-D) or hexahedra (3-D) numbered lexicographically
// (i fastest) on an ni x nj [x nk] lattice -- the layout of a structured block
// written as SU2 -- are recognised from the face/cell connectivity the generic
// path already built.  For each such block the fused kernel needs: the lattice
// extents, the faces of each lattice direction in lattice order with their
// geometry oriented along +i / +j / +k, and the ghost cell behind every boundary
// face.  A batched ensemble is one block per case.  Nothing here changes the
// reference numbering: the generic arrays stay as they are and these are extra.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mesh.hpp"
#include "sblock.hpp"

namespace ibisgb {

struct StructuredLayout {
    int dim = 0;
    int64_t num_faces = 0;           // structured faces (= the mesh's faces)
    std::vector<SBlock> blocks;
    std::vector<STile> tiles;
    std::vector<double> face;        // [7][num_faces]: oriented normal (3), area, centre (3)
    std::vector<int> ghost_map;      // ghost cell id behind each boundary face, per block side
};

// Recognise every block [cell_off[b], cell_off[b+1]) of `m` as a structured
// lattice and fill `out` with tiles of tx x ty x tz cells.  Returns false (and
// the reason in *why) when any block is not one.
bool detect_structured(const Mesh& m, const std::vector<int64_t>& cell_off, int tx, int ty, int tz,
                       StructuredLayout& out, std::string* why);

}  // namespace ibisgb
