// Plain structures shared by the host's structured-block detection and the
// fused stage kernel.
#pragma once

namespace ibisgb {

// One structured block, as the device sees it.
struct SBlock {
    int c0;          // first valid cell
    int ni, nj, nk;  // lattice extents (nk = 1 in 2-D)
    int f0[3];       // first structured face of each direction (i, j, k)
    int g0[6];       // first ghost-map entry of each side (-i, +i, -j, +j, -k, +k)
};

// One tile of the fused kernel: a block and the lattice origin of the tile.
struct STile {
    int block, i0, j0, k0;
};

// Device pointers of the structured view of a context.
struct SbView {
    const SBlock* blocks;
    const STile* tiles;
    int num_tiles;
    const float* face;      // [7][SF]: oriented normal, area, centre
    int SF;
    const int* ghost_map;
    void* prim_out;         // primitives of the new state (the other buffer)
    unsigned* fault;        // plane-marching stage: set when a TMA copy did not complete in time
};

}  // namespace ibisgb
