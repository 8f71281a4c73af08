// Recognition of structured blocks in an already-built Mesh (see structured.hpp).
#include "structured.hpp"

#include <algorithm>

namespace ibisgb {

bool detect_structured(const Mesh& m, const std::vector<int64_t>& cell_off, int tx, int ty, int tz,
                       StructuredLayout& out, std::string* why) {
    auto fail = [&](const std::string& s) {
        if (why) *why = s;
        return false;
    };
    const int dim = m.dim;
    const int nd = 2 * dim;
    const int64_t N = m.N, F = m.F;
    const int MF = m.MF;
    if (dim != 2 && dim != 3) return fail("grid dimension must be 2 or 3");
    out = StructuredLayout{};
    out.dim = dim;
    out.num_faces = F;
    out.face.assign(7 * (size_t)F, 0.0);
    std::vector<char> seen(F, 0);
    int64_t sf = 0, ng = 0;
    for (size_t b = 0; b + 1 < cell_off.size(); b++) {
        const int64_t c0 = cell_off[b], n = cell_off[b + 1] - c0;
        for (int64_t c = c0; c < c0 + n; c++)
            if (m.nfaces[c] != nd) return fail("cells are not all quadrilaterals / hexahedra");
        // lattice extents from the valid neighbours of the first cell (a corner)
        std::vector<int64_t> offs;
        for (int s = 0; s < nd; s++) {
            const int64_t nb = m.cell_nbr[c0 * MF + s];
            if (nb >= c0 && nb < c0 + n) offs.push_back(nb - c0);
        }
        std::sort(offs.begin(), offs.end());
        if ((int)offs.size() != dim || offs[0] != 1) return fail("the first cell is not a lattice corner");
        const int64_t ni = offs[1];
        int64_t nj, nk = 1;
        if (dim == 2) {
            nj = n / ni;
        } else {
            if (offs[2] % ni) return fail("cell numbering is not lexicographic");
            nj = offs[2] / ni;
            nk = n / (ni * nj);
        }
        if (ni * nj * nk != n) return fail("cell count is not a lattice");
        if (ni < 3 || nj < 3 || (dim == 3 && nk < 3)) return fail("lattice too small (fewer than 3 cells a side)");
        const int64_t stride[3] = {1, ni, ni * nj};
        // slot -> direction (0: -i, 1: +i, 2: -j, 3: +j, 4: -k, 5: +k) from an interior cell
        const int64_t ci = c0 + 1 + ni * (1 + (dim == 3 ? nj : 0));
        int dir_of_slot[6] = {-1, -1, -1, -1, -1, -1}, slot_of_dir[6] = {-1, -1, -1, -1, -1, -1};
        for (int s = 0; s < nd; s++) {
            const int64_t off = m.cell_nbr[ci * MF + s] - ci;
            for (int d = 0; d < nd; d++)
                if (off == (d & 1 ? 1 : -1) * stride[d >> 1]) dir_of_slot[s] = d;
            if (dir_of_slot[s] < 0 || slot_of_dir[dir_of_slot[s]] >= 0) return fail("cell neighbours are not a lattice");
            slot_of_dir[dir_of_slot[s]] = s;
        }
        SBlock blk{};
        blk.c0 = (int)c0;
        blk.ni = (int)ni; blk.nj = (int)nj; blk.nk = (int)nk;
        const int64_t ext[3] = {ni, nj, nk};
        const int64_t side_count[6] = {nj * nk, nj * nk, ni * nk, ni * nk, dim == 3 ? ni * nj : 0, dim == 3 ? ni * nj : 0};
        for (int sd = 0; sd < 6; sd++) {
            blk.g0[sd] = (int)ng;
            ng += side_count[sd];
        }
        out.ghost_map.resize(ng, -1);
        for (int a = 0; a < dim; a++) {
            blk.f0[a] = (int)sf;
            sf += (ni + (a == 0)) * (nj + (a == 1)) * (nk + (a == 2));
        }
        auto side_pos = [&](int a, int64_t i, int64_t j, int64_t k) {
            return a == 0 ? j + nj * k : (a == 1 ? i + ni * k : i + ni * j);
        };
        auto face_index = [&](int a, int64_t i, int64_t j, int64_t k) {  // lattice face at the -a side of (i,j,k)
            if (a == 0) return blk.f0[0] + i + (ni + 1) * (j + nj * k);
            if (a == 1) return blk.f0[1] + i + ni * (j + (nj + 1) * k);
            return blk.f0[2] + i + ni * (j + nj * k);
        };
        for (int64_t k = 0; k < nk; k++)
            for (int64_t j = 0; j < nj; j++)
                for (int64_t i = 0; i < ni; i++) {
                    const int64_t c = c0 + i + ni * (j + nj * k);
                    const int64_t ijk[3] = {i, j, k};
                    for (int d = 0; d < nd; d++) {
                        const int a = d >> 1, up = d & 1;
                        const int64_t nb = m.cell_nbr[c * MF + slot_of_dir[d]];
                        const bool inside = up ? ijk[a] + 1 < ext[a] : ijk[a] > 0;
                        if (inside) {
                            if (nb != c + (up ? 1 : -1) * stride[a]) return fail("cell neighbours are not a lattice");
                        } else {
                            if (nb < N) return fail("a lattice boundary face has no ghost cell");
                            out.ghost_map[blk.g0[d] + side_pos(a, i, j, k)] = (int)nb;
                        }
                        if (up && inside) continue;  // interior faces are taken at their upper cell
                        const int64_t f = m.cell_face[c * MF + slot_of_dir[d]];
                        const int64_t lower = up ? c : nb, upper = up ? nb : c;
                        double sign;
                        if (m.left[f] == lower && m.right[f] == upper) sign = 1.0;
                        else if (m.left[f] == upper && m.right[f] == lower) sign = -1.0;
                        else return fail("face sides do not match the lattice");
                        int64_t li[3] = {i, j, k};
                        li[a] += up;
                        const int64_t s = face_index(a, li[0], li[1], li[2]);
                        if (seen[f]++) return fail("a face is shared by two lattice positions");
                        const double v[7] = {sign * m.nx[f], sign * m.ny[f], sign * m.nz[f], m.area[f],
                                             m.fcx[f], m.fcy[f], m.fcz[f]};
                        for (int q = 0; q < 7; q++) out.face[q * (size_t)F + s] = v[q];
                    }
                }
        out.blocks.push_back(blk);
        for (int64_t kt = 0; kt < nk; kt += tz)
            for (int64_t jt = 0; jt < nj; jt += ty)
                for (int64_t it = 0; it < ni; it += tx)
                    out.tiles.push_back(STile{(int)b, (int)it, (int)jt, (int)kt});
    }
    if (sf != F) return fail("faces outside the lattices");
    return true;
}

}  // namespace ibisgb
