"""Checks that the test grids generated by ibis_gb300.grids match the reference's
own fixture files element for element, so that the golden vectors transcribed in
reference_unit_vectors.json (which the reference checks on those files) apply to
the generated grids.  Needs the reference checkout; run by hand:

    python tests/golden/check_reference_fixtures.py /path/to/ibis
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", ".."))
from ibis_gb300 import grids  # noqa: E402


def read_su2(path):
    dim, verts, cells, markers, tag = 0, [], [], {}, None
    lines = [ln.strip() for ln in open(path)]
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("NDIME"):
            dim = int(ln.split("=")[1])
        elif ln.startswith("NPOIN"):
            n = int(ln.split("=")[1])
            verts = [list(map(float, lines[i + 1 + k].split()[:dim])) for k in range(n)]
            i += n
        elif ln.startswith("NELEM"):
            n = int(ln.split("=")[1])
            for k in range(n):
                t = list(map(int, lines[i + 1 + k].split()))
                nv = {9: 4, 12: 8, 5: 3, 10: 4}[t[0]]
                cells.append(t[: 1 + nv])
            i += n
        elif ln.startswith("MARKER_TAG"):
            tag = ln.split("=")[1].strip()
        elif ln.startswith("MARKER_ELEMS"):
            n = int(ln.split("=")[1])
            markers.setdefault(tag, []).extend(
                sorted(map(int, lines[i + 1 + k].split()[1:])) for k in range(n))
            i += n
        i += 1
    return dim, np.array(verts), cells, markers


def same(grid, path):
    dim, verts, cells, markers = read_su2(path)
    assert dim == grid.dim
    assert np.allclose(verts, grid.xyz[:, :dim]), "vertices differ"
    for c, ref in enumerate(cells):
        ids = grid.cell_conn[grid.cell_offsets[c]:grid.cell_offsets[c + 1]]
        assert [int(grid.cell_types[c])] + [int(v) for v in ids] == ref, f"cell {c} differs"
    for tag, elems in markers.items():
        types, offs, conn = grid.markers[tag]
        mine = [sorted(int(v) for v in conn[offs[e]:offs[e + 1]]) for e in range(len(types))]
        assert sorted(mine) == sorted(elems), f"marker {tag} differs"
    print(f"{path}: identical to the generated grid")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(sys.argv[0])} <path of an ibis checkout>")
    ref = sys.argv[1]
    same(grids.unit_square_3x3(), os.path.join(ref, "src/grid/test/grid.su2"))
    same(grids.unit_cube_3x3x3(), os.path.join(ref, "src/grid/test/cube.su2"))
