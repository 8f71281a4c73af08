"""Grids in ibis's SU2 format and config.json documents for the benchmark cases.

ibis reads one SU2 block per simulation (reference: src/grid/grid/grid_io.cpp:218-268)
and a ``config/config.json`` written by its Python prep step
(src/ibis/ibis/commands/prep/prep.py:1134-1175).  gmsh, which the reference's
examples use to build grids, is not available, so the structured grids of the
benchmark cases are generated here directly as SU2 element lists:

* ``ramp_2d``        – 15 degree compression ramp (a supersonic wedge case)
* ``flat_plate_2d``  – laminar flat plate with wall-normal geometric stretching
* ``box_3d``         – unit cube of hexahedra with six boundary markers
* ``unit_square_3x3``/``unit_cube_3x3x3`` – the reference's own 3x3(x3) test grids

Element vertex order follows VTK (quads counter-clockwise, hexes bottom face then
top face), like the reference's SU2 files.
"""
from __future__ import annotations

import copy
import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

VTK_LINE, VTK_TRI, VTK_QUAD, VTK_TETRA, VTK_HEX, VTK_WEDGE, VTK_PYRAMID = 3, 5, 9, 10, 12, 13, 14


@dataclass
class Su2Grid:
    """An SU2 grid held as arrays: vertices, cells and boundary markers."""

    dim: int
    xyz: np.ndarray                      # (nv, 3) float64
    cell_types: np.ndarray               # (nc,) int32 VTK codes
    cell_offsets: np.ndarray             # (nc+1,) int64
    cell_conn: np.ndarray                # flat int64 vertex ids
    markers: dict = field(default_factory=dict)  # tag -> (types, offsets, conn)

    @property
    def num_cells(self) -> int:
        return int(self.cell_types.shape[0])

    def write(self, path: str) -> None:
        """Write the grid as an SU2 text file, as ibis's prep step expects."""
        with open(path, "w") as f:
            f.write(f"NDIME= {self.dim}\n")
            f.write(f"NELEM= {self.num_cells}\n")
            off = self.cell_offsets
            for c in range(self.num_cells):
                ids = " ".join(str(int(v)) for v in self.cell_conn[off[c]:off[c + 1]])
                f.write(f"{int(self.cell_types[c])} {ids} {c}\n")
            f.write(f"NPOIN= {self.xyz.shape[0]}\n")
            for i, p in enumerate(self.xyz):
                coords = " ".join(repr(float(x)) for x in p[: self.dim])
                f.write(f"{coords} {i}\n")
            f.write(f"NMARK= {len(self.markers)}\n")
            for tag, (types, offs, conn) in self.markers.items():
                f.write(f"MARKER_TAG= {tag}\n")
                f.write(f"MARKER_ELEMS= {len(types)}\n")
                for e in range(len(types)):
                    ids = " ".join(str(int(v)) for v in conn[offs[e]:offs[e + 1]])
                    f.write(f"{int(types[e])} {ids}\n")

    def marker_arrays(self):
        """Markers flattened for the C ABI: names joined by newlines, element
        offsets per marker, element types, element vertex offsets and ids."""
        names, m_off, e_types, e_off, e_conn = [], [0], [], [0], []
        for tag, (types, offs, conn) in self.markers.items():
            names.append(tag)
            for e in range(len(types)):
                e_types.append(int(types[e]))
                ids = conn[offs[e]:offs[e + 1]]
                e_conn.extend(int(v) for v in ids)
                e_off.append(len(e_conn))
            m_off.append(len(e_types))
        return ("\n".join(names), np.asarray(m_off, np.int64), np.asarray(e_types, np.int32),
                np.asarray(e_off, np.int64), np.asarray(e_conn, np.int64))


def _markers_from_lists(lists: dict) -> dict:
    out = {}
    for tag, (etype, elems) in lists.items():
        elems = np.asarray(elems, np.int64).reshape(len(elems), -1)
        n, k = elems.shape
        out[tag] = (np.full(n, etype, np.int32), np.arange(0, n * k + 1, k, dtype=np.int64),
                    elems.reshape(-1))
    return out


def structured_2d(X: np.ndarray, Y: np.ndarray, bottom_tags=None) -> Su2Grid:
    """Quads on a (ni+1, nj+1) vertex lattice; vertex id = i + (ni+1) j.

    Markers: ``west`` (i=0), ``east`` (i=ni), ``north`` (j=nj) and the bottom
    (j=0), split by ``bottom_tags(i) -> tag`` when given (default ``south``)."""
    ni, nj = X.shape[0] - 1, X.shape[1] - 1
    vid = lambda i, j: i + (ni + 1) * j  # noqa: E731
    xyz = np.zeros(((ni + 1) * (nj + 1), 3))
    xyz[:, 0] = X.T.reshape(-1)
    xyz[:, 1] = Y.T.reshape(-1)
    ii, jj = np.meshgrid(np.arange(ni), np.arange(nj), indexing="xy")
    ii, jj = ii.reshape(-1), jj.reshape(-1)  # cell c = i + ni j
    conn = np.stack([vid(ii, jj), vid(ii + 1, jj), vid(ii + 1, jj + 1), vid(ii, jj + 1)], 1)
    lists = {"west": [], "east": [], "north": []}
    for j in range(nj):
        lists["west"].append((vid(0, j), vid(0, j + 1)))
        lists["east"].append((vid(ni, j), vid(ni, j + 1)))
    for i in range(ni):
        lists["north"].append((vid(i, nj), vid(i + 1, nj)))
        tag = bottom_tags(i) if bottom_tags else "south"
        lists.setdefault(tag, []).append((vid(i, 0), vid(i + 1, 0)))
    markers = _markers_from_lists({k: (VTK_LINE, v) for k, v in lists.items() if v})
    n = ni * nj
    return Su2Grid(2, xyz, np.full(n, VTK_QUAD, np.int32), np.arange(0, 4 * n + 1, 4, dtype=np.int64),
                   conn.reshape(-1).astype(np.int64), markers)


def _cells(g: Su2Grid):
    return [g.cell_conn[g.cell_offsets[c]:g.cell_offsets[c + 1]] for c in range(g.num_cells)]


def _grid_from_cells(g: Su2Grid, types, cells, markers, xyz=None) -> Su2Grid:
    lens = np.array([len(c) for c in cells], np.int64)
    return Su2Grid(g.dim, g.xyz if xyz is None else xyz, np.asarray(types, np.int32),
                   np.concatenate([[0], np.cumsum(lens)]).astype(np.int64),
                   np.concatenate(cells).astype(np.int64), markers)


def _split_marker_quads(g: Su2Grid, faces: set) -> dict:
    """Boundary quads split into the two triangles that are faces of the cells
    (the diagonal through the first vertex, or the other one)."""
    out = {}
    for tag, (types, offs, conn) in g.markers.items():
        tris = []
        for e in range(len(types)):
            a, b, c, d = conn[offs[e]:offs[e + 1]]
            if frozenset((a, b, c)) in faces:
                tris += [(a, b, c), (a, c, d)]
            else:
                tris += [(a, b, d), (b, c, d)]
        out[tag] = (np.full(len(tris), VTK_TRI, np.int32), np.arange(0, 3 * len(tris) + 1, 3, dtype=np.int64),
                    np.asarray(tris, np.int64).reshape(-1))
    return out


def triangulate_2d(g: Su2Grid) -> Su2Grid:
    """Each quad (v0, v1, v2, v3) as two triangles, the diagonal alternating
    with the cell index; the boundary markers are unchanged."""
    cells, types = [], []
    for k, (a, b, c, d) in enumerate(_cells(g)):
        if k % 2 == 0:
            cells += [np.array([a, b, c]), np.array([a, c, d])]
        else:
            cells += [np.array([a, b, d]), np.array([b, c, d])]
        types += [VTK_TRI, VTK_TRI]
    return _grid_from_cells(g, types, cells, g.markers)


def tetrahedralize(g: Su2Grid) -> Su2Grid:
    """Each hexahedron as six tetrahedra around its diagonal v0-v6 (conforming
    between neighbours of a lexicographic hex grid); boundary quads split to match."""
    cells, faces = [], set()
    for h in _cells(g):
        for t in ((0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)):
            tet = h[list(t)]
            cells.append(tet)
            for f in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
                faces.add(frozenset(tet[list(f)]))
    return _grid_from_cells(g, [VTK_TETRA] * len(cells), cells, _split_marker_quads(g, faces))


def shuffle_cells(g: Su2Grid, seed: int = 0) -> Su2Grid:
    """The same grid with its cells listed in a seeded random order (as some
    unstructured generators write them); vertices and markers unchanged.  Cell k
    of the result is cell perm[k] of g, perm = np.random.default_rng(seed).permutation(num_cells)."""
    perm = np.random.default_rng(seed).permutation(g.num_cells)
    lens = (g.cell_offsets[1:] - g.cell_offsets[:-1])[perm]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    idx = np.arange(off[-1]) - np.repeat(off[:-1], lens) + np.repeat(g.cell_offsets[:-1][perm], lens)
    out = copy.copy(g)
    out.cell_conn = g.cell_conn[idx]
    out.cell_types = g.cell_types[perm]
    out.cell_offsets = off
    return out


def tet_channel_case(n: int, shuffle_seed: int | None = None, **kw):
    """A 3-D channel of n^3 hexahedra split into 6 n^3 tetrahedra (optionally listed
    in shuffled order): supersonic inflow (west, Mach ~2 at 300 K, 1e5 Pa, slightly
    oblique) and outflow (east), slip walls elsewhere.  Returns (grid, config, inflow)."""
    gas = ideal_gas(287.0)
    inflow = flow_state(gas, 300.0, 1e5, 700.0, 30.0, 20.0)
    g = tetrahedralize(box_3d(n))
    if shuffle_seed is not None:
        g = shuffle_cells(g, shuffle_seed)
    b = {"west": supersonic_inflow(inflow), "east": supersonic_outflow(), "south": slip_wall(),
         "north": slip_wall(), "bottom": slip_wall(), "top": slip_wall()}
    return g, make_config(3, b, gas=gas, **kw), inflow


def prisms_3d(g: Su2Grid) -> Su2Grid:
    """Each hexahedron as two wedges (triangular prisms) split by its v0-v2 / v4-v6
    diagonal plane; the bottom and top boundary quads split to match."""
    cells, faces = [], set()
    for h in _cells(g):
        for w in ((0, 1, 2, 4, 5, 6), (0, 2, 3, 4, 6, 7)):
            wed = h[list(w)]
            cells.append(wed)
            faces.add(frozenset(wed[[0, 1, 2]]))
            faces.add(frozenset(wed[[3, 4, 5]]))
    markers = {}
    split = _split_marker_quads(g, faces)
    for tag, m in g.markers.items():
        conn = m[2].reshape(-1, 4)
        if all(frozenset(q[[0, 1, 2]]) in faces or frozenset(q[[0, 1, 3]]) in faces for q in conn):
            markers[tag] = split[tag]  # a face of triangles
        else:
            markers[tag] = m
    return _grid_from_cells(g, [VTK_WEDGE] * len(cells), cells, markers)


def pyramids_3d(g: Su2Grid) -> Su2Grid:
    """Each hexahedron as six pyramids on its faces with the apex at a new vertex
    at the hex centre; the boundary quads are the pyramids' bases, unchanged."""
    cells, extra = [], []
    nv = g.xyz.shape[0]
    hex_faces = ((0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7))
    for h in _cells(g):
        apex = nv + len(extra)
        extra.append(g.xyz[h].mean(axis=0))
        for f in hex_faces:
            cells.append(np.concatenate([h[list(f)], [apex]]))
    xyz = np.vstack([g.xyz, np.asarray(extra)])
    return _grid_from_cells(g, [VTK_PYRAMID] * len(cells), cells, g.markers, xyz)


def unit_square_3x3() -> Su2Grid:
    """The reference's 3x3 quad test grid (src/grid/test/grid.su2) with its tags."""
    x = np.arange(4, dtype=float)
    X, Y = np.meshgrid(x, x, indexing="ij")
    g = structured_2d(X, Y)
    rename = {"south": "slip_wall_bottom", "east": "outflow", "north": "slip_wall_top",
              "west": "inflow"}
    g.markers = {rename[k]: v for k, v in g.markers.items()}
    return g


def ramp_2d(ni=256, nj=128, length=1.0, height=0.5, ramp_start=0.2, angle_deg=15.0) -> Su2Grid:
    """Compression ramp: bottom wall flat to ``ramp_start`` then inclined at
    ``angle_deg``; vertical grid lines, uniform spacing between wall and top.
    Markers: ``inflow`` (x=0), ``outflow`` (x=length), ``wall`` (bottom),
    ``top`` (y=height)."""
    x = np.linspace(0.0, length, ni + 1)
    yb = np.where(x > ramp_start, (x - ramp_start) * math.tan(math.radians(angle_deg)), 0.0)
    eta = np.linspace(0.0, 1.0, nj + 1)
    X = np.repeat(x[:, None], nj + 1, 1)
    Y = yb[:, None] + (height - yb[:, None]) * eta[None, :]
    g = structured_2d(X, Y, bottom_tags=lambda i: "wall")
    rename = {"west": "inflow", "east": "outflow", "north": "top", "wall": "wall"}
    g.markers = {rename[k]: v for k, v in g.markers.items()}
    return g


def hicks_henne(s: np.ndarray, peak: float, width: float = 3.0) -> np.ndarray:
    """Hicks-Henne bump sin(pi s^m)^width on s in [0, 1], m = ln 0.5 / ln peak,
    which is 1 at s = peak and 0 at both ends."""
    s = np.clip(s, 0.0, 1.0)
    m = math.log(0.5) / math.log(peak)
    return np.sin(math.pi * s ** m) ** width


def ramp_bump_peaks(n: int = 16) -> np.ndarray:
    return (np.arange(n) + 0.5) / n


def ramp_2d_bumps(ni=512, nj=256, length=1.0, height=0.5, ramp_start=0.2, angle_deg=15.0,
                  bumps=None) -> Su2Grid:
    """Compression ramp with its inclined surface perturbed by Hicks-Henne bumps:
    the wall point at ramp coordinate s = (x - ramp_start) / (length - ramp_start)
    moves by d(s) = sum_k bumps[k] hicks_henne(s, peak_k) (metres) along the
    ramp's normal, and every grid point above it by d(s) (1 - eta), eta = j / nj,
    so the displacement fades to zero at the top boundary.  Peaks are spread
    evenly over the ramp (ramp_bump_peaks); bumps=None gives ramp_2d."""
    g = ramp_2d(ni, nj, length, height, ramp_start, angle_deg)
    if bumps is None:
        return g
    bumps = np.asarray(bumps, np.float64)
    x = np.linspace(0.0, length, ni + 1)
    sc = (x - ramp_start) / (length - ramp_start)
    d = np.zeros(ni + 1)
    on = sc > 0.0
    for a, pk in zip(bumps, ramp_bump_peaks(len(bumps))):
        d[on] += a * hicks_henne(sc[on], pk)
    th = math.radians(angle_deg)
    nx, ny = -math.sin(th), math.cos(th)
    eta = np.arange(nj + 1) / nj
    D = d[:, None] * (1.0 - eta[None, :])  # (ni+1, nj+1)
    xyz = g.xyz.copy()
    vid = np.arange((ni + 1) * (nj + 1)).reshape(nj + 1, ni + 1).T  # vertex id = i + (ni+1) j
    xyz[vid.reshape(-1), 0] += (D * nx).reshape(-1)
    xyz[vid.reshape(-1), 1] += (D * ny).reshape(-1)
    g.xyz = xyz
    return g


def stretched_spacing(n: int, total: float, first: float, ratio: float) -> np.ndarray:
    """Wall-normal node positions: geometric growth ``ratio`` from ``first``,
    capped at the uniform spacing that fills ``total`` with the remaining cells.
    (Pure geometric growth 1e-5 * 1.05^j over 256 cells would reach ~53 m.)"""
    best = None
    for m in range(n + 1):
        grown = first * (ratio ** np.arange(m))
        s = grown.sum()
        if m < n:
            h = (total - s) / (n - m)
            if h >= (grown[-1] if m else first):
                best = np.concatenate([grown, np.full(n - m, h)])
    if best is None:
        raise ValueError("stretching cannot fill the domain")
    y = np.concatenate([[0.0], np.cumsum(best)])
    y[-1] = total
    return y


def flat_plate_2d(ni=512, nj=256, x0=-0.05, x1=1.0, height=0.4, first=1e-5, ratio=1.05) -> Su2Grid:
    """Flat plate: uniform in x over [x0, x1]; wall-normal stretching from the
    plate.  Markers: ``inflow``, ``outflow``, ``top``, ``slip`` (bottom, x<0),
    ``wall`` (bottom, x>=0)."""
    x = np.linspace(x0, x1, ni + 1)
    y = stretched_spacing(nj, height, first, ratio)
    X, Y = np.meshgrid(x, y, indexing="ij")
    g = structured_2d(X, Y, bottom_tags=lambda i: "slip" if x[i] < 0.0 - 1e-12 else "wall")
    rename = {"west": "inflow", "east": "outflow", "north": "top", "slip": "slip", "wall": "wall"}
    g.markers = {rename[k]: v for k, v in g.markers.items()}
    return g


def box_3d(nx: int, ny: int | None = None, nz: int | None = None, lx=1.0, ly=1.0, lz=1.0) -> Su2Grid:
    """Hexahedra on a uniform box; vertex id = i + (nx+1)(j + (ny+1) k),
    cell id = i + nx (j + ny k).  Markers ``west``/``east`` (x), ``south``/
    ``north`` (y), ``bottom``/``top`` (z), as in the reference's cube.su2."""
    ny = ny or nx
    nz = nz or nx
    vx, vy, vz = nx + 1, ny + 1, nz + 1
    xs, ys, zs = np.linspace(0, lx, vx), np.linspace(0, ly, vy), np.linspace(0, lz, vz)
    Z, Yy, Xx = np.meshgrid(zs, ys, xs, indexing="ij")
    xyz = np.stack([Xx.reshape(-1), Yy.reshape(-1), Z.reshape(-1)], 1)
    vid = lambda i, j, k: i + vx * (j + vy * k)  # noqa: E731
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.reshape(-1), j.reshape(-1), k.reshape(-1)
    conn = np.stack([vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
                     vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1),
                     vid(i, j + 1, k + 1)], 1).astype(np.int64)
    # boundary quads
    a, b = np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")
    a, b = a.reshape(-1), b.reshape(-1)
    west = np.stack([vid(0, a, b), vid(0, a + 1, b), vid(0, a + 1, b + 1), vid(0, a, b + 1)], 1)
    east = np.stack([vid(nx, a, b), vid(nx, a + 1, b), vid(nx, a + 1, b + 1), vid(nx, a, b + 1)], 1)
    a, b = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    a, b = a.reshape(-1), b.reshape(-1)
    south = np.stack([vid(a, 0, b), vid(a + 1, 0, b), vid(a + 1, 0, b + 1), vid(a, 0, b + 1)], 1)
    north = np.stack([vid(a, ny, b), vid(a + 1, ny, b), vid(a + 1, ny, b + 1), vid(a, ny, b + 1)], 1)
    a, b = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    a, b = a.reshape(-1), b.reshape(-1)
    bottom = np.stack([vid(a, b, 0), vid(a + 1, b, 0), vid(a + 1, b + 1, 0), vid(a, b + 1, 0)], 1)
    top = np.stack([vid(a, b, nz), vid(a + 1, b, nz), vid(a + 1, b + 1, nz), vid(a, b + 1, nz)], 1)
    markers = _markers_from_lists({"west": (VTK_QUAD, west), "east": (VTK_QUAD, east),
                                   "south": (VTK_QUAD, south), "north": (VTK_QUAD, north),
                                   "bottom": (VTK_QUAD, bottom), "top": (VTK_QUAD, top)})
    n = nx * ny * nz
    return Su2Grid(3, xyz, np.full(n, VTK_HEX, np.int32), np.arange(0, 8 * n + 1, 8, dtype=np.int64),
                   conn.reshape(-1), markers)


def unit_cube_3x3x3() -> Su2Grid:
    """The reference's 3x3x3 hex test grid (src/grid/test/cube.su2) in [0,1]^3."""
    return box_3d(3)


# ---------------------------------------------------------------------------
# config.json documents (the keys prep.py writes; prep.py:1134-1175)
# ---------------------------------------------------------------------------

def ideal_gas(R=287.0) -> dict:
    """IdealGas(R): Cv = 5/2 R, Cp = 7/2 R, gamma = Cp/Cv (gas_model.h:51-56)."""
    Cv, Cp = 5.0 / 2.0 * R, 7.0 / 2.0 * R
    return {"type": "ideal_gas", "R": R, "Cv": Cv, "Cp": Cp, "gamma": Cp / Cv}


def flow_state(gas: dict, T: float, p: float, vx=0.0, vy=0.0, vz=0.0) -> dict:
    """A prep FlowState as_dict (ibis_py_utils.py:32-37); rho and energy from p, T."""
    return {"p": p, "T": T, "rho": p / (gas["R"] * T), "energy": gas["Cv"] * T,
            "vx": vx, "vy": vy, "vz": vz}


def bc(pre_reconstruction, pre_viscous_grad=(), post_convective_flux=(), ghost_cells=True) -> dict:
    return {"pre_reconstruction": list(pre_reconstruction),
            "post_convective_flux": list(post_convective_flux),
            "pre_viscous_grad": list(pre_viscous_grad), "ghost_cells": ghost_cells}


# prep.py:541-617
def supersonic_inflow(fs: dict) -> dict:
    return bc([{"type": "flow_state_copy", "flow_state": fs}])


def supersonic_outflow() -> dict:
    return bc([{"type": "internal_copy"}])


def slip_wall() -> dict:
    return bc([{"type": "internal_copy_reflect_normal"}])


def adiabatic_no_slip_wall() -> dict:
    return bc([{"type": "internal_copy_reflect_normal"}], [{"type": "internal_vel_copy_reflect"}])


def fixed_temperature_no_slip_wall(T: float) -> dict:
    return bc([{"type": "internal_copy_reflect_normal"}],
              [{"type": "internal_vel_copy_reflect"}, {"type": "fix_temperature", "temperature": T}])


def subsonic_inflow(fs: dict) -> dict:
    return bc([{"type": "subsonic_inflow", "flow_state": fs}])


def subsonic_outflow(p: float) -> dict:
    return bc([{"type": "subsonic_outflow", "pressure": p}])


def constant_flux(fs: dict) -> dict:
    return bc([{"type": "flow_state_copy", "flow_state": fs}],
              post_convective_flux=[{"type": "constant_flux", "flow_state": fs}])


def boundary_layer_inflow(height, velocity_profile, temperature_profile, pressure: float) -> dict:
    """prep.py:549-556: ghosts take vx(y) and T(y) from natural cubic splines over
    the wall-normal coordinate (at least 4 points), p fixed, vy = vz = 0."""
    return bc([{"type": "boundary_layer_profile",
                "profile": {"height": list(map(float, height)), "v": list(map(float, velocity_profile)),
                            "T": list(map(float, temperature_profile)), "p": float(pressure)}}])


def periodic(partner: str, offset) -> dict:
    """Periodic ghost copy from the matching cell across the domain.  An
    extension: the reference has no periodic boundary action."""
    return bc([{"type": "periodic_copy", "partner": partner, "offset": list(map(float, offset))}])


SSP_RK3 = {"a": [[1.0], [0.25, 0.25]], "b": [1 / 6, 1 / 6, 2 / 3], "c": [1.0, 0.5]}  # prep.py:852-853


def make_config(dim, boundaries, *, flux="hanel", ldfss_delta=2.0, order=2,
                limiter="barth_jespersen", epsilon=1e-25, thermo="rho_u", viscous=False,
                signal_factor=4.0, gas=None, mu_0=1.716e-5, T_0=273.0, T_s=110.0, Pr=0.72,
                solver=None) -> dict:
    """A config.json document with the reference's defaults
    (share/defaults/{convective_flux,barth_jespersen,viscous_flux,runge_kutta}.json)."""
    gas = gas or ideal_gas()
    fc = {"type": flux}
    if flux == "ldfss2":
        fc["delta"] = ldfss_delta
    lim = {"type": limiter}
    if limiter == "barth_jespersen":
        lim["epsilon"] = epsilon
    return {
        "convective_flux": {"flux_calculator": fc, "reconstruction_order": order,
                            "limiter": lim, "thermo_interpolator": thermo},
        "viscous_flux": {"enabled": viscous, "signal_factor": signal_factor},
        "solver": solver or runge_kutta(),
        "grid": {"boundaries": copy.deepcopy(boundaries), "dimensions": dim,
                 "motion": {"enabled": False}},
        "gas_model": gas,
        "transport_properties": {
            "viscosity": {"type": "sutherland", "mu_0": mu_0, "T_0": T_0, "T_s": T_s},
            "thermal_conductivity": {"type": "constant_prandtl_number", "Pr": Pr}},
        "io": {"flow_format": "native_binary"},
    }


def runge_kutta(cfl=0.5, max_step=2000, max_time=1e30, plot_frequency=-1.0, dt_init=-1.0,
                tableau=SSP_RK3, print_frequency=100, plot_every_n_steps=-1, residual_frequency=-1.0,
                residuals_every_n_steps=-1) -> dict:
    """RungeKutta solver block (prep.py:862-903); plot_frequency <= 0 leaves dt unclipped."""
    return {"name": "runge_kutta", "cfl": {"type": "constant", "value": cfl}, "max_time": max_time,
            "max_step": max_step, "print_frequency": print_frequency, "plot_frequency": plot_frequency,
            "plot_every_n_steps": plot_every_n_steps, "dt_init": dt_init, "butcher_tableau": tableau,
            "residual_frequency": residual_frequency, "residuals_every_n_steps": residuals_every_n_steps}


def write_case(directory, grid, config, T, p, vx, vy, vz=None):
    """An ibis case directory as the prep step leaves it: config/config.json,
    io/grid/0000/block_0000.su2 and the initial flow io/flow/0000 (T, p, vx, vy[,
    vz] and meta_data.json) in the config's native flow format."""
    os.makedirs(os.path.join(directory, "config"), exist_ok=True)
    os.makedirs(os.path.join(directory, "io", "grid", "0000"), exist_ok=True)
    flow = os.path.join(directory, "io", "flow", "0000")
    os.makedirs(flow, exist_ok=True)
    with open(os.path.join(directory, "config", "config.json"), "w") as f:
        f.write(to_json(config))
    grid.write(os.path.join(directory, "io", "grid", "0000", "block_0000.su2"))
    binary = config["io"]["flow_format"] == "native_binary"
    fields = {"T": T, "p": p, "vx": vx, "vy": vy}
    if vz is not None:
        fields["vz"] = vz
    for name, arr in fields.items():
        arr = np.ascontiguousarray(arr, np.float64)
        if binary:
            arr.tofile(os.path.join(flow, name))
        else:
            with open(os.path.join(flow, name), "w") as f:
                f.write("".join(f"{x:.16f}\n" for x in arr))
    with open(os.path.join(flow, "meta_data.json"), "w") as f:
        json.dump({"time": 0.0}, f, indent=4)


def steady_state(cfl=None, max_steps=100, tolerance=1e-10, max_iters=30, tol=1e-2,
                 linear_solver=None) -> dict:
    """SteadyState solver block (prep.py:957-985) with a GMRES linear solver."""
    return {"name": "steady_state",
            "cfl": cfl or {"type": "constant", "value": 0.5},
            "max_steps": max_steps, "print_frequency": 10, "plot_frequency": 10,
            "diagnostics_frequency": 1, "tolerance": tolerance,
            "linear_solver": linear_solver or {"type": "gmres", "max_iters": max_iters, "tol": tol}}


def to_json(config: dict) -> str:
    return json.dumps(config, indent=2, sort_keys=True)


# ---------------------------------------------------------------------------
# benchmark cases
# ---------------------------------------------------------------------------

def mach_state(gas: dict, mach: float, T: float, p: float, angle_deg: float = 0.0) -> dict:
    a = math.sqrt(gas["gamma"] * gas["R"] * T)
    u = mach * a
    th = math.radians(angle_deg)
    return flow_state(gas, T, p, u * math.cos(th), u * math.sin(th))


def ramp_case(ni=256, nj=128, mach=2.0, T=300.0, p=101325.0, angle_deg=15.0, **kw):
    """2-D Euler compression ramp, Mach 2 at p=101325 Pa, T=300 K; supersonic
    in/outflow, slip wall below and above.  Returns (grid, config, inflow)."""
    gas = ideal_gas(287.0)
    inflow = mach_state(gas, mach, T, p)
    grid = ramp_2d(ni, nj, angle_deg=angle_deg)
    bnds = {"inflow": supersonic_inflow(inflow), "outflow": supersonic_outflow(),
            "wall": slip_wall(), "top": slip_wall()}
    return grid, make_config(2, bnds, gas=gas, **kw), inflow


def ramp_ensemble(n_cases=64, seed=0, smallest=(64, 32), largest=(512, 256), mach=(1.5, 4.0),
                  angle_deg=(5.0, 20.0), T=(200.0, 400.0), p=101325.0, **kw):
    """Independent compression-ramp cases for a batched ensemble: grid sizes
    log-uniform between ``smallest`` and ``largest`` cells (aspect 2:1 kept),
    inflow Mach, ramp angle and inflow temperature uniform in the given ranges,
    all drawn from ``seed``.  Returns a list of (grid, config, inflow, params)."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(smallest[0]), math.log(largest[0])
    out = []
    for _ in range(n_cases):
        ni = int(round(math.exp(rng.uniform(lo, hi)) / 2.0)) * 2
        nj = ni * smallest[1] // smallest[0]
        prm = {"ni": ni, "nj": nj, "mach": float(rng.uniform(*mach)),
               "angle_deg": float(rng.uniform(*angle_deg)), "T": float(rng.uniform(*T))}
        g, c, inf = ramp_case(ni, nj, mach=prm["mach"], T=prm["T"], p=p, angle_deg=prm["angle_deg"], **kw)
        out.append((g, c, inf, prm))
    return out


def ramp_bump_case(ni=512, nj=256, mach=2.0, T=300.0, p=101325.0, angle_deg=15.0, bumps=None, **kw):
    """The steady-state (JFNK and adjoint) case's geometry: the compression ramp of ramp_case with its
    surface perturbed by Hicks-Henne bumps (ramp_2d_bumps).  Returns (grid, config, inflow)."""
    gas = ideal_gas(287.0)
    inflow = mach_state(gas, mach, T, p)
    grid = ramp_2d_bumps(ni, nj, angle_deg=angle_deg, bumps=bumps)
    bnds = {"inflow": supersonic_inflow(inflow), "outflow": supersonic_outflow(),
            "wall": slip_wall(), "top": slip_wall()}
    return grid, make_config(2, bnds, gas=gas, **kw), inflow


def flat_plate_case(ni=512, nj=256, mach=2.0, T=220.0, Re_per_m=1e5, Pr=0.71, **kw):
    """2-D laminar flat plate: Sutherland air, Pr=0.71, Mach 2 at T=220 K with
    density chosen for Re=1e5 per metre; adiabatic no-slip wall from x=0."""
    gas = ideal_gas(287.0)
    mu = 1.716e-5 * (T / 273.0) ** 1.5 * (273.0 + 110.0) / (T + 110.0)
    u = mach * math.sqrt(gas["gamma"] * gas["R"] * T)
    rho = Re_per_m * mu / u
    p = rho * gas["R"] * T
    inflow = flow_state(gas, T, p, u, 0.0)
    grid = flat_plate_2d(ni, nj)
    bnds = {"inflow": supersonic_inflow(inflow), "outflow": supersonic_outflow(),
            "top": supersonic_outflow(), "slip": slip_wall(), "wall": adiabatic_no_slip_wall()}
    return grid, make_config(2, bnds, gas=gas, viscous=True, Pr=Pr, **kw), inflow


def box_case(n=64, ny=None, nz=None, **kw):
    """3-D periodic unit box of n x ny x nz cells (ny, nz default to n), ideal gas
    gamma=1.4 with R=1 (so T = p/rho)."""
    gas = ideal_gas(1.0)
    bnds = {"west": periodic("east", (1, 0, 0)), "east": periodic("west", (-1, 0, 0)),
            "south": periodic("north", (0, 1, 0)), "north": periodic("south", (0, -1, 0)),
            "bottom": periodic("top", (0, 0, 1)), "top": periodic("bottom", (0, 0, -1))}
    return box_3d(n, ny, nz), make_config(3, bnds, gas=gas, **kw)


def box_initial_condition(n: int, gas: dict, seed=0, kmax=4, amp=0.05, mach_rms=0.3):
    """rho=1, p=1 plus the sum of Fourier modes 0<|k|<=kmax with seeded random
    phases at ``amp`` relative amplitude; a divergence-free velocity (curl of a
    random vector potential A_c = sum_k cos(2 pi k.x + phi_kc)/|k|^2) scaled to
    rms Mach ``mach_rms``.  Sampled at the cell centres x = (i + 1/2)/n by
    inverse FFT.  Returns (T, p, vx, vy, vz) in cell order i + n (j + n k)."""
    rng = np.random.default_rng(seed)
    ks = [(a, b, d) for a in range(-kmax, kmax + 1) for b in range(-kmax, kmax + 1)
          for d in range(-kmax, kmax + 1) if 0 < a * a + b * b + d * d <= kmax * kmax]
    spec = np.zeros((5, n, n, n), np.complex128)  # rho, p, ux, uy, uz; axes (k_z, k_y, k_x)
    for (a, b, d) in ks:
        ph = rng.uniform(0, 2 * np.pi, 5)
        shift = np.exp(1j * np.pi * (a + b + d) / n)  # samples at (j + 1/2)/n
        idx = (d % n, b % n, a % n)
        spec[0][idx] += np.exp(1j * ph[0]) * shift
        spec[1][idx] += np.exp(1j * ph[1]) * shift
        # sin(theta + phi) = Re(-i e^{i(theta + phi)}); dA_c/dx_j = -2 pi k_j sin(...)/|k|^2
        k = (a, b, d)
        k2 = float(a * a + b * b + d * d)
        e = [-1j * np.exp(1j * ph[2 + c]) * shift for c in range(3)]
        dA = lambda c, j: -2 * np.pi * k[j] * e[c] / k2  # noqa: E731
        spec[2][idx] += dA(2, 1) - dA(1, 2)
        spec[3][idx] += dA(0, 2) - dA(2, 0)
        spec[4][idx] += dA(1, 0) - dA(0, 1)
    fields = np.fft.ifftn(spec, axes=(1, 2, 3)).real * (n ** 3)
    rho_p, p_p, u = fields[0], fields[1], fields[2:5]
    rho = 1.0 + amp * rho_p / np.abs(rho_p).max()
    p = 1.0 + amp * p_p / np.abs(p_p).max()
    a_mean = math.sqrt(gas["gamma"] * gas["R"] * 1.0)
    u = u * (mach_rms * a_mean / math.sqrt((u ** 2).sum(0).mean()))
    T = p / (rho * gas["R"])
    f = lambda v: np.ascontiguousarray(v.reshape(-1))  # noqa: E731  (k slowest, i fastest)
    return f(T), f(p), f(u[0]), f(u[1]), f(u[2])
