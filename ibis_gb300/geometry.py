"""The grid geometry the engine computes (face normals, tangents, centres and
areas; cell centroids and volumes; ghost centroids) restated on numpy arrays of
vertex coordinates, so that it can be evaluated on complex coordinates: the
complex step h of x + i h dx gives the exact directional derivative of every
geometric quantity along a vertex displacement dx.  Chained with the engine's
geometry adjoint (Simulation.geometry_adjoint) this is the derivative of an
objective with respect to vertex displacements, e.g. shape parameters.

The formulas follow the engine's mesh builder, which follows the reference:
Interfaces compute_centres / compute_areas / compute_orientations
(interface.h:180-323), Cells centroids and volumes (cell.h:228-300, geom.h:66-83)
and the ghost centroids mirrored through the face centre (grid.h:364-403)."""
from __future__ import annotations

import numpy as np

# VTK cell type codes of the 2-D elements whose volume is an area
_VTK_TRI, _VTK_QUAD = 5, 9


def _tri_area(a, b, c):
    ab, ac = b - a, c - a
    cx = ab[..., 1] * ac[..., 2] - ab[..., 2] * ac[..., 1]
    cy = ab[..., 2] * ac[..., 0] - ab[..., 0] * ac[..., 2]
    cz = ab[..., 0] * ac[..., 1] - ab[..., 1] * ac[..., 0]
    return 0.5 * np.sqrt(cx * cx + cy * cy + cz * cz)


class GridTopology:
    """What the geometry needs besides vertex coordinates, from a Simulation's
    dumps (reference numbering) and its Su2Grid (cell vertex lists)."""

    def __init__(self, sim, grid):
        self.dim = sim.dim
        self.N, self.G, self.F = sim.num_cells, sim.num_ghost_cells, sim.num_faces
        self.face_vertices = sim.dump("face_vertices")
        self.left, self.right = sim.dump("left"), sim.dump("right")
        self.ghost_face = sim.dump("ghost_face")
        self.cell_faces = sim.dump("cell_faces")
        self.outsigns = sim.dump("outsigns")
        self.cell_types = np.asarray(grid.cell_types)
        self.cell_offsets = np.asarray(grid.cell_offsets)
        self.cell_conn = np.asarray(grid.cell_conn)

    def geometry(self, xyz: np.ndarray):
        """(face (13, F): n, t1, t2, centre, area; cell (4, N+G): centroid, volume),
        the layouts of the face / cell geometry dumps, for vertex coordinates xyz
        (num_vertices, 3), real or complex."""
        X = np.asarray(xyz)
        dt = np.result_type(X.dtype, np.float64)
        N, G, F = self.N, self.G, self.F
        fv = self.face_vertices
        nv = (fv >= 0).sum(axis=1)
        P = [X[np.where(fv[:, k] >= 0, fv[:, k], 0)] for k in range(4)]
        fc = sum(np.where((fv[:, k] >= 0)[:, None], P[k], 0) for k in range(4)) / nv[:, None]
        line = nv == 2
        tri = nv == 3
        e = P[1] - P[0]
        area = np.where(line, np.sqrt((e * e).sum(axis=1)),
                        np.where(tri, _tri_area(P[0], P[1], P[2]),
                                 _tri_area(P[0], P[1], P[2]) + _tri_area(P[0], P[2], P[3])))
        t1 = e / np.sqrt((e * e).sum(axis=1))[:, None]
        s = P[2] - P[0]
        proj = (t1 * s).sum(axis=1)
        p = s - proj[:, None] * t1
        with np.errstate(invalid="ignore", divide="ignore"):
            t2s = p / np.sqrt((p * p).sum(axis=1))[:, None]
        t2 = np.where(line[:, None], np.array([0.0, 0.0, 1.0]), t2s)
        n = np.stack([t1[:, 1] * t2[:, 2] - t1[:, 2] * t2[:, 1],
                      t1[:, 2] * t2[:, 0] - t1[:, 0] * t2[:, 2],
                      t1[:, 0] * t2[:, 1] - t1[:, 1] * t2[:, 0]], axis=1)
        face = np.concatenate([n.T, t1.T, t2.T, fc.T, area[None, :]]).astype(dt)
        # cells
        off, conn, types = self.cell_offsets, self.cell_conn, self.cell_types
        cnt = off[1:] - off[:-1]
        owner = np.repeat(np.arange(N), cnt)
        cc = np.zeros((N + G, 3), dt)
        for d in range(3):
            cc[:N, d] = np.bincount(owner, weights=X[conn, d].real, minlength=N) / cnt
            if np.iscomplexobj(X):
                cc[:N, d] = cc[:N, d] + 1j * np.bincount(owner, weights=X[conn, d].imag, minlength=N) / cnt
        vol = np.zeros(N + G, dt)
        v0, v1, v2 = X[conn[off[:-1]]], X[conn[off[:-1] + 1]], X[conn[off[:-1] + 2]]
        if self.dim == 2:
            v3 = X[conn[np.minimum(off[:-1] + 3, len(conn) - 1)]]
            vol[:N] = np.where(types == _VTK_QUAD, _tri_area(v0, v1, v2) + _tri_area(v0, v2, v3),
                               _tri_area(v0, v1, v2))
        else:
            cf, osg = self.cell_faces, self.outsigns
            ok = cf >= 0
            fcf = np.where(ok, cf, 0)
            dot = sum(fc[fcf, d] * osg * n[fcf, d] for d in range(3)) * area[fcf]
            vol[:N] = np.where(ok, dot, 0).sum(axis=1) / 3.0
        # ghost centroids: the valid cell's centroid mirrored through the face centre
        f = self.ghost_face
        valid = np.where(self.left[f] < N, self.left[f], self.right[f])
        ghost = np.where(self.left[f] < N, self.right[f], self.left[f])
        cc[ghost] = 2.0 * fc[f] - cc[valid]
        cell = np.concatenate([cc.T, vol[None, :]])
        return face, cell

    def directional_derivative(self, xyz: np.ndarray, dxyz: np.ndarray, h: float = 1e-30):
        """d(face, cell)/d(xyz) . dxyz by the complex step."""
        face, cell = self.geometry(np.asarray(xyz, np.float64) + 1j * h * np.asarray(dxyz, np.float64))
        return face.imag / h, cell.imag / h
