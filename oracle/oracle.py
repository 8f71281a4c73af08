"""ORACLE — test infrastructure only.

ctypes wrapper of the CPU restatement of ibis's residual path (oracle_core.cpp).
Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, always as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP, no FMA contraction)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_longlong, C.c_void_p,
                                 C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_char_p,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_last_error.restype = C.c_char_p
        L.orc_last_error.argtypes = [C.c_void_p]
        L.orc_sizes.argtypes = [C.c_void_p, _lp]
        L.orc_connectivity.argtypes = [C.c_void_p, _lp, _lp, _lp, _ip, _lp, C.c_int]
        L.orc_ghosts.argtypes = [C.c_void_p, C.c_char_p, _lp, _lp, C.c_longlong]
        L.orc_geometry.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_lsq_r.argtypes = [C.c_void_p, _dp]
        L.orc_gradient.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_set_ic.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.c_void_p]
        L.orc_get_prims.argtypes = [C.c_void_p, _dp]
        L.orc_put_prims.argtypes = [C.c_void_p, _dp]
        L.orc_residual.argtypes = [C.c_void_p, _dp, C.c_int, C.c_void_p]
        L.orc_recon_dump.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_face_dump.argtypes = [C.c_void_p, _dp, C.c_void_p]
        L.orc_estimate_dt.restype = C.c_double
        L.orc_estimate_dt.argtypes = [C.c_void_p]
        L.orc_count_bad_cells.restype = C.c_longlong
        L.orc_count_bad_cells.argtypes = [C.c_void_p]
        L.orc_rk_initialise.argtypes = [C.c_void_p]
        L.orc_rk_steps.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_count_step_flops.argtypes = [C.c_void_p, _lp]
        L.orc_get_conserved.argtypes = [C.c_void_p, _dp]
        L.orc_steady_initialise.argtypes = [C.c_void_p]
        L.orc_jvp.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int]
        L.orc_geometry_jvp.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int]
        L.orc_flow_state_jvp.argtypes = [C.c_void_p, C.c_char_p, _dp, _dp, C.c_int]
        L.orc_steady_rhs.argtypes = [C.c_void_p, _dp]
        L.orc_steady_steps.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_steady_conserved.argtypes = [C.c_void_p, _dp]
        L.orc_dense_gmres.argtypes = [C.c_int, _dp, _dp, _dp, C.c_int, C.c_double, C.c_void_p,
                                      C.c_int, C.c_double, _dp]
        L.orc_cubic_spline.argtypes = [C.c_int, _dp, _dp, C.c_int, _dp, _dp]
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


class Oracle:
    """One ibis simulation restated on the CPU.

    ``grid`` is an ``ibis_gb300.grids.Su2Grid`` or a path to an SU2 file;
    ``kind`` is ``"real"`` (Sim<double>) or ``"dual"`` (the steady solver's
    dual-number linearisation)."""

    def __init__(self, config: dict, grid, kind: str = "real"):
        L = lib()
        err = C.create_string_buffer(1024)
        text = json.dumps(config).encode()
        k = 0 if kind == "real" else 1
        self._keep = []
        if isinstance(grid, (str, os.PathLike)):
            h = L.orc_create(text, os.fspath(grid).encode(), k, 0, 0, None, 0, None, None, None, 0,
                             b"", None, None, None, None, err, 1024)
        else:
            names, m_off, e_types, e_off, e_conn = grid.marker_arrays()
            arrs = [np.ascontiguousarray(grid.xyz, np.float64),
                    np.ascontiguousarray(grid.cell_types, np.int32),
                    np.ascontiguousarray(grid.cell_offsets, np.int64),
                    np.ascontiguousarray(grid.cell_conn, np.int64), m_off, e_types, e_off, e_conn]
            self._keep = arrs
            p = [a.ctypes.data for a in arrs]
            h = L.orc_create(text, None, k, grid.dim, grid.xyz.shape[0], p[0], grid.num_cells, p[1],
                             p[2], p[3], len(grid.markers), names.encode(), p[4], p[5], p[6], p[7],
                             err, 1024)
        if not h:
            raise RuntimeError("oracle: " + err.value.decode())
        self.h = h
        self.kind = kind
        s = np.zeros(5, np.int64)
        self._check(L.orc_sizes(h, s))
        self.N, self.G, self.F, self.dim, self.max_faces = (int(x) for x in s)
        self.nc = self.dim + 2

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + lib().orc_last_error(self.h).decode())

    # --- grid --------------------------------------------------------------
    def connectivity(self):
        mf = self.max_faces
        left, right = np.zeros(self.F, np.int64), np.zeros(self.F, np.int64)
        cf, nb = np.zeros(self.N * mf, np.int64), np.zeros(self.N * mf, np.int64)
        os_ = np.zeros(self.N * mf, np.int32)
        self._check(lib().orc_connectivity(self.h, left, right, cf, os_, nb, mf))
        return dict(left=left, right=right, cell_faces=cf.reshape(self.N, mf),
                    outsigns=os_.reshape(self.N, mf), neighbours=nb.reshape(self.N, mf))

    def ghosts(self, tag: str):
        cap = self.G + self.F
        ids, faces = np.zeros(cap, np.int64), np.zeros(cap, np.int64)
        n = lib().orc_ghosts(self.h, tag.encode(), ids, faces, cap)
        if n < 0:
            self._check(-1)
        return ids[:n], faces[:n]

    def geometry(self):
        face = np.zeros(13 * self.F)
        cell = np.zeros(4 * (self.N + self.G))
        self._check(lib().orc_geometry(self.h, face, cell))
        face = face.reshape(13, self.F)
        cell = cell.reshape(4, self.N + self.G)
        return dict(normal=face[0:3], tan1=face[3:6], tan2=face[6:9], centre=face[9:12],
                    area=face[12], centroid=cell[0:3], volume=cell[3])

    def lsq_r(self):
        r = np.zeros(self.N * 6)
        self._check(lib().orc_lsq_r(self.h, r))
        return r.reshape(self.N, 6)

    def gradient(self, values):
        g = np.zeros(self.N * 3)
        self._check(lib().orc_gradient(self.h, np.ascontiguousarray(values, np.float64), g))
        return g.reshape(self.N, 3)

    # --- flow --------------------------------------------------------------
    def set_initial_condition(self, T, p, vx, vy, vz=None):
        arrs = [np.ascontiguousarray(a, np.float64) for a in (T, p, vx, vy)]
        vz = None if vz is None else np.ascontiguousarray(vz, np.float64)
        self._check(lib().orc_set_ic(self.h, *arrs, None if vz is None else vz.ctypes.data))

    def primitives(self):
        out = np.zeros(7 * (self.N + self.G))
        self._check(lib().orc_get_prims(self.h, out))
        return out.reshape(7, self.N + self.G)

    def put_primitives(self, prims):
        self._check(lib().orc_put_prims(self.h, np.ascontiguousarray(prims, np.float64).reshape(-1)))

    def residual(self, allow_reconstruction=True, branches=False):
        d = np.zeros(self.N * self.nc)
        br = np.zeros(self.N * 5, np.uint32) if branches else None
        self._check(lib().orc_residual(self.h, d, int(allow_reconstruction),
                                       None if br is None else br.ctypes.data))
        d = d.reshape(self.N, self.nc)
        return (d, br.reshape(self.N, 5)) if branches else d

    def recon_dump(self):
        lim, grad = np.zeros(self.N * 7), np.zeros(self.N * 21)
        self._check(lib().orc_recon_dump(self.h, lim, grad))
        return lim.reshape(self.N, 7), grad.reshape(self.N, 7, 3)

    def face_dump(self):
        flux, ffs = np.zeros(self.F * self.nc), np.zeros(7 * self.F)
        self._check(lib().orc_face_dump(self.h, flux, ffs.ctypes.data))
        return flux.reshape(self.F, self.nc), ffs.reshape(7, self.F)

    def estimate_dt(self):
        return lib().orc_estimate_dt(self.h)

    def count_bad_cells(self):
        return lib().orc_count_bad_cells(self.h)

    def rk_initialise(self):
        self._check(lib().orc_rk_initialise(self.h))

    def rk_steps(self, n):
        out = np.zeros(9)
        self._check(lib().orc_rk_steps(self.h, int(n), out))
        return dict(t=out[0], dt=out[1], stable_dt=out[2], norms=out[3:9])

    def count_step_flops(self):
        """Exact floating-point operation counts of one Runge-Kutta step (with its
        estimate_dt) from the current initial state: the restatement instantiated
        on a counting scalar.  Returns add, mul, div, sqrt, pow (arithmetic) and
        other (abs/min/max/floor/copysign) totals over the grid."""
        out = np.zeros(6, np.int64)
        self._check(lib().orc_count_step_flops(self.h, out))
        return dict(zip(("add", "mul", "div", "sqrt", "pow", "other"), (int(x) for x in out)))

    def conserved(self):
        out = np.zeros(self.N * self.nc)
        if self.kind == "real":
            self._check(lib().orc_get_conserved(self.h, out))
        else:
            self._check(lib().orc_steady_conserved(self.h, out))
        return out.reshape(self.N, self.nc)

    # --- steady / dual ------------------------------------------------------
    def steady_initialise(self):
        self._check(lib().orc_steady_initialise(self.h))

    def jvp(self, v, dt_star=0.0, allow_reconstruction=True):
        """(I/dt* - dR/dU) v via the reference's dual numbers; dt_star <= 0 drops
        the 1/dt* term (returns -dR/dU v)."""
        out = np.zeros(self.N * self.nc)
        self._check(lib().orc_jvp(self.h, np.ascontiguousarray(v, np.float64).reshape(-1), out,
                                  float(dt_star), int(allow_reconstruction)))
        return out

    def geometry_jvp(self, dface, dcell, allow_reconstruction=True):
        """dR/dgeometry . (dface, dcell) at the current steady state by the reference's
        dual numbers seeded in the geometry (dface 13 x F, dcell 4 x (N+G), the
        layouts of the face / cell geometry dumps); returns N x n_conserved."""
        out = np.zeros(self.N * self.nc)
        self._check(lib().orc_geometry_jvp(self.h, np.ascontiguousarray(dface, np.float64).reshape(-1),
                                           np.ascontiguousarray(dcell, np.float64).reshape(-1), out,
                                           int(allow_reconstruction)))
        return out.reshape(self.N, self.nc)

    def flow_state_jvp(self, tag, dfs, allow_reconstruction=True):
        """dR/dfs . dfs at the current steady state by the reference's dual numbers
        seeded in boundary `tag`'s flow state (dfs: T, p, rho, energy, vx, vy, vz)
        on every action of it that carries one; returns N x n_conserved."""
        out = np.zeros(self.N * self.nc)
        self._check(lib().orc_flow_state_jvp(self.h, tag.encode(), np.ascontiguousarray(dfs, np.float64).reshape(7),
                                             out, int(allow_reconstruction)))
        return out.reshape(self.N, self.nc)

    def steady_rhs(self):
        out = np.zeros(self.N * self.nc)
        self._check(lib().orc_steady_rhs(self.h, out))
        return out

    def steady_steps(self, n):
        out = np.zeros(4 * n)
        self._check(lib().orc_steady_steps(self.h, int(n), out))
        return out.reshape(n, 4)


def dense_gmres(A, b, max_iters, tol, P=None, max_prec_iters=0, prec_tol=0.0):
    """The reference's GMRES (or FGMRES when P is given) on a small dense system."""
    A = np.ascontiguousarray(A, np.float64)
    n = A.shape[0]
    x = np.zeros(n)
    info = np.zeros(3)
    Pc = None if P is None else np.ascontiguousarray(P, np.float64)
    rc = lib().orc_dense_gmres(n, A.reshape(-1), np.ascontiguousarray(b, np.float64), x, max_iters,
                               tol, None if Pc is None else Pc.ctypes.data, max_prec_iters, prec_tol,
                               info)
    if rc != 0:
        raise RuntimeError("oracle gmres failed")
    return x, dict(success=bool(info[0]), n_iters=int(info[1]), residual=info[2])


def cubic_spline(x, y, q):
    """The boundary-layer profile's natural cubic spline through (x, y), evaluated at q."""
    x = np.ascontiguousarray(x, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    out = np.zeros(len(q))
    if lib().orc_cubic_spline(len(x), x, np.ascontiguousarray(y, np.float64), len(q), q, out) != 0:
        raise ValueError("cubic spline needs at least 4 points and as many y as x")
    return out


def num_threads() -> int:
    return lib().orc_num_threads()
