"""Python face of the GB300 residual engine, mirroring ibis's host interface.

``Simulation`` bundles what ibis keeps in ``Sim<T>`` (src/simulation/simulation/
simulation.h:13-23: GridBlock, FiniteVolume, IdealGas, TransportProperties) plus
the RungeKutta driver state, and exposes the same operations under the
reference's names:

* ``compute_dudt``     FiniteVolume<T>::compute_dudt   (finite_volume.cpp:56-96)
* ``estimate_dt``      FiniteVolume<T>::estimate_dt    (finite_volume.cpp:130-184)
* ``count_bad_cells``  FiniteVolume<T>::count_bad_cells (finite_volume.cpp:257-270)
* ``take_steps``       RungeKutta::take_step, n times  (runge_kutta.cpp:131-203)
* ``L2_norms``         ConservedQuantities::L2_norms of the first stage
                       (conserved_quantities.cpp:40-69)

Every call goes through the C ABI of libibisgb.so (include/ibisgb.h); arrays
are numpy (host) or torch CUDA tensors (device, zero copy).
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _lib
from ._lib import PRECISION, NewtonStatus, RkStatus, Sizes, check

DUMPS = {"left": (0, np.int64), "right": (1, np.int64), "cell_faces": (2, np.int64),
         "outsigns": (3, np.int32), "neighbours": (4, np.int64), "ghost_source": (5, np.int64),
         "face_geometry": (6, np.float64), "cell_geometry": (7, np.float64),
         "limiter_branches": (8, np.uint32), "limiters": (9, np.float64),
         "face_flux": (10, np.float64), "ghost_face": (11, np.int64), "ghost_boundary": (12, np.int64),
         "face_flux_mixed": (13, np.float64), "cell_order": (14, np.int64), "face_order": (15, np.int64),
         "face_vertices": (16, np.int64)}


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def _stream_arg(stream):
    """A torch stream as the C ABI's stream argument.  The C ABI reads NULL as
    "the context's own stream", so torch's legacy default stream (handle 0) is
    passed as cudaStreamLegacy (handle 1) to keep the call ordered with it."""
    if stream is None:
        return None
    return C.c_void_p(stream.cuda_stream or 1)


class Simulation:
    """One ibis simulation (one grid block) on the current CUDA device.

    ``config`` is a config.json document (dict or JSON text, as written by
    ibis's prep step); ``grid`` is an ``ibis_gb300.grids.Su2Grid`` or the path
    of an SU2 file."""

    def __init__(self, config, grid):
        L = _lib.load()
        text = config if isinstance(config, str) else json.dumps(config)
        self.config = json.loads(text)
        h = C.c_void_p()
        if isinstance(grid, (str, os.PathLike)):
            rc = L.ibisgb_create(text.encode(), os.fspath(grid).encode(), C.byref(h))
        else:
            names, m_off, e_types, e_off, e_conn = grid.marker_arrays()
            xyz = np.ascontiguousarray(grid.xyz, np.float64)
            ct = np.ascontiguousarray(grid.cell_types, np.int32)
            co = np.ascontiguousarray(grid.cell_offsets, np.int64)
            cv = np.ascontiguousarray(grid.cell_conn, np.int64)
            rc = L.ibisgb_create_from_arrays(text.encode(), grid.dim, xyz.shape[0], _ptr(xyz),
                                             grid.num_cells, _ptr(ct), _ptr(co), _ptr(cv),
                                             len(grid.markers), names.encode(), _ptr(m_off),
                                             _ptr(e_types), _ptr(e_off), _ptr(e_conn), C.byref(h))
        check(rc, None)
        self._attach(h)

    def _attach(self, h):
        L = _lib.load()
        self._h = h
        s = Sizes()
        check(L.ibisgb_get_sizes(h, C.byref(s)), h)
        self.num_cells, self.num_ghost_cells, self.num_faces = s.num_cells, s.num_ghost_cells, s.num_faces
        self.dim, self.max_faces, self.n_conserved = s.dim, s.max_faces_per_cell, s.n_conserved
        self.num_boundaries = s.num_boundaries

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().ibisgb_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name, *args):
        check(getattr(_lib.load(), name)(self._h, *args), self._h)

    # ---------------------------------------------------------------- state
    def set_primitives(self, T, p, vx, vy, vz=None):
        """Initial condition of the valid cells (NativeBinaryInput::read + primatives_to_conserved)."""
        arrs = [np.ascontiguousarray(a, np.float64) for a in (T, p, vx, vy)]
        vz_a = None if vz is None else np.ascontiguousarray(vz, np.float64)
        for a in arrs + ([vz_a] if vz_a is not None else []):
            if a.shape != (self.num_cells,):
                raise ValueError(f"expected {self.num_cells} values per field")
        self._call("ibisgb_set_primitives", *[_ptr(a) for a in arrs],
                   None if vz_a is None else _ptr(vz_a))

    def primitives(self) -> dict:
        N = self.num_cells
        out = {k: np.empty(N) for k in ("rho", "p", "T", "e", "vx", "vy", "vz")}
        self._call("ibisgb_get_primitives", *[_ptr(out[k]) for k in ("rho", "p", "T", "e", "vx", "vy", "vz")])
        return out

    def conserved(self, out: np.ndarray | None = None) -> np.ndarray:
        """Conserved state (N, n_conserved); ``out`` may be a (pinned) host buffer."""
        if out is None:
            out = np.empty((self.num_cells, self.n_conserved))
        self._call("ibisgb_get_conserved", _ptr(out))
        return out

    def set_conserved(self, U: np.ndarray) -> None:
        """Replace the conserved state (N, n_conserved), e.g. from a pinned host buffer."""
        U = np.ascontiguousarray(U, np.float64)
        if U.shape != (self.num_cells, self.n_conserved):
            raise ValueError("U has the wrong shape")
        self._call("ibisgb_set_conserved", _ptr(U))

    def set_conserved_into(self, U, stream=None) -> None:
        """Replace the conserved state from a contiguous float64 CUDA tensor (N, n_conserved)."""
        if not (U.is_cuda and U.element_size() == 8 and U.is_contiguous()):
            raise ValueError("U must be a contiguous float64 CUDA tensor")
        if tuple(U.shape) != (self.num_cells, self.n_conserved):
            raise ValueError("U has the wrong shape")
        s = _stream_arg(stream)
        self._call("ibisgb_set_conserved_device", C.c_void_p(U.data_ptr()), s)

    def stream_handle(self) -> int:
        """The context's cudaStream_t as an integer (torch.cuda.ExternalStream(ptr))."""
        s = C.c_void_p()
        self._call("ibisgb_get_stream", C.byref(s))
        return s.value or 0

    def kernel_times(self, precision: str = "mixed", reps: int = 10) -> dict:
        """Mean device ms of the residual's kernels (CUDA events on the context stream)."""
        out = np.zeros(4)
        self._call("ibisgb_kernel_times", PRECISION[precision], int(reps), _ptr(out))
        return {"recon": out[0], "face": out[1], "update": out[2], "residual": out[3]}

    # ------------------------------------------------------------ autotuner
    @staticmethod
    def launch_variants() -> list:
        """The launch-variant table: (threads per block, minimum blocks per SM)."""
        L = _lib.load()
        n = C.c_int32()
        check(L.ibisgb_launch_variants(C.byref(n), None, None))
        th = np.zeros(n.value, np.int32)
        mb = np.zeros(n.value, np.int32)
        check(L.ibisgb_launch_variants(C.byref(n), _ptr(th), _ptr(mb)))
        return list(zip(th.tolist(), mb.tolist()))

    def autotune(self, precision: str = "mixed") -> dict:
        """Time every launch variant of the recon, face and update kernels on this
        grid and keep the fastest; returns the choice and the mean times (ms)."""
        nv = len(self.launch_variants())
        w = np.zeros(3, np.int32)
        t = np.zeros(3 * nv)
        self._call("ibisgb_autotune", PRECISION[precision], _ptr(w), _ptr(t))
        t = t.reshape(3, nv)
        return {"variants": dict(zip(("recon", "face", "update"), w.tolist())),
                "ms": {k: t[i].round(4).tolist() for i, k in enumerate(("recon", "face", "update"))}}

    def set_launch_variants(self, precision: str, recon: int, face: int, update: int) -> None:
        w = np.array([recon, face, update], np.int32)
        self._call("ibisgb_set_launch_variants", PRECISION[precision], _ptr(w))

    def set_fused(self, mode: int) -> None:
        """Fused stage on structured blocks: -1 autotuner decides, 0 off, 1 on."""
        self._call("ibisgb_set_fused", int(mode))

    def fused_info(self) -> dict:
        el, en = C.c_int32(), C.c_int32()
        t = np.zeros(2)
        why = C.create_string_buffer(256)
        self._call("ibisgb_fused_info", C.byref(el), C.byref(en), _ptr(t), why, 256)
        return {"eligible": bool(el.value), "enabled": bool(en.value), "fused_ms": t[0], "generic_ms": t[1],
                "reason": why.value.decode()}

    def set_fused_kind(self, kind: int, planes_per_cta: int = 0) -> None:
        """Kernel of the fused stage: -1 autotuner decides, 0 the tile kernel, 1 the
        plane-marching kernel (one 3-D block), with planes_per_cta planes per CTA
        (0: tuned)."""
        self._call("ibisgb_set_fused_kind", int(kind), int(planes_per_cta))

    def fused_kind(self) -> dict:
        el, on, kc = C.c_int32(), C.c_int32(), C.c_int32()
        t = np.zeros(2)
        why = C.create_string_buffer(256)
        self._call("ibisgb_fused_kind", C.byref(el), C.byref(on), C.byref(kc), _ptr(t), why, 256)
        return {"march_eligible": bool(el.value), "march": bool(on.value), "planes_per_cta": kc.value,
                "tile_ms": t[0], "march_ms": t[1], "reason": why.value.decode()}

    def set_cell_flux(self, mode: int) -> None:
        """Per-cell flux path of the mixed build: -1 autotuner decides, 0 off, 1 on."""
        self._call("ibisgb_set_cell_flux", int(mode))

    def cell_flux_info(self) -> dict:
        el, en, w = C.c_int32(), C.c_int32(), C.c_int32()
        t = np.zeros(2)
        self._call("ibisgb_cell_flux_info", C.byref(el), C.byref(en), C.byref(w), _ptr(t))
        return {"eligible": bool(el.value), "enabled": bool(en.value), "variant": w.value, "cell_ms": t[0],
                "generic_ms": t[1]}

    # ------------------------------------------------------------- residual
    def compute_dudt(self, precision: str = "f64") -> np.ndarray:
        """dU/dt of the valid cells, (N, n_conserved) in the reference's cell order."""
        out = np.empty((self.num_cells, self.n_conserved))
        self._call("ibisgb_residual", PRECISION[precision], _ptr(out))
        return out

    def compute_dudt_into(self, out, precision: str = "f64", stream=None):
        """As compute_dudt into a CUDA tensor of shape (N, n_conserved), float64."""
        if not (out.is_cuda and out.dtype.is_floating_point and out.element_size() == 8 and out.is_contiguous()):
            raise ValueError("out must be a contiguous float64 CUDA tensor")
        if tuple(out.shape) != (self.num_cells, self.n_conserved):
            raise ValueError("out has the wrong shape")
        s = _stream_arg(stream)
        self._call("ibisgb_residual_device", PRECISION[precision], C.c_void_p(out.data_ptr()), s)
        return out

    def estimate_dt(self) -> float:
        dt = C.c_double()
        self._call("ibisgb_estimate_dt", C.byref(dt))
        return dt.value

    def count_bad_cells(self) -> int:
        n = C.c_int64()
        self._call("ibisgb_count_bad_cells", C.byref(n))
        return n.value

    # ----------------------------------------------------------- time march
    def take_steps(self, n: int, precision: str = "f64") -> dict:
        """n explicit Runge-Kutta steps on the device; returns t, dt, stable_dt, steps."""
        st = RkStatus()
        self._call("ibisgb_rk_run", PRECISION[precision], int(n), C.byref(st))
        return {"t": st.t, "dt": st.dt, "stable_dt": st.stable_dt, "steps": st.steps,
                "bad_cells": st.bad_cells, "device_ms": st.device_ms}

    def take_steps_host(self, U_in, U_out, steps: int = 1, precision: str = "f64") -> dict:
        """For each pair (U_in[j], U_out[j]) of host arrays (N, n_conserved): the state
        from U_in[j], `steps` Runge-Kutta steps, the new state into U_out[j]
        (ibisgb_rk_run_host: the next upload and the previous read-back overlap the
        steps when the arrays are pinned).  Returns the last job's status."""
        arrs_in = [np.ascontiguousarray(a, np.float64) for a in U_in]
        if len(arrs_in) != len(U_out) or not arrs_in:
            raise ValueError("U_in and U_out need the same, nonzero number of arrays")
        shape = (self.num_cells, self.n_conserved)
        for a in list(arrs_in) + list(U_out):
            if a.shape != shape or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                raise ValueError(f"expected contiguous float64 arrays of shape {shape}")
        pin = (C.c_void_p * len(arrs_in))(*[a.ctypes.data for a in arrs_in])
        pout = (C.c_void_p * len(U_out))(*[a.ctypes.data for a in U_out])
        st = RkStatus()
        self._call("ibisgb_rk_run_host", PRECISION[precision], len(arrs_in), int(steps), pin, pout, C.byref(st))
        return {"t": st.t, "dt": st.dt, "stable_dt": st.stable_dt, "steps": st.steps,
                "bad_cells": st.bad_cells, "device_ms": st.device_ms}

    # ------------------------------------------------------- steady / JFNK
    def matrix_vector_product(self, v, inv_dt_star: float = 0.0, allow_reconstruction: bool = True):
        """inv_dt_star * v - (dR/dU) v for v of shape (N, n_conserved) (host arrays);
        SteadyStateLinearisation::matrix_vector_product (steady_state.cpp:52-128)."""
        v = np.ascontiguousarray(v, np.float64).reshape(-1)
        if v.size != self.num_cells * self.n_conserved:
            raise ValueError("v has the wrong size")
        out = np.empty_like(v)
        self._call("ibisgb_jvp", _ptr(v), _ptr(out), float(inv_dt_star), int(allow_reconstruction))
        return out.reshape(self.num_cells, self.n_conserved)

    def matrix_vector_product_into(self, v, out, inv_dt_star: float = 0.0,
                                   allow_reconstruction: bool = True, stream=None):
        """Device version for CUDA float64 tensors of shape (N, n_conserved)."""
        for t in (v, out):
            if not (t.is_cuda and t.element_size() == 8 and t.is_contiguous()):
                raise ValueError("expected contiguous float64 CUDA tensors")
        s = _stream_arg(stream)
        self._call("ibisgb_jvp_device", C.c_void_p(v.data_ptr()), C.c_void_p(out.data_ptr()),
                   float(inv_dt_star), int(allow_reconstruction), s)
        return out

    def vector_jacobian_product(self, w, allow_reconstruction: bool = True, ghosts: bool = False):
        """(dR/dU)^T w for w of shape (N, n_conserved) (host arrays), the transpose of
        matrix_vector_product's Jacobian; with ghosts, also the adjoint of every
        ghost cell's primitives (G, 7: rho, p, T, e, vx, vy, vz)."""
        w = np.ascontiguousarray(w, np.float64).reshape(-1)
        if w.size != self.num_cells * self.n_conserved:
            raise ValueError("w has the wrong size")
        out = np.empty_like(w)
        g = np.empty((self.num_ghost_cells, 7)) if ghosts else None
        self._call("ibisgb_vjp", _ptr(w), _ptr(out), None if g is None else _ptr(g), int(allow_reconstruction))
        out = out.reshape(self.num_cells, self.n_conserved)
        return (out, g) if ghosts else out

    def set_geometry(self, face, cell) -> None:
        """Replace the grid geometry (ibisgb_set_geometry): face (13, F) and cell (4, N+G)
        in the layouts of the face / cell geometry dumps."""
        f = np.ascontiguousarray(face, np.float64)
        c = np.ascontiguousarray(cell, np.float64)
        if f.shape != (13, self.num_faces) or c.shape != (4, self.num_cells + self.num_ghost_cells):
            raise ValueError("face must be (13, F) and cell (4, N+G)")
        self._call("ibisgb_set_geometry", _ptr(f), _ptr(c))

    def shared_tables(self, precision: str = "mixed") -> dict:
        """The geometry-table layout of `precision` (ibisgb_shared_tables): lsq_shared,
        whether the least-squares weights and face offsets are kept once per face slot
        (a uniform lattice), and face_classes, the number of shared face-geometry rows
        (0: per face)."""
        a, b = C.c_int32(), C.c_int32()
        self._call("ibisgb_shared_tables", PRECISION[precision], C.byref(a), C.byref(b))
        return {"lsq_shared": bool(a.value), "face_classes": int(b.value)}

    _FS_KEYS = ("T", "p", "rho", "energy", "vx", "vy", "vz")

    def boundary_tags(self) -> list:
        """The boundary tags in the order the engine numbers them (sorted)."""
        return sorted(self.config["grid"]["boundaries"].keys())

    def flow_state(self, tag: str) -> dict:
        """The flow state of boundary `tag` in the engine (ibisgb_get_flow_state), as the
        config's flow_state object: T, p, rho, energy, vx, vy, vz."""
        fs = np.empty(7)
        self._call("ibisgb_get_flow_state", tag.encode(), _ptr(fs))
        return dict(zip(self._FS_KEYS, (float(x) for x in fs)))

    def set_flow_state(self, tag: str, fs: dict) -> None:
        """Give every action of boundary `tag` that carries a flow state the state fs
        (a flow_state object: T, p, rho, energy, vx, vy, vz; ibisgb_set_flow_state).
        rho and energy are taken as given: build fs with grids.flow_state for a
        state consistent with the gas model."""
        a = np.array([float(fs[k]) for k in self._FS_KEYS])
        self._call("ibisgb_set_flow_state", tag.encode(), _ptr(a))

    def flow_state_adjoint(self, w, allow_reconstruction: bool = True) -> dict:
        """w^T dR/d(flow state) for w of shape (N, n_conserved) (ibisgb_vjp_flow_state):
        {tag: array of 7 (T, p, rho, energy, vx, vy, vz)} for every boundary; zeros for
        boundaries without a flow state."""
        w = np.ascontiguousarray(w, np.float64).reshape(-1)
        if w.size != self.num_cells * self.n_conserved:
            raise ValueError("w has the wrong size")
        tags = self.boundary_tags()
        out = np.empty((max(len(tags), 1), 7))
        self._call("ibisgb_vjp_flow_state", _ptr(w), _ptr(out), int(allow_reconstruction))
        return {t: out[b].copy() for b, t in enumerate(tags)}

    def set_scratch_poison(self, on: bool) -> None:
        """Fill the derivative kernels' scratch buffers with NaN before each tangent /
        adjoint call (ibisgb_set_scratch_poison): a check that no call reads an entry it
        did not write."""
        self._call("ibisgb_set_scratch_poison", int(bool(on)))

    def flow_state_tangent(self, dfs: dict, allow_reconstruction: bool = True) -> np.ndarray:
        """dR/dfs . dfs (ibisgb_jvp_flow_state) for {tag: direction of 7 (T, p, rho,
        energy, vx, vy, vz)} (boundaries left out do not move); returns (N, n_conserved)."""
        tags = self.boundary_tags()
        d = np.zeros((max(len(tags), 1), 7))
        for t, row in dfs.items():
            d[tags.index(t)] = np.asarray(row, np.float64).reshape(7)
        out = np.empty((self.num_cells, self.n_conserved))
        self._call("ibisgb_jvp_flow_state", _ptr(d), _ptr(out), int(allow_reconstruction))
        return out

    def geometry_tangent(self, dface, dcell, allow_reconstruction: bool = True) -> np.ndarray:
        """dR/dgeometry . (dface, dcell) (ibisgb_jvp_geometry) for dface (13, F) and
        dcell (4, N+G) in the layouts of the face / cell geometry dumps; returns
        (N, n_conserved)."""
        df = np.ascontiguousarray(dface, np.float64)
        dc = np.ascontiguousarray(dcell, np.float64)
        if df.shape != (13, self.num_faces) or dc.shape != (4, self.num_cells + self.num_ghost_cells):
            raise ValueError("dface must be (13, F) and dcell (4, N+G)")
        out = np.empty((self.num_cells, self.n_conserved))
        self._call("ibisgb_jvp_geometry", _ptr(df), _ptr(dc), _ptr(out), int(allow_reconstruction))
        return out

    def geometry_adjoint(self, w, allow_reconstruction: bool = True):
        """w^T dR/dgeometry (ibisgb_vjp_geometry) for w of shape (N, n_conserved):
        (face, cell) with face (13, F) = adjoints of n, t1, t2, face centre, area
        (the rows of dump("face_geometry")) and cell (4, N+G) = adjoints of the
        centroids and volumes (the rows of dump("cell_geometry"))."""
        w = np.ascontiguousarray(w, np.float64).reshape(-1)
        if w.size != self.num_cells * self.n_conserved:
            raise ValueError("w has the wrong size")
        face = np.empty((13, self.num_faces))
        cell = np.empty((4, self.num_cells + self.num_ghost_cells))
        self._call("ibisgb_vjp_geometry", _ptr(w), _ptr(face), _ptr(cell), int(allow_reconstruction))
        return face, cell

    def vector_jacobian_product_into(self, w, out, ghost_out=None, allow_reconstruction: bool = True,
                                     stream=None):
        """Device version for contiguous float64 CUDA tensors (N, n_conserved); ghost_out (G, 7) optional."""
        for t in (w, out) + ((ghost_out,) if ghost_out is not None else ()):
            if not (t.is_cuda and t.element_size() == 8 and t.is_contiguous()):
                raise ValueError("expected contiguous float64 CUDA tensors")
        s = _stream_arg(stream)
        g = None if ghost_out is None else C.c_void_p(ghost_out.data_ptr())
        self._call("ibisgb_vjp_device", C.c_void_p(w.data_ptr()), C.c_void_p(out.data_ptr()), g,
                   int(allow_reconstruction), s)
        return out

    def adjoint_step(self, g, lam, cfl: float) -> dict:
        """One pseudo-time step of the steady adjoint J^T lambda = -g (ibisgb_adjoint_step);
        g and lam are contiguous float64 CUDA tensors (N, n_conserved), lam updated in place."""
        from ._lib import AdjointStatus
        for t in (g, lam):
            if not (t.is_cuda and t.element_size() == 8 and t.is_contiguous()):
                raise ValueError("expected contiguous float64 CUDA tensors")
        st = AdjointStatus()
        self._call("ibisgb_adjoint_step", C.c_void_p(g.data_ptr()), C.c_void_p(lam.data_ptr()), float(cfl),
                   C.byref(st))
        return {"residual_norm": st.residual_norm, "scaled_residual_norm": st.scaled_residual_norm,
                "gmres_iterations": st.gmres_iterations, "gmres_converged": bool(st.gmres_converged),
                "gmres_residual": st.gmres_residual, "dt_star": st.dt_star}

    def set_adjoint_krylov(self, max_iters: int) -> None:
        """GMRES length of adjoint_step (0: the steady solver's max_iters)."""
        self._call("ibisgb_set_adjoint_krylov", int(max_iters))

    def steady_initialise(self, precision: str = "f64"):
        """Jfnk::initialise: residual and initial norms at the current state."""
        self._call("ibisgb_steady_initialise", PRECISION[precision])

    def newton_step(self, precision: str = "f64") -> dict:
        """One JFNK step (Jfnk::step): GMRES on (I/dt* - J) dU = R(U), U += dU."""
        st = NewtonStatus()
        self._call("ibisgb_newton_step", PRECISION[precision], C.byref(st))
        return {"relative_residual": st.relative_residual, "residual_norms": list(st.residual_norms),
                "gmres_iterations": st.gmres_iterations, "gmres_converged": bool(st.gmres_converged),
                "gmres_residual": st.gmres_residual, "dt_star": st.dt_star, "cfl": st.cfl,
                "step": st.step, "initial_norms": list(st.initial_norms)}

    def L2_norms(self) -> np.ndarray:
        """global, mass, momentum_x, momentum_y, momentum_z, energy of the first-stage residual."""
        out = np.empty(6)
        self._call("ibisgb_l2_norms", _ptr(out))
        return out

    def synchronize(self):
        self._call("ibisgb_synchronize")

    # ---------------------------------------------------------------- dumps
    def numbering(self) -> dict:
        """Whether the device arrays use an internal (reverse Cuthill-McKee) order,
        and the cell graph's bandwidth in the reference's and the internal order."""
        r, b0, b1 = C.c_int32(), C.c_int64(), C.c_int64()
        self._call("ibisgb_numbering", C.byref(r), C.byref(b0), C.byref(b1))
        return {"renumbered": bool(r.value), "bandwidth_reference": b0.value, "bandwidth_internal": b1.value}

    def dump(self, name: str) -> np.ndarray:
        which, dt = DUMPS[name]
        N, F, G, MF, NT, nc = (self.num_cells, self.num_faces, self.num_ghost_cells, self.max_faces,
                               self.num_cells + self.num_ghost_cells, self.n_conserved)
        shape = {"left": (F,), "right": (F,), "cell_faces": (N, MF), "outsigns": (N, MF),
                 "neighbours": (N, MF), "ghost_source": (G,), "face_geometry": (13, F),
                 "cell_geometry": (4, NT), "limiter_branches": (N, 5), "limiters": (5, N),
                 "face_flux": (F, nc), "ghost_face": (G,), "ghost_boundary": (G,),
                 "face_flux_mixed": (F, nc), "cell_order": (N,), "face_order": (F,), "face_vertices": (F, 4)}[name]
        out = np.empty(shape, dt)
        self._call("ibisgb_get_dump", which, _ptr(out), out.nbytes)
        return out


class Batch(Simulation):
    """Independent cases advanced together in one context (``ibisgb_batch_create``).

    The cases' valid cells are concatenated in case order, so every per-cell
    array of the batch (initial fields, primitives, conserved state, dU/dt) is
    the cases' arrays stacked; ``split`` cuts one back into per-case pieces.
    Each case keeps its own boundary conditions and Runge-Kutta control, so
    ``take_steps`` advances every case by one step of its own dt.  The source
    ``Simulation`` objects are left unchanged."""

    def __init__(self, cases):
        L = _lib.load()
        cases = list(cases)
        arr = (C.c_void_p * len(cases))(*[c._h.value for c in cases])
        h = C.c_void_p()
        check(L.ibisgb_batch_create(arr, len(cases), C.byref(h)), None)
        self.config = cases[0].config
        self._attach(h)
        n = C.c_int32()
        check(L.ibisgb_batch_layout(h, C.byref(n), None, None, None), h)
        self.n_cases = n.value
        self.cell_offsets = np.zeros(self.n_cases + 1, np.int64)
        self.face_offsets = np.zeros(self.n_cases + 1, np.int64)
        self.ghost_offsets = np.zeros(self.n_cases + 1, np.int64)
        check(L.ibisgb_batch_layout(h, None, _ptr(self.cell_offsets), _ptr(self.face_offsets),
                                    _ptr(self.ghost_offsets)), h)

    def split(self, a):
        """Per-case views of an array whose first axis runs over the batch's valid cells."""
        return [a[self.cell_offsets[c]:self.cell_offsets[c + 1]] for c in range(self.n_cases)]

    def case_status(self) -> list:
        """Runge-Kutta status of every case after the last ``take_steps``."""
        st = (RkStatus * self.n_cases)()
        self._call("ibisgb_batch_status", st)
        return [{"t": x.t, "dt": x.dt, "stable_dt": x.stable_dt, "steps": x.steps,
                 "bad_cells": x.bad_cells} for x in st]
