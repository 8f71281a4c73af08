"""ORACLE -- test infrastructure only.

ctypes wrapper of the reference itself: ibis's own sources compiled unchanged
against this project's subset headers of Kokkos / nlohmann::json / spdlog /
doctest (oracle/Makefile.ref -> oracle/_ref/libibisref.so), driven through
oracle/ref_harness.cpp.  Only tests and the fixture generator use it, as the
checker; it needs an ibis checkout to build, so it exists only where one is.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIBS = {"serial": os.path.join(REF_DIR, "libibisref.so"), "openmp": os.path.join(REF_DIR, "libibisref_omp.so")}
DOCTESTS = os.path.join(REF_DIR, "ref_doctests")

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_libs = {}


def build(checkout: str, jobs: int = 8) -> None:
    """Compile the reference from an ibis checkout with oracle/Makefile.ref and
    prepare the working directory its doctests expect."""
    subprocess.run(["make", "-s", "-f", "Makefile.ref", f"REF={checkout}", f"-j{jobs}"], cwd=HERE, check=True)
    os.makedirs(os.path.join(REF_DIR, "t", "a", "b", "c"), exist_ok=True)
    link = os.path.join(REF_DIR, "t", "src")
    if os.path.islink(link):
        os.remove(link)
    os.symlink(os.path.join(checkout, "src"), link)


def available(kind: str = "serial") -> bool:
    return os.path.exists(LIBS[kind])


def lib(kind: str = "serial"):
    if kind in _libs:
        return _libs[kind]
    L = C.CDLL(LIBS[kind])
    L.ref_last_error.restype = C.c_char_p
    L.ref_threads.restype = C.c_int
    L.ref_fv_create.restype = C.c_void_p
    L.ref_fv_create.argtypes = [C.c_char_p, C.c_char_p]
    for name in ("ref_rk_create", "ref_ss_create"):
        getattr(L, name).restype = C.c_void_p
        getattr(L, name).argtypes = [C.c_char_p]
    for name in ("ref_fv_destroy", "ref_rk_destroy", "ref_ss_destroy"):
        getattr(L, name).argtypes = [C.c_void_p]
    L.ref_fv_sizes.argtypes = [C.c_void_p, _lp]
    L.ref_rk_sizes.argtypes = [C.c_void_p, _lp]
    L.ref_fv_set_prims.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.c_void_p]
    L.ref_fv_residual.argtypes = [C.c_void_p, _dp, C.c_int]
    L.ref_fv_limiters.argtypes = [C.c_void_p, _dp]
    L.ref_fv_gradients.argtypes = [C.c_void_p, _dp]
    L.ref_fv_prims.argtypes = [C.c_void_p, _dp]
    L.ref_fv_estimate_dt.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    L.ref_rk_steps.argtypes = [C.c_void_p, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_double),
                               C.POINTER(C.c_double)]
    L.ref_rk_conserved.argtypes = [C.c_void_p, _dp]
    L.ref_ss_jv.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int]
    L.ref_ss_step.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.POINTER(C.c_longlong)]
    L.ref_ss_conserved.argtypes = [C.c_void_p, _dp]
    L.ref_run_case.argtypes = [C.c_char_p]
    _libs[kind] = L
    return L


def _check(L, rc):
    if rc != 0:
        raise RuntimeError("reference: " + L.ref_last_error().decode())


def _config_text(config) -> str:
    return config if isinstance(config, str) else json.dumps(config)


class RefResidual:
    """FiniteVolume<double> of the reference on one grid (residual, limiters,
    gradients, estimate_dt at a state set from T, p, v)."""

    def __init__(self, config, grid, kind: str = "serial"):
        self.L = lib(kind)
        self._tmp = tempfile.TemporaryDirectory()
        path = os.path.join(self._tmp.name, "block_0000.su2")
        grid.write(path)
        self.h = self.L.ref_fv_create(_config_text(config).encode(), path.encode())
        if not self.h:
            raise RuntimeError("reference: " + self.L.ref_last_error().decode())
        s = np.zeros(4, np.int64)
        _check(self.L, self.L.ref_fv_sizes(self.h, s))
        self.N, self.G, self.F, self.dim = (int(x) for x in s)
        self.nc = self.dim + 2

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_fv_destroy(self.h)
            self.h = None

    def set_initial_condition(self, T, p, vx, vy, vz=None):
        a = [np.ascontiguousarray(x, np.float64) for x in (T, p, vx, vy)]
        z = None if vz is None else np.ascontiguousarray(vz, np.float64)
        _check(self.L, self.L.ref_fv_set_prims(self.h, *a, None if z is None else z.ctypes.data))

    def residual(self, allow_reconstruction=True):
        out = np.zeros(self.N * self.nc)
        _check(self.L, self.L.ref_fv_residual(self.h, out, int(allow_reconstruction)))
        return out.reshape(self.N, self.nc)

    def limiters(self):
        """N x 7 (rho, p, T, u, vx, vy, vz), NaN where the reference keeps none."""
        out = np.zeros(self.N * 7)
        _check(self.L, self.L.ref_fv_limiters(self.h, out))
        return out.reshape(self.N, 7)

    def gradients(self):
        """N x 7 x 3 in the order of limiters()."""
        out = np.zeros(self.N * 21)
        _check(self.L, self.L.ref_fv_gradients(self.h, out))
        return out.reshape(self.N, 7, 3)

    def primitives(self):
        out = np.zeros(7 * (self.N + self.G))
        _check(self.L, self.L.ref_fv_prims(self.h, out))
        return out.reshape(7, self.N + self.G)

    def estimate_dt(self):
        d = C.c_double()
        _check(self.L, self.L.ref_fv_estimate_dt(self.h, C.byref(d)))
        return d.value


class RefRungeKutta:
    """The reference's RungeKutta solver on a case directory written by
    ibis_gb300.grids.write_case (initialised from its flow files)."""

    def __init__(self, case_dir: str, kind: str = "serial"):
        self.L = lib(kind)
        self.h = self.L.ref_rk_create(case_dir.encode())
        if not self.h:
            raise RuntimeError("reference: " + self.L.ref_last_error().decode())
        s = np.zeros(4, np.int64)
        _check(self.L, self.L.ref_rk_sizes(self.h, s))
        self.N, self.G, self.F, self.dim = (int(x) for x in s)
        self.nc = self.dim + 2

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_rk_destroy(self.h)
            self.h = None

    def steps(self, n: int) -> dict:
        t, dt, sec = C.c_double(), C.c_double(), C.c_double()
        rc = self.L.ref_rk_steps(self.h, int(n), C.byref(t), C.byref(dt), C.byref(sec))
        if rc < 0:
            _check(self.L, rc)
        return {"t": t.value, "dt": dt.value, "seconds": sec.value, "bad_cells": rc == 1}

    def conserved(self):
        out = np.zeros(self.N * self.nc)
        _check(self.L, self.L.ref_rk_conserved(self.h, out))
        return out.reshape(self.N, self.nc)


class RefSteadyState:
    """The reference's SteadyState (JFNK) solver on a case directory."""

    def __init__(self, case_dir: str, kind: str = "serial"):
        self.L = lib(kind)
        self.h = self.L.ref_ss_create(case_dir.encode())
        if not self.h:
            raise RuntimeError("reference: " + self.L.ref_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_ss_destroy(self.h)
            self.h = None

    def jvp(self, v, dt_star, allow_reconstruction=True):
        """v / dt_star - dR/dU v by the reference's dual numbers."""
        v = np.ascontiguousarray(v, np.float64).reshape(-1)
        out = np.zeros_like(v)
        _check(self.L, self.L.ref_ss_jv(self.h, v, out, float(dt_star), int(allow_reconstruction)))
        return out

    def newton_step(self) -> dict:
        r, d, it = C.c_double(), C.c_double(), C.c_longlong()
        _check(self.L, self.L.ref_ss_step(self.h, C.byref(r), C.byref(d), C.byref(it)))
        return {"relative_residual": r.value, "dt_star": d.value, "gmres_iterations": it.value}

    def conserved(self, N, nc):
        out = np.zeros(N * nc)
        _check(self.L, self.L.ref_ss_conserved(self.h, out))
        return out.reshape(N, nc)


def run_case(case_dir: str, kind: str = "serial") -> int:
    """The reference's own driver (make_solver + Solver::solve) on a case
    directory, as `ibis run` runs it; returns solve()'s result (0: done)."""
    L = lib(kind)
    rc = L.ref_run_case(case_dir.encode())
    if rc < 0:
        _check(L, rc)
    return rc


def run_prep(case_dir: str, checkout: str) -> None:
    """The reference's unchanged prep step (src/ibis/ibis/commands/prep/prep.py,
    main(job.py, share)) in case_dir, with its pybind11 module built here
    (Makefile.ref pyapi); run in a child process, as `ibis prep` runs it in its
    own interpreter."""
    code = ("import sys\n"
            f"sys.path[:0] = [{os.path.join(checkout, 'src/ibis/ibis/commands')!r}, "
            f"{os.path.join(checkout, 'src/ibis/ibis/commands/prep')!r}, {REF_DIR!r}]\n"
            "import prep\n"
            f"prep.main('job.py', {os.path.join(checkout, 'share')!r})\n")
    subprocess.run([sys.executable, "-c", code], cwd=case_dir, check=True, capture_output=True, text=True)


def run_doctests(timeout: float = 600.0) -> subprocess.CompletedProcess:
    """The TEST_CASEs ibis keeps in its sources, run by its own doctest main.
    They read fixtures at ../../../src/grid/test/ relative to the working
    directory, so they run three levels below a directory linking the
    checkout's src (see build)."""
    return subprocess.run([DOCTESTS], cwd=os.path.join(REF_DIR, "t", "a", "b", "c"), capture_output=True,
                          text=True, timeout=timeout)
