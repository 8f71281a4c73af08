"""Golden outputs of the reference itself -- ibis's own sources compiled here
against the project's subset headers (oracle/Makefile.ref) and driven through
oracle/ref.py -- for the tests that run where no ibis checkout exists (the
oracle's CPU tests, and the GPU tests on the GPU host).  Run by hand after
building the reference:

    python -c "from oracle import ref; ref.build('<ibis checkout>')"
    python tests/golden/make_ref_fixtures.py

Writes tests/golden/reference_outputs.npz (arrays) and
tests/golden/reference_outputs.json (scalars, hashes, provenance):

* residual/<case>, limiters/<case>, estimate_dt: FiniteVolume::compute_dudt
  (finite_volume.cpp:56-96), the Barth-Jespersen limiter values and
  FiniteVolume::estimate_dt on the matched test cases of tests/cases.py;
* rk/ramp64x32: RungeKutta::take_step (runge_kutta.cpp:131-203) on the 64 x 32
  compression ramp for 500 steps from the uniform inflow state, with the
  reference's aliased stage derivatives, the final conserved state;
* rk/ramp256x128 (hash only): the same on the 256 x 128 ramp for 2000 steps,
  the CPU-runnable benchmark case;
* jv/ramp: SteadyStateLinearisation::matrix_vector_product
  (steady_state.cpp:52-128) on the 24 x 12 ramp at the random state of
  tests/cases.py, for one seeded direction;
* jfnk/ramp_*: the relative residual and GMRES iterations of the first Newton
  steps of SteadyState (GMRES and FGMRES, steady_state.cpp:175-326).
"""
import copy
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from ibis_gb300 import grids  # noqa: E402
from oracle import ref  # noqa: E402
from tests.cases import case  # noqa: E402

# (name, kwargs) of tests/cases.py that the reference accepts.  Left out: the
# periodic box (periodic_copy is this project's extension, the reference has no
# such action); the boundary-layer profile (its spline reads past the end of
# its arrays, so its ghost states depend on memory that follows them); the
# p_T thermo pair (the reference indexes gradient arrays it never allocated
# and faults, see test_reference_cpu.py).
RESIDUAL_CASES = [
    ("ramp", {}), ("ramp", {"flux": "ausmdv"}), ("ramp", {"flux": "ldfss2"}), ("ramp", {"flux": "rusanov"}),
    ("ramp", {"thermo": "rho_p"}), ("ramp", {"thermo": "rho_T"}), ("ramp", {"limiter": "unlimited"}),
    ("ramp", {"order": 1}), ("plate", {}), ("box_inout", {}), ("subsonic", {}), ("tri", {}), ("tet", {}),
    ("wedge", {}), ("pyramid", {}), ("pyramid", {"flux": "ausmdv", "thermo": "rho_p"}), ("tiny2d", {}),
    ("tiny3d", {}), ("cflux_ramp", {}), ("cflux_ramp", {"flux": "ldfss2"}), ("cflux_box", {}),
]


def key(name, kw):
    return name + "".join(f"-{k}={v}" for k, v in sorted(kw.items()))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()


def ramp_case_dir(ni, nj, aliased=True, solver=None):
    g, c, inf = grids.ramp_case(ni, nj)
    c = copy.deepcopy(c)
    if solver is not None:
        c["solver"] = solver
    elif aliased:
        c["solver"]["stage_derivatives"] = "aliased"
    n = g.num_cells
    ic = (np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    d = tempfile.mkdtemp()
    grids.write_case(d, g, c, *ic)
    return d, g, c, ic


def main():
    if not ref.available("serial"):
        sys.exit("build the reference first: python -c \"from oracle import ref; ref.build('<ibis checkout>')\"")
    arrays, meta = {}, {"generator": "tests/golden/make_ref_fixtures.py",
                        "reference": "ibis sources compiled with oracle/Makefile.ref (Serial space, "
                                     "-ffp-contract=off)",
                        "residual": {}, "rk": {}, "jv": {}, "jfnk": {}}
    for name, kw in RESIDUAL_CASES:
        g, c, st = case(name, **kw)
        r = ref.RefResidual(c, g)
        r.set_initial_condition(*st)
        k = key(name, kw)
        arrays[f"residual/{k}"] = r.residual()
        arrays[f"limiters/{k}"] = r.limiters()
        meta["residual"][k] = {"estimate_dt": r.estimate_dt(), "sha256": sha(arrays[f"residual/{k}"])}
        print("residual", k, flush=True)

    d, g, c, ic = ramp_case_dir(64, 32)
    rk = ref.RefRungeKutta(d)
    s = rk.steps(500)
    arrays["rk/ramp64x32"] = rk.conserved()
    meta["rk"]["ramp64x32"] = {"steps": 500, "t": s["t"], "dt": s["dt"], "stage_derivatives": "aliased",
                               "sha256": sha(arrays["rk/ramp64x32"])}
    print("rk ramp64x32", s, flush=True)

    d, g, c, ic = ramp_case_dir(256, 128)
    rk = ref.RefRungeKutta(d, "serial")  # the operation-order build (the OpenMP one is for timing)
    s = rk.steps(2000)
    U = rk.conserved()
    meta["rk"]["ramp256x128"] = {"steps": 2000, "t": s["t"], "dt": s["dt"], "stage_derivatives": "aliased",
                                 "sha256": sha(U), "norms": [float(np.linalg.norm(U[:, q])) for q in range(4)],
                                 "seconds": s["seconds"]}
    print("rk ramp256x128", s, flush=True)

    g, c, st = case("ramp")
    for linear in ("gmres", "fgmres"):
        ls = ({"type": "gmres", "max_iters": 15, "tol": 1e-3} if linear == "gmres" else
              {"type": "fgmres", "max_iters": 10, "tolerance": 1e-3, "max_preconditioner_iters": 3,
               "preconditioner_tolerance": 1e-1})
        cs = copy.deepcopy(c)
        cs["solver"] = grids.steady_state(cfl={"type": "constant", "value": 2.0}, linear_solver=ls)
        d = tempfile.mkdtemp()
        grids.write_case(d, g, cs, *st[:4])
        ss = ref.RefSteadyState(d)
        if linear == "gmres":
            v = np.random.default_rng(7).standard_normal(g.num_cells * 4)
            arrays["jv/ramp/v"] = v
            arrays["jv/ramp/result"] = ss.jvp(v, 1e-4)
            meta["jv"]["ramp"] = {"dt_star": 1e-4, "case": "ramp (tests/cases.py)", "seed": 7}
        hist = [ss.newton_step() for _ in range(6)]
        meta["jfnk"][f"ramp_{linear}"] = {"linear_solver": ls, "cfl": 2.0, "history": hist}
        print("jfnk", linear, hist[-1], flush=True)

    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **arrays)
    with open(os.path.join(HERE, "reference_outputs.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main()
