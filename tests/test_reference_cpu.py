"""The oracle against the reference itself.

tests/golden/reference_outputs.{npz,json} hold outputs of ibis's own sources,
compiled unchanged against the project's subset headers (oracle/Makefile.ref)
and run through oracle/ref.py (tests/golden/make_ref_fixtures.py made them).
The oracle must reproduce them:

* FiniteVolume::compute_dudt, the Barth-Jespersen limiter values and
  estimate_dt: bit for bit, on every matched case the reference accepts
  (every flux calculator, the rho_u / rho_p / rho_T thermo pairs, first order,
  unlimited, viscous, subsonic and constant-flux boundaries, every element type);
* RungeKutta: bit for bit, with the reference's aliased stage derivatives
  ("stage_derivatives": "aliased"), after 500 steps of the 64 x 32 ramp and
  (by hash) 2000 steps of the 256 x 128 ramp;
* the dual-number Jv of SteadyStateLinearisation: to the last bit or so
  (<= 1e-15 of the largest component);
* the first JFNK steps (GMRES and FGMRES): the same GMRES iteration counts and
  relative residuals to 1e-12.

Where the reference is built here (oracle/_ref), its own doctests run too, and
the two behaviours recorded in the fixtures' docstring are checked on it
directly: the p_T thermo pair faults, and its RungeKutta without aliasing is
not the reference's.
"""
import copy
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from ibis_gb300 import grids
from oracle import ref
from oracle.oracle import Oracle
from tests.cases import case
from tests.golden.make_ref_fixtures import RESIDUAL_CASES, key

HERE = os.path.dirname(os.path.abspath(__file__))
ARR = np.load(os.path.join(HERE, "golden", "reference_outputs.npz"))
META = json.load(open(os.path.join(HERE, "golden", "reference_outputs.json")))
# the reference's limiter columns (rho, p, T, u, vx, vy, vz) in the oracle's
# recon dump (rho, u, p, T, vx, vy, vz)
REF_TO_ORACLE = [0, 2, 3, 1, 4, 5, 6]

needs_ref = pytest.mark.skipif(not ref.available(), reason="the reference is not built here (oracle/_ref)")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()


def aliased_ramp(ni, nj):
    g, c, inf = grids.ramp_case(ni, nj)
    c = copy.deepcopy(c)
    c["solver"]["stage_derivatives"] = "aliased"
    n = g.num_cells
    ic = (np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    return g, c, ic


@pytest.mark.parametrize("name,kw", RESIDUAL_CASES, ids=[key(n, k) for n, k in RESIDUAL_CASES])
def test_oracle_residual_and_limiters_equal_the_reference(name, kw):
    g, c, st = case(name, **kw)
    o = Oracle(c, g)
    o.set_initial_condition(*st)
    k = key(name, kw)
    assert np.array_equal(o.residual(), ARR[f"residual/{k}"])
    assert o.estimate_dt() == META["residual"][k]["estimate_dt"]
    cf = c["convective_flux"]
    if cf["reconstruction_order"] == 2 and cf["limiter"]["type"] == "barth_jespersen":
        lim_ref = ARR[f"limiters/{k}"]
        lim, _ = o.recon_dump()
        for j in range(7):
            if np.all(np.isfinite(lim_ref[:, j])):
                assert np.array_equal(lim[:, REF_TO_ORACLE[j]], lim_ref[:, j]), j


def test_oracle_runge_kutta_equals_the_reference_with_aliased_stages():
    g, c, ic = aliased_ramp(64, 32)
    o = Oracle(c, g)
    o.set_initial_condition(*ic)
    o.rk_initialise()
    st = o.rk_steps(500)
    m = META["rk"]["ramp64x32"]
    assert st["t"] == m["t"]
    assert np.array_equal(o.conserved(), ARR["rk/ramp64x32"])


def test_oracle_runge_kutta_equals_the_reference_on_the_256x128_ramp():
    g, c, ic = aliased_ramp(256, 128)
    o = Oracle(c, g)
    o.set_initial_condition(*ic)
    o.rk_initialise()
    st = o.rk_steps(2000)
    m = META["rk"]["ramp256x128"]
    assert st["t"] == m["t"]
    assert sha(o.conserved()) == m["sha256"]


def test_oracle_dual_jv_equals_the_reference():
    g, c, st = case("ramp")
    c["solver"] = grids.steady_state(cfl={"type": "constant", "value": 2.0},
                                     linear_solver={"type": "gmres", "max_iters": 15, "tol": 1e-3})
    o = Oracle(c, g, kind="dual")
    o.set_initial_condition(*st)
    o.steady_initialise()
    got = o.jvp(ARR["jv/ramp/v"], META["jv"]["ramp"]["dt_star"])
    want = ARR["jv/ramp/result"]
    assert np.abs(got - want).max() <= 1e-15 * np.abs(want).max()


@pytest.mark.parametrize("linear", ["gmres", "fgmres"])
def test_oracle_jfnk_history_equals_the_reference(linear):
    m = META["jfnk"][f"ramp_{linear}"]
    g, c, st = case("ramp")
    c["solver"] = grids.steady_state(cfl={"type": "constant", "value": m["cfl"]}, linear_solver=m["linear_solver"])
    o = Oracle(c, g, kind="dual")
    o.set_initial_condition(*st)
    o.steady_initialise()
    hist = o.steady_steps(len(m["history"]))
    assert [int(x) for x in hist[:, 1]] == [h["gmres_iterations"] for h in m["history"]]
    assert np.allclose(hist[:, 0], [h["relative_residual"] for h in m["history"]], rtol=1e-12, atol=0)


@needs_ref
def test_reference_doctests_pass():
    r = ref.run_doctests()
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout


@needs_ref
def test_reference_p_T_thermo_pair_faults():
    # the reference requests gradients of p and u for the p_T pair but limits and
    # reconstructs p and T (convective_flux.cpp:53-55 vs :198-201, 322-331), so it
    # reads a temperature gradient it never allocated
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from oracle.ref import RefResidual\nfrom tests.cases import case\n"
            "g, c, st = case('ramp', thermo='p_T'); r = RefResidual(c, g); r.set_initial_condition(*st)\n"
            "r.residual()\n" % os.path.dirname(HERE))
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert p.returncode < 0, (p.returncode, p.stderr[-2000:])


@needs_ref
def test_reference_runge_kutta_aliases_its_stage_derivatives():
    g, c, ic = aliased_ramp(32, 16)
    d = tempfile.mkdtemp()
    c_sep = copy.deepcopy(c)
    del c_sep["solver"]["stage_derivatives"]
    grids.write_case(d, g, c_sep, *ic)  # the reference reads no stage_derivatives key
    r = ref.RefRungeKutta(d)
    r.steps(20)
    out = {}
    for mode, cfg in (("aliased", c), ("separate", c_sep)):
        o = Oracle(cfg, g)
        o.set_initial_condition(*ic)
        o.rk_initialise()
        o.rk_steps(20)
        out[mode] = o.conserved()
    assert np.array_equal(r.conserved(), out["aliased"])
    assert not np.array_equal(r.conserved(), out["separate"])
