"""The GPU engine against the reference itself (the golden outputs of ibis's
own sources compiled unchanged, tests/golden/reference_outputs.*, made by
tests/golden/make_ref_fixtures.py where an ibis checkout exists).

* F64_EXACT residual: bit for bit on every matched case, except where the
  reference calls pow() (Sutherland's law, LDFSS2): CUDA's and glibc's pow may
  differ in the last bit, <= 1e-14 of the gross flux per cell.
* F64_EXACT Runge-Kutta with the reference's aliased stage derivatives
  ("stage_derivatives": "aliased"): bit for bit after 500 steps of the 64 x 32
  ramp and, by hash, after 2000 steps of the 256 x 128 ramp (the CPU-runnable
  benchmark case) -- the final time included.
* The tangent Jv (the reference's dual-number semantics): <= 1e-12 of the
  largest component.
"""
import copy
import hashlib
import json
import os

import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from tests.cases import case
from tests.golden.make_ref_fixtures import RESIDUAL_CASES, key

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ARR = np.load(os.path.join(HERE, "golden", "reference_outputs.npz"))
META = json.load(open(os.path.join(HERE, "golden", "reference_outputs.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()


def gross_scale(name, kw):
    from oracle.oracle import Oracle
    from tests.cases import gross_flux_scale
    g, c, st = case(name, **kw)
    o = Oracle(c, g)
    o.set_initial_condition(*st)
    o.residual()
    return gross_flux_scale(o)


@pytest.mark.parametrize("name,kw", RESIDUAL_CASES, ids=[key(n, k) for n, k in RESIDUAL_CASES])
def test_exact_residual_equals_the_reference(name, kw):
    g, c, st = case(name, **kw)
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    r = sim.compute_dudt("f64_exact")
    want = ARR[f"residual/{key(name, kw)}"]
    uses_pow = c["viscous_flux"]["enabled"] or c["convective_flux"]["flux_calculator"]["type"] == "ldfss2"
    if uses_pow:
        scale = gross_scale(name, kw)
        assert (np.abs(r - want) / scale).max() <= 1e-14
    else:
        assert np.array_equal(r, want), np.abs(r - want).max()


def _aliased(ni, nj):
    g, c, inf = grids.ramp_case(ni, nj)
    c = copy.deepcopy(c)
    c["solver"]["stage_derivatives"] = "aliased"
    n = g.num_cells
    sim = Simulation(c, g)
    sim.set_primitives(np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    return sim


def test_exact_runge_kutta_equals_the_reference_64x32():
    sim = _aliased(64, 32)
    st = sim.take_steps(500, "f64_exact")
    assert st["t"] == META["rk"]["ramp64x32"]["t"]
    assert np.array_equal(sim.conserved(), ARR["rk/ramp64x32"])


def test_exact_runge_kutta_equals_the_reference_256x128_2000_steps():
    sim = _aliased(256, 128)
    st = sim.take_steps(2000, "f64_exact")
    m = META["rk"]["ramp256x128"]
    assert st["t"] == m["t"]
    assert sha(sim.conserved()) == m["sha256"]


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("mixed_ff", 1e-6)])
def test_fast_builds_follow_the_reference_runge_kutta(precision, tol):
    sim = _aliased(64, 32)
    sim.take_steps(500, precision)
    U, want = sim.conserved(), ARR["rk/ramp64x32"]
    errs = [np.linalg.norm(U[:, q] - want[:, q]) / np.linalg.norm(want[:, q]) for q in range(4)]
    assert max(errs) <= tol, errs


def test_tangent_jv_equals_the_reference_dual_jv():
    g, c, st = case("ramp")
    c["solver"] = grids.steady_state(cfl={"type": "constant", "value": 2.0},
                                     linear_solver={"type": "gmres", "max_iters": 15, "tol": 1e-3})
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    got = sim.matrix_vector_product(ARR["jv/ramp/v"], 1.0 / META["jv"]["ramp"]["dt_star"])
    want = ARR["jv/ramp/result"]
    assert np.abs(got.reshape(-1) - want).max() <= 1e-12 * np.abs(want).max()
