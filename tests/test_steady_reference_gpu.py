"""The GPU engine's JFNK (tangent Jv, device GMRES) converged on the same steady
case as the reference's own SteadyState (tests/golden/reference_steady_ramp64x32.*):
the 64 x 32 Hicks-Henne ramp, first order, residual-based CFL, GMRES(30).  The
first ten relative residuals agree to 1e-6 (1e-3 with FMA contraction) and the
converged conserved state to
1e-10 relative L2 per component (both stop below 1e-12 relative residual), in
the bitwise-exact and the plain FP64 builds."""
import json
import os

import numpy as np
import pytest

from ibis_gb300 import Simulation
from tests.golden.make_steady_fixture import TOL, steady_case

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
U_REF = np.load(os.path.join(HERE, "golden", "reference_steady_ramp64x32.npz"))["U"]
META = json.load(open(os.path.join(HERE, "golden", "reference_steady_ramp64x32.json")))


@pytest.mark.parametrize("precision", ["f64_exact", "f64"])
def test_jfnk_converges_to_the_reference_steady_state(precision):
    g, c, ic = steady_case()
    sim = Simulation(c, g)
    sim.set_primitives(*ic)
    sim.steady_initialise(precision)
    hist = []
    while len(hist) < 200:
        hist.append(sim.newton_step(precision)["relative_residual"])
        if hist[-1] < TOL:
            break
    assert hist[-1] < TOL, hist[-5:]
    assert abs(len(hist) - META["newton_steps"]) <= 2
    U = sim.conserved()
    for q in range(4):
        assert np.linalg.norm(U[:, q] - U_REF[:, q]) <= 1e-10 * np.linalg.norm(U_REF[:, q]), q
    # FMA contraction (the plain FP64 build) moves the early history a little more than rounding order does
    rtol = 1e-6 if precision == "f64_exact" else 1e-3
    assert np.allclose(hist[:10], META["history"][:10], rtol=rtol, atol=0)
