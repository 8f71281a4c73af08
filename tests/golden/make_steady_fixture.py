"""A converged steady state of the reference's own JFNK (SteadyState::take_step on
ibis's unchanged sources, oracle/Makefile.ref), for the tests that converge the
same case on the oracle and on the GPU (tests/test_steady_reference_*.py).

The case is the 64 x 32 Hicks-Henne ramp (15 degrees; the inflow Mach number and
the 16 bump amplitudes drawn from seed 0 as the benchmark draws them), first
order, residual-based CFL (growth threshold 1, power 1.5, start 5), GMRES(30) to
1e-3 per Newton step, from the uniform inflow state, stepped until the relative
global residual is below 1e-12.  Run by hand where an ibis checkout is built
(python -c "from oracle import ref; ref.build('<checkout>')"):

    python tests/golden/make_steady_fixture.py
"""
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from ibis_gb300 import grids  # noqa: E402
from oracle import ref  # noqa: E402

NI, NJ, TOL, MAX_STEPS = 64, 32, 1e-12, 200


def steady_case():
    rng = np.random.default_rng(0)
    mach = float(rng.uniform(1.5, 3.0))
    bumps = rng.uniform(-0.002, 0.002, 16)
    cfl = {"type": "residual_based", "growth_threshold": 1.0, "power": 1.5, "start_cfl": 5.0, "max_cfl": 1e12}
    solver = grids.steady_state(cfl=cfl, max_iters=30, tol=1e-3, max_steps=1000)
    g, c, inf = grids.ramp_bump_case(NI, NJ, mach=mach, bumps=bumps, solver=solver, order=1)
    n = g.num_cells
    ic = (np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    return g, c, ic


def main():
    if not ref.available("serial"):
        sys.exit("build the reference first: python -c \"from oracle import ref; ref.build('<ibis checkout>')\"")
    g, c, ic = steady_case()
    d = tempfile.mkdtemp()
    grids.write_case(d, g, c, *ic)
    ss = ref.RefSteadyState(d)
    hist = []
    while len(hist) < MAX_STEPS:
        hist.append(ss.newton_step())
        if hist[-1]["relative_residual"] < TOL:
            break
    U = ss.conserved(g.num_cells, 4)
    np.savez_compressed(os.path.join(HERE, "reference_steady_ramp64x32.npz"), U=U)
    meta = {"generator": "tests/golden/make_steady_fixture.py", "case": f"{NI}x{NJ} Hicks-Henne ramp, first order",
            "newton_steps": len(hist), "relative_residual": hist[-1]["relative_residual"],
            "history": [h["relative_residual"] for h in hist]}
    with open(os.path.join(HERE, "reference_steady_ramp64x32.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(meta["newton_steps"], meta["relative_residual"])


if __name__ == "__main__":
    main()
