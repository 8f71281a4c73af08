"""Discrete-adjoint gradient of the integrated ramp pressure force (the Hicks-
Henne ramp of the 512 x 256 steady-state case, on a reduced grid) with respect to the inflow Mach
number and the bump amplitudes (the shape terms through the geometry adjoint
kernels), against central differences of the force
between steady states re-converged at perturbed parameters (relative 1e-5).
A 10-degree ramp with second-order (unlimited) reconstruction on a grid small
enough (12 x 6 cells, 288 unknowns) for one GMRES cycle of 300 to solve each
Newton system: Newton-Krylov with the residual-based CFL converges to
round-off, so the differences of the force are accurate to the required
digits.  (The 15-degree ramp's reflected shocks keep this small grid from
settling in pseudo-time.)"""
import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from ibis_gb300.adjoint import (bump_displacements, mach_sensitivity, shape_gradient, shape_sensitivity_fd,
                                solve_adjoint, steady_solve, wall_force)

pytestmark = pytest.mark.gpu

NI, NJ, M0 = 12, 6, 2.0
B0 = np.random.default_rng(0).uniform(-0.002, 0.002, 16)
FORCE = {"tag": "wall", "x_min": 0.2}


def make(mach=M0, bumps=B0):
    cfl = {"type": "residual_based", "growth_threshold": 1.0, "power": 1.0, "start_cfl": 2.0, "max_cfl": 1e12}
    solver = grids.steady_state(cfl=cfl, max_iters=300, tol=1e-12, max_steps=200)
    g, c, inf = grids.ramp_bump_case(NI, NJ, mach=mach, bumps=bumps, angle_deg=10.0, limiter="unlimited",
                                     solver=solver)
    sim = Simulation(c, g)
    n = sim.num_cells
    sim.set_primitives(np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    return sim


def solved(**kw):
    sim = make(**kw)
    hist = steady_solve(sim, tol=1e-13)
    assert hist[-1]["relative_residual"] < 1e-13, [h["relative_residual"] for h in hist]
    return sim


def test_force_gradient_matches_central_differences():
    sim = solved()
    J, dJdU = wall_force(sim, **FORCE)
    assert J > 0
    lam, hist = solve_adjoint(sim, dJdU, tol=1e-13)
    assert hist[-1]["scaled_residual_norm"] <= 1e-13 * hist[0]["scaled_residual_norm"], \
        [h["scaled_residual_norm"] for h in hist]
    # Mach
    dM = mach_sensitivity(sim, lam)
    h = 1e-6 * M0
    fd = (wall_force(solved(mach=M0 + h), **FORCE)[0] - wall_force(solved(mach=M0 - h), **FORCE)[0]) / (2 * h)
    assert abs(dM - fd) <= 1e-5 * abs(fd), (dM, fd)
    # every bump through the geometry adjoint; two of them against re-converged
    # central differences, all against central differences of R and J at fixed U
    U = sim.conserved()
    grid = grids.ramp_2d_bumps(NI, NJ, angle_deg=10.0, bumps=B0)
    gadj = sim.geometry_adjoint(lam)
    disp = bump_displacements(NI, NJ, angle_deg=10.0)
    grads = [shape_gradient(sim, grid, lam, d, geometry_adjoint=gadj, **FORCE) for d in disp]
    for k in range(len(B0)):
        fdu = shape_sensitivity_fd(lambda b: make(bumps=b), B0, U, lam, k, h=1e-7, **FORCE)
        assert abs(grads[k] - fdu) <= 1e-5 * max(abs(fdu), 1e-3 * max(abs(x) for x in grads)), (k, grads[k], fdu)
    for k in (4, 11):
        b_p, b_m = B0.copy(), B0.copy()
        b_p[k] += 1e-7
        b_m[k] -= 1e-7
        fd = (wall_force(solved(bumps=b_p), **FORCE)[0] - wall_force(solved(bumps=b_m), **FORCE)[0]) / 2e-7
        assert abs(grads[k] - fd) <= 1e-5 * abs(fd), (k, grads[k], fd)
