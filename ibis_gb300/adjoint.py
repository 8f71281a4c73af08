"""Discrete adjoint of the steady problem and the gradient of an integrated wall
pressure force with respect to the inflow Mach number and grid-shape
parameters (the Hicks-Henne ramp of grids.ramp_bump_case).

The reference has no adjoint or objective; this module defines them on top of
the engine's tangent / adjoint kernels:

* the objective is the pressure force on the faces of a wall boundary,
  J = sum_f p_c A_f (-n_out,f)[component], with p_c the pressure of the wall
  cell (first order at the wall, like the reference's slip-wall ghost, whose
  pressure is the cell's) and n_out the cell's outward normal;
* the adjoint lambda solves J_R^T lambda = -dJ/dU at the converged state
  (ibisgb_adjoint_step, pseudo-time continuation on the device);
* dJ/dM = lambda . dR/dM through the inflow ghost cells (ibisgb_vjp's ghost
  adjoint; the inflow ghost velocity is M a at fixed T and p);
* dJ/dalpha_k = dJ/dalpha_k|_U + lambda . dR/dalpha_k|_U, the partials at
  fixed U by central differences of the residual and of J on perturbed grids.
"""
from __future__ import annotations

import math

import numpy as np

from .simulation import Simulation


def _bound_index(sim: Simulation, tag: str) -> int:
    tags = sorted(sim.config["grid"]["boundaries"].keys())
    return tags.index(tag)


def wall_force(sim: Simulation, tag: str = "wall", x_min: float | None = None, component: int = 1):
    """(J, dJ/dU) of the pressure force on boundary `tag` (faces with centre x >= x_min)."""
    gas = sim.config["gas_model"]
    k = gas["R"] / gas["Cv"]
    sel = sim.dump("ghost_boundary") == _bound_index(sim, tag)
    faces = sim.dump("ghost_face")[sel]
    cells = sim.dump("ghost_source")[sel]
    fg = sim.dump("face_geometry")
    n = fg[0:3, faces]
    area = fg[12, faces]
    left = sim.dump("left")[faces]
    n_out = np.where(left == cells, n, -n)
    wgt = area * (-n_out[component])
    if x_min is not None:
        wgt = np.where(fg[9, faces] >= x_min, wgt, 0.0)
    U = sim.conserved()
    dim = sim.dim
    rho = U[cells, 0]
    m = U[cells, 1:dim + 1]
    E = U[cells, dim + 1]
    m2 = (m * m).sum(axis=1)
    p = k * (E - 0.5 * m2 / rho)
    J = float(np.sum(wgt * p))
    dJ = np.zeros_like(U)
    np.add.at(dJ[:, 0], cells, wgt * k * 0.5 * m2 / (rho * rho))
    for d in range(dim):
        np.add.at(dJ[:, 1 + d], cells, -wgt * k * m[:, d] / rho)
    np.add.at(dJ[:, dim + 1], cells, wgt * k)
    return J, dJ


def steady_solve(sim: Simulation, tol: float = 1e-10, max_steps: int = 200, precision: str = "f64_exact"):
    """Newton-Krylov steps (ibisgb_newton_step) until the relative residual is below tol."""
    sim.steady_initialise(precision)
    hist = []
    for _ in range(max_steps):
        st = sim.newton_step(precision)
        hist.append(st)
        if st["relative_residual"] < tol or not np.isfinite(st["relative_residual"]):
            break
    return hist


def solve_adjoint(sim: Simulation, dJdU: np.ndarray, tol: float = 1e-10, cfl0: float = 10.0,
                  growth: float = 4.0, cfl_max: float = 1e12, max_steps: int = 100):
    """lambda with J_R^T lambda = -dJ/dU at the current state, by the device's
    pseudo-time continuation (the CFL grows geometrically); returns (lambda, history)."""
    import torch
    g = torch.tensor(np.ascontiguousarray(dJdU), dtype=torch.float64, device="cuda")
    lam = torch.zeros_like(g)
    g0 = float(torch.linalg.vector_norm(g))
    cfl, hist = cfl0, []
    for _ in range(max_steps):
        st = sim.adjoint_step(g, lam, cfl)
        hist.append(st)
        if st["residual_norm"] <= tol * g0:
            break
        cfl = min(cfl * growth, cfl_max)
    torch.cuda.synchronize()
    return lam.cpu().numpy(), hist


def mach_sensitivity(sim: Simulation, lam: np.ndarray, tag: str = "inflow", flow_angle_deg: float = 0.0) -> float:
    """lambda . dR/dM: the inflow ghost velocity is M a (cos, sin of the flow angle) at fixed T, p."""
    gas = sim.config["gas_model"]
    fs = sim.config["grid"]["boundaries"][tag]["pre_reconstruction"][0]["flow_state"]
    a = math.sqrt(gas["gamma"] * gas["R"] * fs["T"])
    _, gadj = sim.vector_jacobian_product(lam, ghosts=True)
    sel = sim.dump("ghost_boundary") == _bound_index(sim, tag)
    th = math.radians(flow_angle_deg)
    return float(np.sum(gadj[sel, 4]) * a * math.cos(th) + np.sum(gadj[sel, 5]) * a * math.sin(th))


def shape_sensitivity(make_sim, bumps: np.ndarray, U: np.ndarray, lam: np.ndarray, k: int, h: float = 1e-7,
                      **force_kw) -> float:
    """dJ/dalpha_k|_U + lambda . dR/dalpha_k|_U, both by central differences on
    grids rebuilt with bump k moved by +-h (make_sim(bumps) -> Simulation)."""
    vals = []
    for sgn in (1.0, -1.0):
        b = np.array(bumps, np.float64)
        b[k] += sgn * h
        s = make_sim(b)
        s.set_conserved(U)
        R = s.compute_dudt("f64_exact")
        J, _ = wall_force(s, **force_kw)
        vals.append((J, R))
    dJ = (vals[0][0] - vals[1][0]) / (2 * h)
    dR = (vals[0][1] - vals[1][1]) / (2 * h)
    return float(dJ + np.sum(lam * dR))
