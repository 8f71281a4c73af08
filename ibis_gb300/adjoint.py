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
* dJ/dalpha_k = dJ/dalpha_k|_U + lambda . dR/dalpha_k|_U: lambda^T dR/dgeometry
  from the engine's geometry adjoint (ibisgb_vjp_geometry), chained to the
  vertex displacement of each Hicks-Henne bump through the complex-step
  derivative of the grid geometry (ibis_gb300.geometry).
"""
from __future__ import annotations

import math

import numpy as np

from .simulation import Simulation


def _bound_index(sim: Simulation, tag: str) -> int:
    tags = sorted(sim.config["grid"]["boundaries"].keys())
    return tags.index(tag)


def _wall_faces(sim: Simulation, tag: str):
    sel = sim.dump("ghost_boundary") == _bound_index(sim, tag)
    return sim.dump("ghost_face")[sel], sim.dump("ghost_source")[sel]


def _force(sim: Simulation, U, fg, faces, cells, x_min, component):
    """J = sum p_c A_f (-n_out)[component] over the wall faces (fg may be complex)."""
    k = sim.config["gas_model"]["R"] / sim.config["gas_model"]["Cv"]
    n = fg[0:3, faces]
    left = sim.dump("left")[faces]
    n_out = np.where(left == cells, n, -n)
    wgt = fg[12, faces] * (-n_out[component])
    if x_min is not None:
        wgt = np.where(fg[9, faces].real >= x_min, wgt, 0.0)
    dim = sim.dim
    rho, m, E = U[cells, 0], U[cells, 1:dim + 1], U[cells, dim + 1]
    m2 = (m * m).sum(axis=1)
    p = k * (E - 0.5 * m2 / rho)
    return np.sum(wgt * p), wgt, k


def wall_force(sim: Simulation, tag: str = "wall", x_min: float | None = None, component: int = 1):
    """(J, dJ/dU) of the pressure force on boundary `tag` (faces with centre x >= x_min)."""
    faces, cells = _wall_faces(sim, tag)
    U = sim.conserved()
    J, wgt, k = _force(sim, U, sim.dump("face_geometry"), faces, cells, x_min, component)
    dim = sim.dim
    rho, m = U[cells, 0], U[cells, 1:dim + 1]
    m2 = (m * m).sum(axis=1)
    dJ = np.zeros_like(U)
    np.add.at(dJ[:, 0], cells, wgt * k * 0.5 * m2 / (rho * rho))
    for d in range(dim):
        np.add.at(dJ[:, 1 + d], cells, -wgt * k * m[:, d] / rho)
    np.add.at(dJ[:, dim + 1], cells, wgt * k)
    return float(J), dJ


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
                  growth: float = 4.0, cfl_max: float = 1e12, max_steps: int = 2000, krylov: int = 100,
                  stall_steps: int = 200):
    """lambda with J_R^T lambda = -dJ/dU at the current state, by the device's
    pseudo-time continuation (the CFL grows geometrically; restarted GMRES of
    `krylov` vectors on the variable-scaled J^T once it is large; 0 keeps the
    steady solver's length) until the scaled residual is below tol of its first
    value, or has not fallen by 10% in stall_steps steps (its rounding floor);
    returns (lambda, history)."""
    import torch
    sim.set_adjoint_krylov(krylov)
    g = torch.tensor(np.ascontiguousarray(dJdU), dtype=torch.float64, device="cuda")
    lam = torch.zeros_like(g)
    cfl, hist, first = cfl0, [], None
    best, best_at = math.inf, 0
    for k in range(max_steps):
        st = sim.adjoint_step(g, lam, cfl)
        hist.append(st)
        r = st["scaled_residual_norm"]
        first = r if first is None else first
        if r <= tol * first or not np.isfinite(r):
            break
        if r < 0.9 * best:
            best, best_at = r, k
        elif k - best_at >= stall_steps:  # no 10% gain in stall_steps steps: at the rounding floor
            break
        cfl = min(cfl * growth, cfl_max)
    torch.cuda.synchronize()
    return lam.cpu().numpy(), hist


def inflow_sensitivity(sim: Simulation, lam: np.ndarray, tag: str = "inflow") -> np.ndarray:
    """lambda . dR/dtheta for boundary `tag`'s inflow parameters theta = (T, p, vx, vy,
    vz): the flow-state adjoint (ibisgb_vjp_flow_state: every action of the boundary
    that carries the state, ghost cells and constant-flux faces) chained through
    rho = p / (R T), energy = Cv T."""
    gas = sim.config["gas_model"]
    fs = sim.flow_state(tag)
    g = sim.flow_state_adjoint(lam)[tag]
    T, p, R = fs["T"], fs["p"], gas["R"]
    return np.array([g[0] - g[2] * p / (R * T * T) + g[3] * gas["Cv"], g[1] + g[2] / (R * T), g[4], g[5], g[6]])


def mach_sensitivity(sim: Simulation, lam: np.ndarray, tag: str = "inflow", flow_angle_deg: float = 0.0) -> float:
    """lambda . dR/dM: the inflow velocity is M a (cos, sin of the flow angle) at fixed T, p."""
    gas = sim.config["gas_model"]
    a = math.sqrt(gas["gamma"] * gas["R"] * sim.flow_state(tag)["T"])
    th = math.radians(flow_angle_deg)
    d = inflow_sensitivity(sim, lam, tag)
    return float(d[2] * a * math.cos(th) + d[3] * a * math.sin(th))


def shape_gradient(sim: Simulation, grid, lam: np.ndarray, dxyz: np.ndarray, tag: str = "wall",
                   x_min: float | None = None, component: int = 1, topology=None, geometry_adjoint=None) -> float:
    """dJ/dalpha = dJ/dalpha|_U + lambda . dR/dalpha|_U for the vertex displacement
    dxyz per unit alpha (num_vertices x 3): the engine's geometry adjoint
    lambda^T dR/dgeometry (ibisgb_vjp_geometry, one evaluation serves every
    parameter; pass it as geometry_adjoint to reuse it) contracted with the
    complex-step derivative of the grid geometry (ibis_gb300.geometry), plus the
    force's own dependence on the wall faces' areas and normals."""
    from .geometry import GridTopology
    topo = topology or GridTopology(sim, grid)
    fb, cb = geometry_adjoint if geometry_adjoint is not None else sim.geometry_adjoint(lam)
    h = 1e-30
    fz, cz = topo.geometry(np.asarray(grid.xyz, np.float64) + 1j * h * np.asarray(dxyz, np.float64))
    faces, cells = _wall_faces(sim, tag)
    Jz, _, _ = _force(sim, sim.conserved(), fz, faces, cells, x_min, component)
    return float(Jz.imag / h + np.sum(fb * fz.imag / h) + np.sum(cb * cz.imag / h))


def shape_sensitivity_fd(make_sim, bumps: np.ndarray, U: np.ndarray, lam: np.ndarray, k: int, h: float = 1e-7,
                         **force_kw) -> float:
    """The same derivative for bump k by central differences at fixed U of the
    residual and of J on grids rebuilt with bump k moved by +-h (make_sim(bumps)
    -> Simulation); a check of shape_gradient."""
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


def bump_displacements(ni: int, nj: int, n_bumps: int = 16, **kw) -> list:
    """Vertex displacement of the Hicks-Henne ramp grid per unit amplitude of each
    bump (grids.ramp_2d_bumps is linear in the amplitudes)."""
    from . import grids
    base = grids.ramp_2d(ni, nj, **kw).xyz
    out = []
    for k in range(n_bumps):
        e = np.zeros(n_bumps)
        e[k] = 1.0
        out.append(grids.ramp_2d_bumps(ni, nj, bumps=e, **kw).xyz - base)
    return out


def converge(sim: Simulation, precision: str = "f64", rel_tol: float | None = 1e-12, abs_tol: float | None = None,
             max_steps: int = 400):
    """Newton-Krylov steps until the global residual norm is below abs_tol, or,
    without abs_tol, the relative residual below rel_tol; returns the history."""
    sim.steady_initialise(precision)
    hist = []
    for _ in range(max_steps):
        st = sim.newton_step(precision)
        hist.append(st)
        r = st["residual_norms"][0]
        if not np.isfinite(r):
            break
        if abs_tol is not None and r <= abs_tol:
            break
        if abs_tol is None and st["relative_residual"] <= rel_tol:
            break
    return hist


def gradient_check(ni: int = 512, nj: int = 256, seed: int = 0, order: int = 1, step: float = 1e-6,
                   tol: float = 1e-12, n_bumps: int = 16) -> dict:
    """The pressure force on the ramp (x >= 0.2) of the Hicks-Henne ramp case
    (grids.ramp_bump_case, 15 degrees; Mach U[1.5, 3] and n_bumps amplitudes
    U[-0.002, 0.002] m from `seed`, as the benchmark draws them): its adjoint
    gradient with respect to the Mach number and every amplitude, and central
    differences (step `step`) of the force between states re-converged at the
    perturbed parameters, each started from the base state and converged to the
    same absolute residual (tol times the cold start's initial residual)."""
    from . import grids
    rng = np.random.default_rng(seed)
    mach = float(rng.uniform(1.5, 3.0))
    bumps = rng.uniform(-0.002, 0.002, n_bumps)
    cfl = {"type": "residual_based", "growth_threshold": 1.0, "power": 1.5, "start_cfl": 5.0, "max_cfl": 1e12}
    solver = grids.steady_state(cfl=cfl, max_iters=30, tol=1e-3, max_steps=1000)
    force = {"tag": "wall", "x_min": 0.2}

    def make(m, b):
        g, c, inf = grids.ramp_bump_case(ni, nj, mach=m, bumps=b, solver=solver, order=order)
        s = Simulation(c, g)
        n = s.num_cells
        s.set_primitives(np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
        return s

    base = make(mach, bumps)
    h0 = converge(base, rel_tol=tol)
    abs_tol = tol * h0[0]["initial_norms"][0]
    U0 = base.conserved()
    J0, dJdU = wall_force(base, **force)
    lam, ah = solve_adjoint(base, dJdU, tol=1e-10)
    grads = [mach_sensitivity(base, lam)]
    from .geometry import GridTopology
    grid = grids.ramp_2d_bumps(ni, nj, bumps=bumps)
    topo = GridTopology(base, grid)
    gadj = base.geometry_adjoint(lam)
    grads += [shape_gradient(base, grid, lam, dx, topology=topo, geometry_adjoint=gadj, **force)
              for dx in bump_displacements(ni, nj, n_bumps)]

    newton = []

    def J_at(m, b):
        s = make(m, b)
        s.set_conserved(U0)
        h = converge(s, abs_tol=abs_tol)
        newton.append(len(h))
        return wall_force(s, **force)[0]

    fds = [(J_at(mach + step, bumps) - J_at(mach - step, bumps)) / (2 * step)]
    for k in range(n_bumps):
        bp, bm = bumps.copy(), bumps.copy()
        bp[k] += step
        bm[k] -= step
        fds.append((J_at(mach, bp) - J_at(mach, bm)) / (2 * step))
    rel = [abs(g - f) / abs(f) for g, f in zip(grads, fds)]
    return {"grid": f"{ni}x{nj}", "order": order, "mach": mach, "force": J0, "step": step,
            "base_newton_steps": len(h0), "base_relative_residual": h0[-1]["relative_residual"],
            "adjoint_steps": len(ah),
            "adjoint_relative_residual": ah[-1]["scaled_residual_norm"] / ah[0]["scaled_residual_norm"],
            "gradient": grads, "central_differences": fds, "relative_errors": rel,
            "newton_steps_per_perturbed_solve": newton}
