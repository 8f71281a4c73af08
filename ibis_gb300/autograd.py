"""torch.autograd wrapper of the residual: R(U) = dU/dt of a Simulation as a
differentiable function of the conserved state, with the hand-written tangent
(forward mode) and adjoint (reverse mode) kernels as its derivatives.

    from ibis_gb300.autograd import residual
    U = torch.tensor(sim.conserved(), device="cuda", requires_grad=True)
    R = residual(sim, U)              # FiniteVolume::compute_dudt, FP64
    (R * w).sum().backward()          # U.grad = (dR/dU)^T w, ibisgb_vjp_device

The forward pass evaluates the residual in the FP64_EXACT build (the
reference's operation order), so the backward pass is the exact transpose of
the derivative of what forward returned.  Both run on the current CUDA stream.

Every call goes through the pybind11 module _ibisgb_py (csrc/python/ibisgb_py.cpp),
the sibling of the reference's python_api module, which hands the tensors'
device pointers and the current stream to the C ABI.
"""
from __future__ import annotations

import torch

from . import _ibisgb_py as _py  # built by ibis_gb300.build; the import fails loudly when it is missing

_F64_EXACT = 2


class Residual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U, sim):
        if U.dtype != torch.float64 or not U.is_cuda:
            raise TypeError("U must be a float64 CUDA tensor")
        U = U.contiguous()
        _py.set_conserved(sim, U)
        out = torch.empty_like(U)
        _py.residual(sim, _F64_EXACT, out)
        ctx.sim = sim
        ctx.save_for_backward(U)
        ctx.save_for_forward(U)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (U,) = ctx.saved_tensors
        sim = ctx.sim
        _py.set_conserved(sim, U)  # linearise at the forward state
        g = torch.empty_like(U)
        _py.vjp(sim, grad_out.contiguous(), g)
        return g, None

    @staticmethod
    def jvp(ctx, dU, _):
        (U,) = ctx.saved_tensors
        sim = ctx.sim
        _py.set_conserved(sim, U)
        out = torch.empty_like(U)
        _py.jvp(sim, dU.contiguous(), out, 0.0)
        return -out  # the product is inv_dt v - J v


def residual(sim, U):
    """dU/dt of `sim` at conserved state U (float64 CUDA tensor, N x n_conserved)."""
    return Residual.apply(U, sim)


class ResidualGeometry(torch.autograd.Function):
    """R(U, face, cell): the residual as a function of the state and of the grid
    geometry arrays (face: 13 x F normal, tangents, centre, area; cell: 4 x (N+G)
    centroid, volume -- the layouts of the geometry dumps).  The forward pass
    installs the geometry (ibisgb_set_geometry, which forms the least-squares
    factors again); the backward pass is the state and geometry adjoints
    (ibisgb_vjp / ibisgb_vjp_geometry), forward mode the tangents."""

    @staticmethod
    def forward(ctx, U, face, cell, sim):
        for t, name in ((U, "U"), (face, "face"), (cell, "cell")):
            if t.dtype != torch.float64 or not t.is_cuda:
                raise TypeError(f"{name} must be a float64 CUDA tensor")
        sim.set_geometry(face.detach().cpu().numpy(), cell.detach().cpu().numpy())
        U = U.contiguous()
        _py.set_conserved(sim, U)
        out = torch.empty_like(U)
        _py.residual(sim, _F64_EXACT, out)
        ctx.sim = sim
        ctx.save_for_backward(U, face, cell)
        ctx.save_for_forward(U, face, cell)
        return out

    @staticmethod
    def _linearise(ctx):
        U, face, cell = ctx.saved_tensors
        ctx.sim.set_geometry(face.detach().cpu().numpy(), cell.detach().cpu().numpy())
        _py.set_conserved(ctx.sim, U)
        return U, face, cell

    @staticmethod
    def backward(ctx, grad_out):
        U, face, cell = ResidualGeometry._linearise(ctx)
        w = grad_out.contiguous()
        gU = torch.empty_like(U)
        _py.vjp(ctx.sim, w, gU)
        gf, gc = torch.empty_like(face), torch.empty_like(cell)
        _py.vjp_geometry(ctx.sim, w, gf, gc)
        return gU, gf, gc, None

    @staticmethod
    def jvp(ctx, dU, dface, dcell, _):
        U, face, cell = ResidualGeometry._linearise(ctx)
        out = torch.zeros_like(U)
        if dU is not None:
            _py.jvp(ctx.sim, dU.contiguous(), out, 0.0)
            out = -out  # the product is inv_dt v - J v
        if dface is not None or dcell is not None:
            g = torch.empty_like(U)
            _py.jvp_geometry(ctx.sim, (dface if dface is not None else torch.zeros_like(face)).contiguous(),
                             (dcell if dcell is not None else torch.zeros_like(cell)).contiguous(), g)
            out = out + g
        return out


def residual_geometry(sim, U, face, cell):
    """dU/dt of `sim` at state U on the geometry (face, cell), differentiable in all three."""
    return ResidualGeometry.apply(U, face, cell, sim)


def _flow_state_values(sim, theta):
    """The 7 flow-state entries (T, p, rho, energy, vx, vy, vz) of the inflow
    parameters theta = (T, p, vx, vy, vz): rho = p / (R T) and energy = Cv T from
    the ideal gas, as the prep step's FlowState.as_dict (ibis_py_utils.py:32-37)."""
    gas = sim.config["gas_model"]
    T, p, vx, vy, vz = (float(x) for x in theta.detach().cpu().tolist())
    return [T, p, p / (gas["R"] * T), gas["Cv"] * T, vx, vy, vz]


class ResidualFlowState(torch.autograd.Function):
    """R(U, theta): the residual as a function of the state and of the inflow
    parameters theta = (T, p, vx, vy, vz) of one boundary (float64 tensor of 5;
    rho and energy follow from T and p through the gas model).  The forward pass
    installs the flow state on every action of the boundary that carries one
    (ibisgb_set_flow_state); the backward pass is the state adjoint and the
    flow-state adjoint (ibisgb_vjp / ibisgb_vjp_flow_state) chained through
    rho = p / (R T), energy = Cv T, forward mode the two tangents (ibisgb_jvp /
    ibisgb_jvp_flow_state)."""

    @staticmethod
    def forward(ctx, U, theta, sim, tag):
        if U.dtype != torch.float64 or not U.is_cuda:
            raise TypeError("U must be a float64 CUDA tensor")
        if theta.numel() != 5:
            raise ValueError("theta must hold T, p, vx, vy, vz")
        _py.set_flow_state(sim, tag, _flow_state_values(sim, theta))
        U = U.contiguous()
        _py.set_conserved(sim, U)
        out = torch.empty_like(U)
        _py.residual(sim, _F64_EXACT, out)
        ctx.sim, ctx.tag = sim, tag
        ctx.save_for_backward(U, theta)
        ctx.save_for_forward(U, theta)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        U, theta = ctx.saved_tensors
        sim = ctx.sim
        _py.set_flow_state(sim, ctx.tag, _flow_state_values(sim, theta))  # linearise at the forward state
        _py.set_conserved(sim, U)
        w = grad_out.contiguous()
        gU = torch.empty_like(U)
        _py.vjp(sim, w, gU)
        tags = sorted(sim.config["grid"]["boundaries"].keys())
        graw = torch.empty((len(tags), 7), dtype=torch.float64, device=U.device)
        _py.vjp_flow_state(sim, w, graw)
        g = graw[tags.index(ctx.tag)].to(theta.device)
        gas = sim.config["gas_model"]
        T, p = theta[0].detach(), theta[1].detach()
        R = gas["R"]
        gT = g[0] - g[2] * p / (R * T * T) + g[3] * gas["Cv"]
        gp = g[1] + g[2] / (R * T)
        return gU, torch.stack([gT, gp, g[4], g[5], g[6]]).reshape(theta.shape), None, None

    @staticmethod
    def jvp(ctx, dU, dtheta, _sim, _tag):
        U, theta = ctx.saved_tensors
        sim = ctx.sim
        _py.set_flow_state(sim, ctx.tag, _flow_state_values(sim, theta))
        _py.set_conserved(sim, U)
        out = torch.zeros_like(U)
        if dU is not None:
            _py.jvp(sim, dU.contiguous(), out, 0.0)
            out = -out  # the product is inv_dt v - J v
        if dtheta is not None:
            # the direction of the 7 flow-state entries: rho = p / (R T), energy = Cv T
            gas = sim.config["gas_model"]
            T, p = (float(x) for x in theta.detach().cpu()[:2])
            dT, dp, dvx, dvy, dvz = (float(x) for x in dtheta.detach().cpu().reshape(5))
            R = gas["R"]
            row = [dT, dp, dp / (R * T) - p * dT / (R * T * T), gas["Cv"] * dT, dvx, dvy, dvz]
            tags = sorted(sim.config["grid"]["boundaries"].keys())
            d = torch.zeros((len(tags), 7), dtype=torch.float64, device=U.device)
            d[tags.index(ctx.tag)] = torch.tensor(row, dtype=torch.float64, device=U.device)
            g = torch.empty_like(U)
            _py.jvp_flow_state(sim, d, g)
            out = out + g
        return out


def residual_flow_state(sim, U, theta, tag: str = "inflow"):
    """dU/dt of `sim` at state U with boundary `tag`'s inflow parameters theta =
    (T, p, vx, vy, vz), differentiable in U and theta."""
    return ResidualFlowState.apply(U, theta, sim, tag)


def _tableau(sim):
    """The Butcher tableau of the config's Runge-Kutta block: a (strictly lower), b."""
    bt = sim.config["solver"]["butcher_tableau"]
    b = list(bt["b"])
    s = len(b)
    a = [[0.0] * s for _ in range(s)]
    for i, row in enumerate(bt.get("a", [])):
        for j, x in enumerate(row):
            a[i + 1][j] = x
    return a, b


def _rk_step(sim, U, dt, a, b):
    """One explicit RK step of the FP64 residual with a given dt: the stage
    combination of RungeKutta::take_step (runge_kutta.cpp:131-203), including its
    a(i, j) < 1e-14 skip, on device tensors; returns U_new and the stage states."""
    S = len(b)
    ks, states = [], []
    for i in range(S):
        Ui = U.clone()
        for j in range(i):
            if j > 0 and a[i][j] < 1e-14:
                continue
            Ui.add_(ks[j], alpha=dt * a[i][j])
        states.append(Ui)
        ks.append(residual_raw(sim, Ui))
    Un = U.clone()
    for j in range(S):
        Un.add_(ks[j], alpha=dt * b[j])
    return Un, states


def residual_raw(sim, U):
    _py.set_conserved(sim, U.contiguous())
    out = torch.empty_like(U)
    _py.residual(sim, _F64_EXACT, out)
    return out


def _vjp_raw(sim, U, w):
    _py.set_conserved(sim, U.contiguous())
    out = torch.empty_like(U)
    _py.vjp(sim, w.contiguous(), out)
    return out


class RungeKuttaSteps(torch.autograd.Function):
    """U_N after N explicit Runge-Kutta steps of the given time steps dts, as a
    differentiable function of U_0.  The backward pass is the discrete adjoint of
    the RK scheme: for each step in reverse, stage by stage,
        kbar_m = dt b_m lam + sum_{l > m} dt a(l, m) Ubar_l,   Ubar_m = (dR/dU)(U^(m))^T kbar_m,
        lam <- lam + sum_m Ubar_m,
    with the adjoint kernel at every stage state.  Only every `checkpoint`-th
    state is kept from the forward pass; the states inside a segment are
    recomputed from its checkpoint when the reverse sweep reaches it, and the
    limiter and flux branches are taken again from those states.  The time steps
    are frozen (inputs), as an adjoint of a fixed time discretisation."""

    @staticmethod
    def forward(ctx, U0, sim, dts, checkpoint):
        a, b = _tableau(sim)
        U = U0.detach().clone()
        saved = {0: U.clone()}
        for n, dt in enumerate(dts):
            U, _ = _rk_step(sim, U, float(dt), a, b)
            if (n + 1) % checkpoint == 0 and n + 1 < len(dts):
                saved[n + 1] = U.clone()
        ctx.sim, ctx.dts, ctx.checkpoint, ctx.saved, ctx.tab = sim, list(dts), checkpoint, saved, (a, b)
        return U

    @staticmethod
    def backward(ctx, gN):
        sim, dts, C = ctx.sim, ctx.dts, ctx.checkpoint
        a, b = ctx.tab
        S = len(b)
        lam = gN.contiguous().clone()
        N = len(dts)
        seg_starts = sorted(ctx.saved)
        for s0 in reversed(seg_starts):
            s1 = min(s0 + C, N)
            # recompute the states of this segment from its checkpoint
            states_n = [ctx.saved[s0]]
            for n in range(s0, s1 - 1):
                states_n.append(_rk_step(sim, states_n[-1], float(dts[n]), a, b)[0])
            for n in reversed(range(s0, s1)):
                dt = float(dts[n])
                _, stages = _rk_step(sim, states_n[n - s0], dt, a, b)
                Ubar = [None] * S
                for m in reversed(range(S)):
                    kbar = lam * (dt * b[m])
                    for l in range(m + 1, S):
                        if m > 0 and a[l][m] < 1e-14:
                            continue
                        if a[l][m] != 0.0:
                            kbar = kbar + Ubar[l] * (dt * a[l][m])
                    Ubar[m] = _vjp_raw(sim, stages[m], kbar)
                for m in range(S):
                    lam = lam + Ubar[m]
        return lam, None, None, None


def rk_steps(sim, U0, dts, checkpoint: int = 8):
    """U after len(dts) RK steps of sim's tableau from U0 (float64 CUDA tensor,
    N x n_conserved), differentiable in U0 with checkpointed reverse sweeps."""
    return RungeKuttaSteps.apply(U0, sim, list(dts), int(checkpoint))
