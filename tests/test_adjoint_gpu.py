"""The adjoint (vector-Jacobian product) kernels of the residual.

* Dot-product test against the tangent: <w, J v> = <J^T w, v> to 1e-12
  relative, on every configuration the tangent covers (viscous included),
  with and without reconstruction; central differences for LDFSS2, whose tangent keeps
  the reference's nonlinear dual floor rule.
* Boundary-state adjoint: the ghost-cell adjoint, contracted with the
  derivative of the inflow ghost state, against central differences of the
  residual in the inflow velocity (step 1e-6 relative): 1e-5.
* torch.autograd: gradcheck of the residual's backward (FP64, limiter-free
  ramp) and forward-mode jvp against the tangent.
"""
import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from tests.cases import case

pytestmark = pytest.mark.gpu


def _setup(name, **kw):
    g, c, st = case(name, **kw)
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    return sim, g, c, st


@pytest.mark.parametrize("name,kw", [("ramp", {}), ("ramp", {"flux": "ausmdv"}), ("ramp", {"flux": "rusanov"}),
                                     ("ramp", {"thermo": "rho_p"}),
                                     ("ramp", {"thermo": "p_T"}), ("ramp", {"limiter": "unlimited"}),
                                     ("ramp", {"order": 1}), ("box", {}), ("box_inout", {}), ("tri", {}),
                                     ("tet", {}), ("wedge", {}), ("pyramid", {}), ("tiny2d", {}),
                                     ("plate", {}), ("plate", {"order": 1}), ("subsonic", {}), ("bl_plate", {}),
                                     ("cflux_ramp", {}), ("cflux_box", {})],
                         ids=lambda x: x if isinstance(x, str) else "-".join(f"{k}={v}" for k, v in x.items()))
@pytest.mark.parametrize("recon", [True, False])
def test_vjp_is_the_transpose_of_the_jvp(name, kw, recon):
    sim, *_ = _setup(name, **kw)
    U = sim.conserved()
    rng = np.random.default_rng(3)
    scale = np.abs(U).mean(axis=0)
    v = rng.standard_normal(U.shape) * scale
    w = rng.standard_normal(U.shape) / scale
    jv = -sim.matrix_vector_product(v, inv_dt_star=0.0, allow_reconstruction=recon)
    jtw = sim.vector_jacobian_product(w, allow_reconstruction=recon)
    lhs, rhs = float(np.sum(w * jv)), float(np.sum(jtw * v))
    mag = float(np.sum(np.abs(w * jv)))
    assert abs(lhs - rhs) <= 1e-12 * mag, (lhs, rhs)


@pytest.mark.parametrize("flux", ["ldfss2", "hanel"])
def test_vjp_matches_central_differences(flux):
    """LDFSS2's tangent keeps the reference's dual floor rule (floor applied to
    the tangent), which is not linear in the direction, so its adjoint (true
    derivative, floor' = 0) is checked against central differences instead."""
    g, c, st = case("ramp", flux=flux, limiter="unlimited")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    U = sim.conserved()
    rng = np.random.default_rng(9)
    scale = np.abs(U).mean(axis=0)
    v = rng.standard_normal(U.shape) * scale
    w = rng.standard_normal(U.shape) / scale
    pred = float(np.sum(sim.vector_jacobian_product(w) * v))
    h = 1e-6
    sim.set_conserved(U + h * v)
    rp = sim.compute_dudt("f64")
    sim.set_conserved(U - h * v)
    rm = sim.compute_dudt("f64")
    fd = float(np.sum(w * (rp - rm) / (2 * h)))
    assert abs(fd - pred) <= 1e-5 * abs(pred), (fd, pred)


def test_inflow_ghost_adjoint_matches_central_differences():
    g, c, st = case("ramp", limiter="unlimited")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    U = sim.conserved()
    rng = np.random.default_rng(5)
    w = rng.standard_normal(U.shape) / np.abs(U).mean(axis=0)
    _, gadj = sim.vector_jacobian_product(w, ghosts=True)
    # inflow ghosts are the first ones (sorted boundary tags: inflow, outflow, top, wall)
    n_in = int(g.markers["inflow"][0].shape[0])
    pred = float(gadj[:n_in, 4].sum())  # d/d(inflow vx) of the ghost state is 1 on vx only
    vx0 = c["grid"]["boundaries"]["inflow"]["pre_reconstruction"][0]["flow_state"]["vx"]
    h = 1e-6 * abs(vx0)
    res = []
    for sgn in (1, -1):
        cc = grids.make_config.__globals__["copy"].deepcopy(c)
        cc["grid"]["boundaries"]["inflow"]["pre_reconstruction"][0]["flow_state"]["vx"] = vx0 + sgn * h
        s2 = Simulation(cc, g)
        s2.set_conserved(U)
        res.append(s2.compute_dudt("f64"))
    fd = float(np.sum(w * (res[0] - res[1]) / (2 * h)))
    assert abs(fd - pred) <= 1e-5 * abs(pred), (fd, pred)


def test_torch_autograd_gradcheck_and_forward_mode():
    torch = pytest.importorskip("torch")
    from torch.autograd.forward_ad import dual_level, make_dual, unpack_dual
    from ibis_gb300.autograd import residual
    g, c, st = case("ramp", ni=10, nj=6, limiter="unlimited")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    U0 = torch.tensor(sim.conserved(), dtype=torch.float64, device="cuda")
    scale = U0.abs().mean(dim=0)
    rscale = residual(sim, U0).abs().mean(dim=0)
    # gradcheck in scaled variables (inputs and outputs of order one), so that one
    # finite-difference step and one tolerance suit every component
    x = (U0 / scale).clone().requires_grad_(True)
    f = lambda x: residual(sim, x * scale) / rscale  # noqa: E731
    assert torch.autograd.gradcheck(f, (x,), eps=1e-6, atol=1e-5, rtol=1e-4, nondet_tol=0.0)
    v = torch.randn_like(U0) * scale
    with dual_level():
        out = residual(sim, make_dual(U0, v))
        jv = unpack_dual(out).tangent
    ref = -torch.tensor(sim.matrix_vector_product(v.cpu().numpy(), inv_dt_star=0.0), device="cuda")
    assert torch.allclose(jv, ref, rtol=1e-12, atol=1e-12 * ref.abs().max().item())


def test_unsteady_adjoint_with_checkpoints():
    """Discrete adjoint of 10 ssp-rk3 steps (frozen time steps, checkpoints every
    3 steps): <dJ/dU0, v> against central differences of J = <w, U_10>, and the
    same gradient with every state kept (checkpoint 1)."""
    torch = pytest.importorskip("torch")
    from ibis_gb300.autograd import rk_steps
    g, c, st = case("ramp", ni=12, nj=6, limiter="unlimited")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    U0 = torch.tensor(sim.conserved(), dtype=torch.float64, device="cuda")
    dt = 0.3 * sim.estimate_dt()
    dts = [dt] * 10
    rng = np.random.default_rng(2)
    scale = U0.abs().mean(dim=0)
    w = torch.tensor(rng.standard_normal(tuple(U0.shape)), device="cuda") / scale
    v = torch.tensor(rng.standard_normal(tuple(U0.shape)), device="cuda") * scale
    grads = []
    for cp in (3, 1):
        x = U0.clone().requires_grad_(True)
        J = (rk_steps(sim, x, dts, checkpoint=cp) * w).sum()
        J.backward()
        grads.append(x.grad.clone())
    assert torch.allclose(grads[0], grads[1], rtol=0, atol=0)
    pred = float((grads[0] * v).sum())
    h = 1e-6
    with torch.no_grad():
        jp = float((rk_steps(sim, U0 + h * v, dts) * w).sum())
        jm = float((rk_steps(sim, U0 - h * v, dts) * w).sum())
    fd = (jp - jm) / (2 * h)
    assert abs(fd - pred) <= 1e-5 * abs(pred), (fd, pred)


def test_torch_autograd_through_the_geometry():
    """The residual as a function of the state and the geometry arrays
    (ibis_gb300.autograd.residual_geometry): gradcheck of the state and geometry
    adjoints against central differences of the residual on geometry installed by
    ibisgb_set_geometry (the least-squares factors formed again), forward mode
    against the geometry tangent, both in scaled variables."""
    torch = pytest.importorskip("torch")
    from torch.autograd.forward_ad import dual_level, make_dual, unpack_dual
    from ibis_gb300.autograd import residual_geometry
    g, c, st = case("ramp", ni=6, nj=3, limiter="unlimited")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    U0 = torch.tensor(sim.conserved(), dtype=torch.float64, device="cuda")
    F0 = torch.tensor(sim.dump("face_geometry"), dtype=torch.float64, device="cuda")
    C0 = torch.tensor(sim.dump("cell_geometry"), dtype=torch.float64, device="cuda")
    su = U0.abs().mean(dim=0)
    sf = F0.abs().mean(dim=1, keepdim=True) + 1e-3
    sc = C0.abs().mean(dim=1, keepdim=True) + 1e-3
    rs = residual_geometry(sim, U0, F0, C0).abs().mean(dim=0)
    xu = (U0 / su).clone().requires_grad_(True)
    xf = (F0 / sf).clone().requires_grad_(True)
    xc = (C0 / sc).clone().requires_grad_(True)
    f = lambda a, b, d: residual_geometry(sim, a * su, b * sf, d * sc) / rs  # noqa: E731
    assert torch.autograd.gradcheck(f, (xu, xf, xc), eps=1e-6, atol=1e-5, rtol=1e-4, nondet_tol=0.0, fast_mode=True)
    # forward mode: the state and geometry tangents together
    du, dfc, dcc = torch.randn_like(U0) * su, torch.randn_like(F0) * sf, torch.randn_like(C0) * sc
    with dual_level():
        out = residual_geometry(sim, make_dual(U0, du), make_dual(F0, dfc), make_dual(C0, dcc))
        jt = unpack_dual(out).tangent
    h = 1e-7
    fd = (residual_geometry(sim, U0 + h * du, F0 + h * dfc, C0 + h * dcc)
          - residual_geometry(sim, U0 - h * du, F0 - h * dfc, C0 - h * dcc)) / (2 * h)
    assert torch.allclose(jt, fd, rtol=1e-5, atol=1e-5 * fd.abs().max().item())
