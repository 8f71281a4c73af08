"""Boundary flow states as parameters: ibisgb_set_flow_state against contexts
built from configs that hold the new state (bit for bit, every precision,
residual and Runge-Kutta steps), and the flow-state adjoint
ibisgb_vjp_flow_state as the transpose of the oracle's dual-number derivative
along a random flow-state perturbation (<w, dR/dfs . d> = <J_fs^T w, d> to
1e-12; LDFSS2 against central differences) -- supersonic, subsonic and
constant-flux inflows, the flow state
copied before the viscous gradients, first and second order, 2-D and 3-D,
every element type, the grid renumbered or not -- the flow-state tangent
ibisgb_jvp_flow_state equal to that dual derivative, and the torch.autograd
Function over the inflow parameters (T, p, vx, vy, vz), reverse and forward
mode, against central differences of the residual."""
import copy

import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from oracle.oracle import Oracle
from tests.cases import case
from tests.test_flow_state_cpu import KEYS, flow_states, make_case

pytestmark = pytest.mark.gpu

CASES = [("ramp", {}, "inflow"), ("ramp", {"limiter": "unlimited"}, "inflow"), ("ramp", {"order": 1}, "inflow"),
         ("ramp", {"flux": "ausmdv"}, "inflow"), ("ramp", {"flux": "rusanov"}, "inflow"),
         ("subsonic", {}, "west"), ("subsonic", {"order": 1}, "west"), ("cflux_ramp", {}, "inflow"),
         ("cflux_box", {}, "top"), ("cflux_box", {}, "west"), ("box_inout", {}, "west"), ("bl_plate", {}, "north"),
         ("plate", {"viscous_inflow": True}, "inflow"), ("plate", {}, "inflow"),
         ("tri", {}, None), ("tet", {}, None), ("wedge", {}, None), ("pyramid", {}, None)]
IDS = [f"{n}-{t}" + "".join(f"-{k}={v}" for k, v in kw.items()) for n, kw, t in CASES]
PRECISIONS = ("f64_exact", "f64", "mixed", "mixed_ff")


def first_tag(g, c, tag):
    return tag if tag is not None else next(iter(g.markers))


def shifted(fs, gas):
    return grids.flow_state(gas, fs["T"] * 1.03, fs["p"] * 0.97, fs["vx"] * 1.02, fs["vy"] + 5.0, fs["vz"] - 3.0)


@pytest.mark.parametrize("name,kw,tag", CASES, ids=IDS)
def test_set_flow_state_is_a_config_with_that_state(name, kw, tag):
    g, c, st = make_case(name, kw)
    tag = first_tag(g, c, tag)
    fs2 = shifted(flow_states(c, tag)[0], c["gas_model"])
    c2 = copy.deepcopy(c)
    for fs in flow_states(c2, tag):
        fs.update(fs2)
    a, b = Simulation(c, g), Simulation(c2, g)
    for s in (a, b):
        s.set_primitives(*st)
    r0 = a.compute_dudt("f64_exact")  # the old state, so that nothing of it can linger
    a.set_flow_state(tag, fs2)
    assert a.flow_state(tag) == {k: float(fs2[k]) for k in KEYS}
    for prec in PRECISIONS:
        ra, rb = a.compute_dudt(prec), b.compute_dudt(prec)
        assert np.array_equal(ra, rb), prec
    assert not np.array_equal(r0, a.compute_dudt("f64_exact"))
    for prec in ("f64", "mixed"):
        for s in (a, b):
            s.set_primitives(*st)
            s.take_steps(2, prec)
        assert np.array_equal(a.conserved(), b.conserved()), prec


def test_set_flow_state_rejects_bad_input():
    g, c, st = case("ramp")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    fs = sim.flow_state("inflow")
    with pytest.raises(Exception, match="no boundary"):
        sim.set_flow_state("nowhere", fs)
    with pytest.raises(Exception, match="has no flow state"):
        sim.set_flow_state("outflow", fs)
    with pytest.raises(Exception, match="finite"):
        sim.set_flow_state("inflow", dict(fs, p=float("nan")))
    assert sim.flow_state("inflow") == fs  # unchanged by the refused calls


@pytest.mark.parametrize("name,kw,tag", CASES, ids=IDS)
def test_flow_state_adjoint_is_the_transpose_of_the_dual_derivative(name, kw, tag):
    g, c, st = make_case(name, kw)
    tag = first_tag(g, c, tag)
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    cs = copy.deepcopy(c)
    cs["solver"] = grids.steady_state()
    o = Oracle(cs, g, kind="dual")
    o.set_initial_condition(*st)
    o.steady_initialise()
    U = sim.conserved()
    rng = np.random.default_rng(17)
    w = rng.standard_normal(U.shape) / np.abs(U).mean(axis=0)
    fs0 = flow_states(c, tag)[0]
    d = rng.standard_normal(7) * np.array([abs(fs0[k]) + 1.0 for k in KEYS])
    if sim.dim == 2:
        d[6] = 0.0
    jd = o.flow_state_jvp(tag, d)
    adj = sim.flow_state_adjoint(w)
    lhs = float(np.sum(w * jd))
    rhs = float(np.dot(adj[tag], d))
    mag = float(np.sum(np.abs(w * jd)))
    assert mag > 0
    assert abs(lhs - rhs) <= 1e-12 * mag, (lhs, rhs, mag)
    for t, row in adj.items():  # boundaries without a flow state have no derivative
        if not flow_states(c, t):
            assert not row.any(), t


@pytest.mark.parametrize("flux", ["ldfss2", "hanel"])
def test_flow_state_adjoint_matches_central_differences(flux):
    """The reference's dual rule for LDFSS2 (floor applied to the tangent) leaves the
    oracle's dual derivative undefined there, so LDFSS2's flow-state adjoint (true
    derivative, floor' = 0) is checked against central differences of the engine's
    residual under ibisgb_set_flow_state instead."""
    g, c, st = case("ramp", flux=flux, limiter="unlimited")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    U = sim.conserved()
    rng = np.random.default_rng(23)
    w = rng.standard_normal(U.shape) / np.abs(U).mean(axis=0)
    fs0 = sim.flow_state("inflow")
    d = rng.standard_normal(7) * np.array([abs(fs0[k]) + 1.0 for k in KEYS])
    d[6] = 0.0
    pred = float(np.dot(sim.flow_state_adjoint(w)["inflow"], d))

    def residual(h):
        sim.set_flow_state("inflow", {k: fs0[k] + h * d[i] for i, k in enumerate(KEYS)})
        return sim.compute_dudt("f64")

    h = 1e-6
    fd = float(np.sum(w * (residual(h) - residual(-h))) / (2 * h))
    assert abs(fd - pred) <= 1e-5 * abs(pred), (fd, pred)


@pytest.mark.parametrize("name,kw,tag", CASES, ids=IDS)
def test_flow_state_tangent_equals_the_oracle_dual_derivative(name, kw, tag):
    """ibisgb_jvp_flow_state: the dual ghost fill and constant-flux faces seeded with
    a flow-state direction give the oracle's dual derivative to 1e-12."""
    g, c, st = make_case(name, kw)
    tag = first_tag(g, c, tag)
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    cs = copy.deepcopy(c)
    cs["solver"] = grids.steady_state()
    o = Oracle(cs, g, kind="dual")
    o.set_initial_condition(*st)
    o.steady_initialise()
    fs0 = flow_states(c, tag)[0]
    d = np.random.default_rng(29).standard_normal(7) * np.array([abs(fs0[k]) + 1.0 for k in KEYS])
    if sim.dim == 2:
        d[6] = 0.0
    jd = o.flow_state_jvp(tag, d)
    jt = sim.flow_state_tangent({tag: d})
    assert np.abs(jd).max() > 0
    assert np.abs(jt - jd).max() <= 1e-12 * np.abs(jd).max(), np.abs(jt - jd).max() / np.abs(jd).max()


def test_flow_state_derivatives_are_independent_of_the_numbering():
    g, c, st = case("tet")
    tag = next(iter(g.markers))
    out = []
    for mode in ("none", "rcm"):
        cc = copy.deepcopy(c)
        cc["grid"]["renumber"] = mode
        sim = Simulation(cc, g)
        sim.set_primitives(*st)
        assert sim.numbering()["renumbered"] == (mode == "rcm")
        U = sim.conserved()
        w = np.random.default_rng(2).standard_normal(U.shape) / np.abs(U).mean(axis=0)
        d = np.random.default_rng(6).standard_normal(7) * 100.0
        out.append((sim.flow_state_adjoint(w)[tag], sim.flow_state_tangent({tag: d})))
    for a, b in zip(out[0], out[1]):
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(a).max())


@pytest.mark.parametrize("name,tag", [("subsonic", "west"), ("cflux_ramp", "inflow")])
def test_torch_autograd_through_the_inflow_parameters(name, tag):
    """ibis_gb300.autograd.residual_flow_state: gradcheck of the state and
    inflow-parameter adjoints (the flow-state adjoint chained through rho = p / (R T),
    energy = Cv T) against central differences of the residual with the state
    installed by ibisgb_set_flow_state, in scaled variables."""
    torch = pytest.importorskip("torch")
    from ibis_gb300.autograd import residual_flow_state
    g, c, st = case(name, **({"ni": 6, "nj": 3} if name == "cflux_ramp" else {}))
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    fs = sim.flow_state(tag)
    U0 = torch.tensor(sim.conserved(), dtype=torch.float64, device="cuda")
    th0 = torch.tensor([fs["T"], fs["p"], fs["vx"], fs["vy"], fs["vz"]], dtype=torch.float64)
    su = U0.abs().mean(dim=0)
    st_ = th0.abs() + 1.0
    rs = residual_flow_state(sim, U0, th0, tag).abs().mean(dim=0)
    xu = (U0 / su).clone().requires_grad_(True)
    xt = (th0 / st_).clone().requires_grad_(True)
    f = lambda a, b: residual_flow_state(sim, a * su, b * st_, tag) / rs  # noqa: E731
    assert torch.autograd.gradcheck(f, (xu, xt), eps=1e-6, atol=1e-5, rtol=1e-4, nondet_tol=0.0, fast_mode=True)
    # forward mode: the state and flow-state tangents together, against central differences
    from torch.autograd.forward_ad import dual_level, make_dual, unpack_dual
    du, dth = torch.randn_like(U0) * su, torch.randn_like(th0) * st_
    with dual_level():
        out = residual_flow_state(sim, make_dual(U0, du), make_dual(th0, dth), tag)
        jt = unpack_dual(out).tangent
    h = 1e-7
    fd = (residual_flow_state(sim, U0 + h * du, th0 + h * dth, tag)
          - residual_flow_state(sim, U0 - h * du, th0 - h * dth, tag)) / (2 * h)
    assert torch.allclose(jt, fd, rtol=1e-5, atol=1e-5 * fd.abs().max().item())
    # the engine is left holding the last flow state it was given
    assert sim.flow_state(tag)["T"] == pytest.approx(fs["T"], rel=1e-5)
