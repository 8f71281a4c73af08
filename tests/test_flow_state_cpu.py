"""The oracle's derivative with respect to a boundary's flow state (orc_flow_state_jvp:
the reference's Dual seeded in every action of the boundary that carries one --
flow_state_copy, subsonic_inflow, constant_flux -- before reconstruction and
before the viscous gradients) against central differences of the oracle's real
residual on configs whose flow state is perturbed: the check of the oracle
itself that the engine's flow-state adjoint is tested against."""
import copy

import numpy as np
import pytest

from ibis_gb300 import grids
from oracle.oracle import Oracle
from tests.cases import case

KEYS = ("T", "p", "rho", "energy", "vx", "vy", "vz")


def flow_states(config, tag):
    """The distinct flow_state objects of boundary `tag` (one dict may serve several actions)."""
    b = config["grid"]["boundaries"][tag]
    out = {}
    for lst in ("pre_reconstruction", "post_convective_flux", "pre_viscous_grad"):
        for a in b[lst]:
            if "flow_state" in a:
                out[id(a["flow_state"])] = a["flow_state"]
    return list(out.values())


def with_viscous_inflow(c):
    """The flat plate's inflow with its flow state copied before the viscous gradients too."""
    fs = c["grid"]["boundaries"]["inflow"]["pre_reconstruction"][0]["flow_state"]
    c["grid"]["boundaries"]["inflow"]["pre_viscous_grad"] = [{"type": "flow_state_copy", "flow_state": fs}]
    return c


CASES = [("ramp", {}, "inflow"), ("ramp", {"order": 1}, "inflow"), ("subsonic", {}, "west"),
         ("cflux_ramp", {}, "inflow"), ("cflux_box", {}, "top"), ("box_inout", {}, "west"),
         ("plate", {"viscous_inflow": True}, "inflow")]
IDS = [f"{n}-{t}" + "".join(f"-{k}={v}" for k, v in kw.items()) for n, kw, t in CASES]


def make_case(name, kw):
    kw = dict(kw)
    visc_in = kw.pop("viscous_inflow", False)
    g, c, st = case(name, **kw)
    if visc_in:
        c = with_viscous_inflow(c)
    return g, c, st


@pytest.mark.parametrize("name,kw,tag", CASES, ids=IDS)
def test_oracle_flow_state_derivative_matches_central_differences(name, kw, tag):
    g, c, st = make_case(name, kw)
    cs = copy.deepcopy(c)
    cs["solver"] = grids.steady_state()
    o = Oracle(cs, g, kind="dual")
    o.set_initial_condition(*st)
    o.steady_initialise()
    fs0 = flow_states(c, tag)[0]
    d = np.random.default_rng(3).standard_normal(7) * np.array([abs(fs0[k]) + 1.0 for k in KEYS])
    jd = o.flow_state_jvp(tag, d)

    def residual(h):
        cc = copy.deepcopy(c)
        for fs in flow_states(cc, tag):
            for k, key in enumerate(KEYS):
                fs[key] += h * d[k]
        r = Oracle(cc, g)
        r.set_initial_condition(*st)
        return r.residual().reshape(jd.shape)

    h = 1e-6
    fd = (residual(h) - residual(-h)) / (2 * h)
    assert np.abs(jd).max() > 0
    assert np.abs(jd - fd).max() <= 1e-7 * np.abs(jd).max()


def test_set_flow_state_on_the_host():
    """ibisgb_set_flow_state / ibisgb_get_flow_state before the device is used: every
    action of the boundary that carries a flow state takes the new one (the pre-
    reconstruction copy and the constant flux of the same boundary), and bad calls
    are refused with the C ABI's error codes and leave the state unchanged."""
    from ibis_gb300 import Batch, Simulation
    from ibis_gb300._lib import IbisgbError
    g, c, _ = case("cflux_ramp")
    sim = Simulation(c, g)
    fs = sim.flow_state("inflow")
    assert fs == {k: float(c["grid"]["boundaries"]["inflow"]["pre_reconstruction"][0]["flow_state"][k])
                  for k in KEYS}
    new = grids.flow_state(c["gas_model"], 310.0, 0.9e5, 650.0, 20.0)
    sim.set_flow_state("inflow", new)
    assert sim.flow_state("inflow") == {k: float(new[k]) for k in KEYS}
    for tag, state in (("nowhere", new), ("outflow", new), ("inflow", dict(new, T=float("inf")))):
        with pytest.raises(IbisgbError, match="ARG"):
            sim.set_flow_state(tag, state)
    assert sim.flow_state("inflow") == {k: float(new[k]) for k in KEYS}
    b = Batch([Simulation(c, g), Simulation(c, g)])
    with pytest.raises(IbisgbError, match="STATE"):
        b.set_flow_state("inflow", new)
