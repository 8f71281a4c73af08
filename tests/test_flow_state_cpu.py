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
