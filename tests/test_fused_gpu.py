"""The fused Runge-Kutta stage for structured blocks against the three-kernel
mixed path and the FP64 path: same state to rounding after several steps, on
2-D and 3-D grids with every boundary kind of the benchmark cases, and on a
batched ensemble in which one case stops early."""
import numpy as np
import pytest

from ibis_gb300 import Batch, Simulation, grids
from tests.cases import case, random_state

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name,kw", [("ramp", {}), ("ramp", {"flux": "ausmdv", "thermo": "rho_p"}),
                                     ("ramp", {"limiter": "unlimited"}), ("box", {}), ("box_inout", {}),
                                     ("box_inout", {"flux": "rusanov", "thermo": "p_T"})],
                         ids=lambda x: x if isinstance(x, str) else "-".join(f"{k}={v}" for k, v in x.items()))
def test_fused_matches_generic_mixed_and_f64(name, kw):
    steps = 12
    g, c, st = case(name, **kw)
    runs = {}
    for label, prec, fused in (("generic", "mixed", 0), ("fused", "mixed", 1), ("f64", "f64", 0)):
        sim = Simulation(c, g)
        sim.set_primitives(*st)
        sim.set_fused(fused)
        out = sim.take_steps(steps, prec)
        assert out["steps"] == steps
        if fused:
            assert sim.fused_info()["enabled"]
        runs[label] = (sim.conserved(), out)
    U_f, o_f = runs["fused"]
    U_g, o_g = runs["generic"]
    U_d, o_d = runs["f64"]
    for q in range(U_f.shape[1]):
        assert _rel(U_f[:, q], U_d[:, q]) <= 1e-6, q
        assert _rel(U_f[:, q], U_g[:, q]) <= 1e-6, q
    assert o_f["t"] == pytest.approx(o_d["t"], rel=1e-6)


def test_fused_odd_step_counts_and_switching():
    """Primitive buffers alternate between fused stages; switching paths and
    stopping on odd step counts must keep one consistent state."""
    g, c, st = case("box")
    a, b = Simulation(c, g), Simulation(c, g)
    for s in (a, b):
        s.set_primitives(*st)
    a.set_fused(1)
    b.set_fused(0)
    for n in (1, 2, 3):
        a.take_steps(n, "mixed")
        b.take_steps(n, "mixed")
        assert _rel(a.conserved()[:, 0], b.conserved()[:, 0]) <= 1e-6
        assert _rel(a.primitives()["p"], b.primitives()["p"]) <= 1e-6
    a.set_fused(0)  # continue the fused state on the generic kernels
    a.take_steps(2, "mixed")
    b.take_steps(2, "mixed")
    assert _rel(a.conserved()[:, 0], b.conserved()[:, 0]) <= 1e-6


def test_fused_batch_with_a_halted_case():
    ens = grids.ramp_ensemble(4, seed=11, smallest=(16, 8), largest=(64, 32))
    res = {}
    for fused in (0, 1):
        sims, states = [], []
        for k, (gg, cc, inf, _) in enumerate(ens):
            cc = dict(cc, solver=dict(cc["solver"]))
            if k == 2:
                cc["solver"]["max_time"] = 6e-6
            sims.append(Simulation(cc, gg))
            states.append(random_state(gg.num_cells, inf["T"], inf["p"], inf["vx"], 2, seed=20 + k, amp=0.03))
        b = Batch(sims)
        b.set_primitives(*[np.concatenate([s[q] for s in states]) for q in range(4)])
        b.set_fused(fused)
        b.take_steps(9, "mixed")
        res[fused] = (b.split(b.conserved()), b.case_status())
    (Ug, sg), (Uf, sf) = res[0], res[1]
    for k in range(4):
        assert sf[k]["steps"] == sg[k]["steps"]
        assert sf[k]["t"] == pytest.approx(sg[k]["t"], rel=1e-6)
        assert _rel(Uf[k][:, 0], Ug[k][:, 0]) <= 1e-6
    assert sf[2]["steps"] < 9
