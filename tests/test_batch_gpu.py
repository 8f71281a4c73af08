"""Batched ensembles on the GPU: one context holding several independent ramp
cases of different sizes, inflow states and ramp angles gives, case by case,
exactly the results of running each case alone (residuals, Runge-Kutta steps
with per-case dt and halting, tangent products)."""
import numpy as np
import pytest

from ibis_gb300 import Batch, Simulation, grids
from tests.cases import random_state

pytestmark = pytest.mark.gpu


def _ensemble(short_case=None):
    ens = grids.ramp_ensemble(4, seed=11, smallest=(16, 8), largest=(64, 32))
    sims, states = [], []
    for k, (g, c, inf, _) in enumerate(ens):
        if k == short_case:
            c["solver"]["max_time"] = 6e-6  # about four steps of this case
        sims.append(Simulation(c, g))
        states.append(random_state(g.num_cells, inf["T"], inf["p"], inf["vx"], 2, seed=20 + k, amp=0.03))
    for s, st in zip(sims, states):
        s.set_primitives(*st[:4])
    b = Batch(sims)
    b.set_primitives(*[np.concatenate([st[q] for st in states]) for q in range(4)])
    return sims, b


@pytest.mark.parametrize("precision", ["f64_exact", "f64", "mixed", "mixed_grad", "mixed_ff"])
def test_batch_residual_equals_cases(precision):
    sims, b = _ensemble()
    r = b.compute_dudt(precision)
    for s, rb in zip(sims, b.split(r)):
        assert np.array_equal(rb, s.compute_dudt(precision))


@pytest.mark.parametrize("precision", ["f64_exact", "mixed", "mixed_ff"])
def test_batch_rk_steps_equal_cases(precision):
    steps = 8
    sims, b = _ensemble(short_case=2)
    st = b.take_steps(steps, precision)
    per = b.case_status()
    U = b.split(b.conserved())
    for k, s in enumerate(sims):
        o = s.take_steps(steps, precision)
        assert per[k]["steps"] == o["steps"]
        assert per[k]["t"] == o["t"] and per[k]["dt"] == o["dt"]
        assert np.array_equal(U[k], s.conserved()), k
    assert per[2]["steps"] < steps  # max_time reached early; the other cases went on
    assert st["steps"] == steps and st["t"] == min(p["t"] for p in per)


def test_batch_estimate_dt_and_jvp():
    sims, b = _ensemble()
    assert b.estimate_dt() == min(s.estimate_dt() for s in sims)
    rng = np.random.default_rng(5)
    v = rng.standard_normal((b.num_cells, b.n_conserved))
    out = b.matrix_vector_product(v, 1e3)
    for s, vb, ob in zip(sims, b.split(v), b.split(out)):
        assert np.array_equal(ob, s.matrix_vector_product(vb, 1e3))


def test_batch_with_profile_and_constant_flux_boundaries():
    """Each case keeps its own boundary-layer profile table and constant-flux
    state when merged into a batch."""
    from tests.cases import case
    sims, states = [], []
    for k, scale in enumerate([1.0, 0.8, 1.1]):
        g, c, st = case("bl_plate")
        prof = c["grid"]["boundaries"]["west"]["pre_reconstruction"][0]["profile"]
        prof["v"] = [scale * x for x in prof["v"]]
        c["grid"]["boundaries"]["north"]["post_convective_flux"][0]["flow_state"]["vx"] *= scale
        sims.append(Simulation(c, g))
        sims[-1].set_primitives(*st[:4])
        states.append(st)
    b = Batch(sims)
    b.set_primitives(*[np.concatenate([st[q] for st in states]) for q in range(4)])
    for prec in ("f64_exact", "mixed"):
        r = b.compute_dudt(prec)
        for s, rb in zip(sims, b.split(r)):
            assert np.array_equal(rb, s.compute_dudt(prec)), prec
    b.take_steps(3, "f64_exact")
    for s, Ub in zip(sims, b.split(b.conserved())):
        s.take_steps(3, "f64_exact")
        assert np.array_equal(Ub, s.conserved())
