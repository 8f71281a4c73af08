"""ibisgb_rk_run_host: Runge-Kutta runs between host buffers with the next
upload and the previous read-back on copy streams, each job's state, primitives
and first local time step formed in one pass.  Every job's output must be the
same bits as set_conserved + rk_run + get_conserved run one job after the other
(pinned and pageable buffers, renumbered grids, viscous, every precision build)."""
import copy

import numpy as np
import pytest

from ibis_gb300 import Simulation
from tests.cases import case

pytestmark = pytest.mark.gpu


def states(sim, n, seed):
    U = sim.conserved()
    rng = np.random.default_rng(seed)
    return [U * (1.0 + 0.01 * rng.standard_normal(U.shape)) for _ in range(n)]


@pytest.mark.parametrize("name,prec,pinned", [("ramp", "mixed", True), ("ramp", "f64_exact", False),
                                              ("tet", "mixed_ff", True), ("box", "f64", True),
                                              ("box", "mixed", True), ("box", "mixed_ff", True),
                                              ("plate", "mixed", True), ("subsonic", "f64", True)])
def test_pipelined_runs_equal_the_calls_one_by_one(name, prec, pinned):
    torch = pytest.importorskip("torch")
    g, c, st = case(name)
    a, b = Simulation(copy.deepcopy(c), g), Simulation(copy.deepcopy(c), g)
    for s in (a, b):
        s.set_primitives(*st)
    ins = states(a, 5, 3)
    want, ts = [], []
    for U in ins:
        a.set_conserved(U)
        ts.append(a.take_steps(2, prec)["t"])
        want.append(a.conserved())

    def buf(x=None):
        if pinned:
            t = torch.empty(x.shape if x is not None else ins[0].shape, dtype=torch.float64, pin_memory=True).numpy()
            if x is not None:
                t[...] = x
            return t
        return np.array(x) if x is not None else np.empty_like(ins[0])

    host_in = [buf(U) for U in ins]
    host_out = [buf() for _ in ins]
    st_b = b.take_steps_host(host_in, host_out, steps=2, precision=prec)
    for j in range(len(ins)):
        assert np.array_equal(host_out[j], want[j]), j
    assert st_b["t"] == ts[-1]
    assert np.array_equal(b.conserved(), want[-1])
