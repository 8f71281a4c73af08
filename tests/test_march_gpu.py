"""The plane-marching fused stage (one 3-D structured block, planes staged into
shared memory by TMA copies) against the tile-fused stage, the three-kernel
mixed path and the FP64 path: same state to rounding after several steps, on
boxes whose extents are not multiples of the 32 x 8 column or of the chunk of
planes, with periodic, supersonic in/out and slip-wall boundaries."""
import numpy as np
import pytest

from ibis_gb300 import Simulation
from tests.cases import case

pytestmark = pytest.mark.gpu

CASES = [
    ("box_ragged", {}),
    ("box_ragged", {"flux": "ausmdv", "thermo": "rho_p"}),
    ("box_inout", {"n": (36, 12, 10)}),
    ("box_inout", {"n": (36, 12, 10), "flux": "rusanov", "thermo": "p_T"}),
    ("box_inout", {"n": (40, 10, 7), "flux": "ldfss2", "limiter": "unlimited"}),
    ("box", {"n": 32}),
]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _run(name, kw, steps, prec="mixed", fused=0, kind=-1, kc=0, max_time=None):
    g, c, st = case(name, **kw)
    if max_time is not None:
        c = dict(c, solver=dict(c["solver"], max_time=max_time))
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    sim.set_fused(fused)
    if fused:
        sim.set_fused_kind(kind, kc)
    out = sim.take_steps(steps, prec)
    return sim, out


@pytest.mark.parametrize("name,kw", CASES,
                         ids=lambda x: x if isinstance(x, str) else "-".join(f"{k}={v}" for k, v in x.items()))
def test_march_matches_tile_generic_and_f64(name, kw):
    steps = 8
    m, om = _run(name, kw, steps, fused=1, kind=1, kc=4)
    assert m.fused_kind()["march"] and m.fused_info()["enabled"]
    t, ot = _run(name, kw, steps, fused=1, kind=0)
    assert not t.fused_kind()["march"]
    g, og = _run(name, kw, steps, fused=0)
    d, od = _run(name, kw, steps, prec="f64")
    for o in (om, ot, og, od):
        assert o["steps"] == steps and o["bad_cells"] == 0
    Um, Ut, Ug, Ud = m.conserved(), t.conserved(), g.conserved(), d.conserved()
    for q in range(Um.shape[1]):
        assert _rel(Um[:, q], Ut[:, q]) <= 1e-6, q
        assert _rel(Um[:, q], Ug[:, q]) <= 1e-6, q
        assert _rel(Um[:, q], Ud[:, q]) <= 1e-6, q
    assert om["t"] == pytest.approx(od["t"], rel=1e-6)
    pm, pg = m.primitives(), g.primitives()
    assert _rel(pm["p"], pg["p"]) <= 1e-6


def test_march_chunk_length_does_not_change_the_bits():
    """Each CTA recomputes the gradients and the k-face below its first plane; any
    number of planes per CTA gives the same state bit for bit."""
    ref = None
    for kc in (1, 2, 3, 4, 16):
        sim, out = _run("box_ragged", {}, 5, fused=1, kind=1, kc=kc)
        assert sim.fused_kind()["planes_per_cta"] == kc
        U = sim.conserved()
        if ref is None:
            ref = U
        else:
            assert np.array_equal(U, ref), kc


def test_march_odd_steps_switching_and_halt():
    """Primitive buffers alternate between stages; stopping on odd step counts,
    switching to the generic kernels and halting at max_time keep one state."""
    a, _ = _run("box_ragged", {}, 0, fused=1, kind=1, kc=4)
    b, _ = _run("box_ragged", {}, 0, fused=0)
    for n in (1, 2, 3):
        a.take_steps(n, "mixed")
        b.take_steps(n, "mixed")
        assert _rel(a.conserved()[:, 0], b.conserved()[:, 0]) <= 1e-6
        assert _rel(a.primitives()["p"], b.primitives()["p"]) <= 1e-6
    a.set_fused(0)
    a.take_steps(2, "mixed")
    b.take_steps(2, "mixed")
    assert _rel(a.conserved()[:, 0], b.conserved()[:, 0]) <= 1e-6
    # a max_time reached after a few steps halts both paths at the same step
    probe, o1 = _run("box_ragged", {}, 1, fused=0)
    tmax = 3.5 * o1["dt"]
    hm, om = _run("box_ragged", {}, 10, fused=1, kind=1, kc=4, max_time=tmax)
    hg, og = _run("box_ragged", {}, 10, fused=0, max_time=tmax)
    assert om["steps"] == og["steps"] < 10
    assert om["t"] == pytest.approx(og["t"], rel=1e-9)
    assert _rel(hm.conserved()[:, 0], hg.conserved()[:, 0]) <= 1e-6
    assert _rel(hm.primitives()["rho"], hg.primitives()["rho"]) <= 1e-6


def test_march_autotuner_times_both_kernels():
    g, c, st = case("box", n=32)
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    sim.set_fused(-1)
    sim.take_steps(1, "mixed")
    k = sim.fused_kind()
    assert k["march_eligible"] and k["tile_ms"] > 0 and k["march_ms"] > 0
    assert k["planes_per_cta"] in (16, 32, 64)
