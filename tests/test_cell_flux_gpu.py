"""The per-cell flux path of the mixed build (each cell recomputes its faces'
convective fluxes inside the update kernel) gives the same bits as the
three-kernel stage: Runge-Kutta steps on every grid kind, a batch with a case
that halts early, and every launch variant."""
import numpy as np
import pytest

from ibis_gb300 import Batch, Simulation, grids
from tests.cases import case, random_state

pytestmark = pytest.mark.gpu


def _pair(name, **kw):
    g, c, st = case(name, **kw)
    a, b = Simulation(c, g), Simulation(c, g)
    for s in (a, b):
        s.set_primitives(*st)
        s.set_fused(0)
    a.set_cell_flux(0)
    b.set_cell_flux(1)
    return a, b


@pytest.mark.parametrize("name,kw", [("ramp", {}), ("ramp", {"order": 1}), ("ramp", {"flux": "ausmdv"}),
                                     ("ramp", {"flux": "ldfss2"}), ("box", {}), ("box_inout", {}), ("tri", {}),
                                     ("tet", {}), ("wedge", {}), ("pyramid", {}), ("tiny2d", {}), ("tiny3d", {})],
                         ids=lambda x: x if isinstance(x, str) else "-".join(f"{k}={v}" for k, v in x.items()))
def test_cell_flux_steps_are_bit_identical(name, kw):
    a, b = _pair(name, **kw)
    assert b.cell_flux_info()["enabled"]
    for n in (1, 4):  # an odd and an even number of steps (the primitive buffers alternate)
        sa, sb = a.take_steps(n, "mixed"), b.take_steps(n, "mixed")
        assert sa["dt"] == sb["dt"] and sa["t"] == sb["t"]
        assert np.array_equal(a.conserved(), b.conserved())
        # the primitives the other entry points read are the current ones
        assert np.array_equal(a.compute_dudt("mixed"), b.compute_dudt("mixed"))


def test_cell_flux_every_variant_and_the_autotuner():
    g, c, st = case("box", n=8)
    ref = None
    for w in range(len(Simulation.launch_variants())):
        s = Simulation(c, g)
        s.set_primitives(*st)
        s.set_fused(0)
        s.set_launch_variants("mixed", w, w, w)
        s.set_cell_flux(1)
        s.take_steps(3, "mixed")
        assert s.cell_flux_info()["variant"] == w
        U = s.conserved()
        ref = U if ref is None else ref
        assert np.array_equal(U, ref), w
    s = Simulation(c, g)
    s.set_primitives(*st)
    s.set_fused(0)
    s.autotune("mixed")
    info = s.cell_flux_info()
    assert info["eligible"] and info["cell_ms"] > 0 and info["generic_ms"] > 0
    s.take_steps(3, "mixed")
    assert np.array_equal(s.conserved(), ref)


def test_cell_flux_in_a_batch_with_a_halting_case():
    ens = grids.ramp_ensemble(3, seed=5, smallest=(16, 8), largest=(48, 24))
    sims, states = [], []
    for k, (g, c, inf, _) in enumerate(ens):
        if k == 1:
            c["solver"]["max_time"] = 6e-6
        s = Simulation(c, g)
        st = random_state(g.num_cells, inf["T"], inf["p"], inf["vx"], 2, seed=40 + k, amp=0.03)
        s.set_primitives(*st[:4])
        sims.append(s)
        states.append(st)
    b1, b2 = Batch(sims), Batch(sims)
    for b in (b1, b2):
        b.set_primitives(*[np.concatenate([st[q] for st in states]) for q in range(4)])
        b.set_fused(0)
    b1.set_cell_flux(0)
    b2.set_cell_flux(1)
    b1.take_steps(9, "mixed")
    b2.take_steps(9, "mixed")
    assert [p["steps"] for p in b1.case_status()] == [p["steps"] for p in b2.case_status()]
    assert b2.case_status()[1]["steps"] < 9
    assert np.array_equal(b1.conserved(), b2.conserved())


@pytest.mark.parametrize("name", ["plate", "cflux_ramp"])
def test_cell_flux_is_refused_where_it_does_not_apply(name):
    from ibis_gb300._lib import IbisgbError
    g, c, st = case(name)
    s = Simulation(c, g)
    assert not s.cell_flux_info()["eligible"]
    with pytest.raises(IbisgbError):
        s.set_cell_flux(1)
