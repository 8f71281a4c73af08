"""Structured-block recognition for the fused stage, on the host (no GPU):
every grid the structured generators write qualifies, batches of them too,
and anything else is refused with a reason."""
import numpy as np
import pytest

from ibis_gb300 import Batch, Simulation, grids
from tests.cases import case


def test_structured_grids_qualify():
    for name in ("ramp", "box", "box_inout"):
        g, c, _ = case(name)
        info = Simulation(c, g).fused_info()
        assert info["eligible"], (name, info["reason"])
        assert not info["enabled"]


def test_batches_of_structured_cases_qualify():
    ens = grids.ramp_ensemble(3, seed=3, smallest=(8, 4), largest=(24, 12))
    b = Batch([Simulation(c, g) for g, c, _, _ in ens])
    assert b.fused_info()["eligible"]


def test_other_grids_and_schemes_are_refused():
    g, c, _ = case("plate")
    info = Simulation(c, g).fused_info()
    assert not info["eligible"] and "viscous" in info["reason"]
    g, c, _ = case("ramp", order=1)
    assert "first-order" in Simulation(c, g).fused_info()["reason"]
    # the same ramp with its cells renumbered is no longer a lattice
    g, c, _ = case("ramp")
    perm = np.random.default_rng(0).permutation(g.num_cells)
    n = g.cell_offsets[1:] - g.cell_offsets[:-1]
    conn = [g.cell_conn[g.cell_offsets[k]:g.cell_offsets[k + 1]] for k in range(g.num_cells)]
    g.cell_conn = np.concatenate([conn[k] for k in perm])
    g.cell_types = g.cell_types[perm]
    g.cell_offsets = np.concatenate([[0], np.cumsum(n[perm])])
    info = Simulation(c, g).fused_info()
    assert not info["eligible"] and info["reason"]
    g = grids.unit_square_3x3()
    bnds = {t: grids.slip_wall() for t in ["slip_wall_bottom", "slip_wall_top", "inflow", "outflow"]}
    assert Simulation(grids.make_config(2, bnds), g).fused_info()["eligible"]


def test_plane_marching_kernel_eligibility():
    """The plane-marching kernel takes one 3-D block whose i-extent and N+G are
    multiples of 4 (TMA copies start on 16-byte boundaries); the host says why not."""
    for name, kw in (("box", {"n": 8}), ("box_ragged", {}), ("box_inout", {"n": (36, 12, 10)})):
        g, c, _ = case(name, **kw)
        k = Simulation(c, g).fused_kind()
        assert k["march_eligible"], (name, k["reason"])
        assert not k["march"]
    g, c, _ = case("box", n=6)
    k = Simulation(c, g).fused_kind()
    assert not k["march_eligible"] and "multiples of 4" in k["reason"]
    g, c, _ = case("ramp")
    k = Simulation(c, g).fused_kind()
    assert not k["march_eligible"] and "three-dimensional" in k["reason"]
    g, c, _ = case("plate")
    assert "viscous" in Simulation(c, g).fused_kind()["reason"]


def test_fused_kind_rejects_bad_arguments_on_the_host():
    """ibisgb_set_fused_kind checks its arguments and the eligibility of the
    plane-marching kernel before touching a GPU."""
    from ibis_gb300._lib import IbisgbError
    g, c, _ = case("ramp")
    sim = Simulation(c, g)
    for kind, planes in ((2, 0), (-2, 0), (0, -1)):
        with pytest.raises(IbisgbError) as e:
            sim.set_fused_kind(kind, planes)
        assert e.value.code == -5, (kind, planes)
    with pytest.raises(IbisgbError) as e:
        sim.set_fused_kind(1, 0)  # a 2-D grid: the plane-marching kernel does not apply
    assert e.value.code == -5 and "three-dimensional" in str(e.value)
    g, c, _ = case("box", n=6)
    with pytest.raises(IbisgbError) as e:
        Simulation(c, g).set_fused_kind(1, 16)
    assert "multiples of 4" in str(e.value)
