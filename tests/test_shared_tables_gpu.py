"""Shared geometry tables on uniform lattices (grid.geometry_tables "auto"):
least-squares weights and face offsets stored once per face slot, and the float
build's face classes (one-byte class per face into shared rows of normal and
side offsets).  The same bits as the per-element tables ("per_element") in every
arithmetic -- residual, limiter values and branches, Runge-Kutta steps -- on
the periodic box and a 2-D channel whose cells are all alike, and per-element
tables wherever the cells differ."""
import copy

import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from tests.cases import case, random_state

pytestmark = pytest.mark.gpu


def uniform_channel():
    """16 x 8 equal squares (spacing 1/16, exact in binary): supersonic in/out, slip walls."""
    X, Y = np.meshgrid(np.linspace(0, 1, 17), np.linspace(0, 0.5, 9), indexing="ij")
    g = grids.structured_2d(X, Y)
    gas = grids.ideal_gas(287.0)
    inflow = grids.flow_state(gas, 300.0, 1e5, 700.0, 40.0)
    b = {"west": grids.supersonic_inflow(inflow), "east": grids.supersonic_outflow(),
         "south": grids.slip_wall(), "north": grids.slip_wall()}
    c = grids.make_config(2, b, gas=gas)
    return g, c, random_state(g.num_cells, 300.0, 1e5, 700.0, 2, seed=12, amp=0.05)


def pair(g, c, st):
    out = []
    for mode in ("auto", "per_element"):
        cc = copy.deepcopy(c)
        cc["grid"]["geometry_tables"] = mode
        sim = Simulation(cc, g)
        sim.set_primitives(*st)
        out.append(sim)
    return out


@pytest.mark.parametrize("which", ["box8", "box16_4", "channel2d"])
def test_shared_tables_give_the_same_bits(which):
    if which == "channel2d":
        g, c, st = uniform_channel()
    else:
        n, nz = (8, 8) if which == "box8" else (16, 4)
        g, c = grids.box_case(n, ny=n, nz=nz)
        st = grids.box_initial_condition(n, c["gas_model"], seed=3) if nz == n else \
            random_state(g.num_cells, 1.0, 1.0, 0.3, 3, seed=13, amp=0.05)
    a, b = pair(g, c, st)
    for prec in ("mixed", "mixed_ff", "f64"):
        ta, tb = a.shared_tables(prec), b.shared_tables(prec)
        assert ta["lsq_shared"] and not tb["lsq_shared"] and tb["face_classes"] == 0, prec
        assert (0 < ta["face_classes"] <= 64) == (prec == "mixed"), (prec, ta)
        assert np.array_equal(a.compute_dudt(prec), b.compute_dudt(prec)), prec
    a.compute_dudt("mixed")
    b.compute_dudt("mixed")
    for d in ("limiter_branches", "limiters"):
        assert np.array_equal(a.dump(d), b.dump(d)), d
    for prec in ("mixed", "mixed_ff", "f64"):
        for s in (a, b):
            s.set_primitives(*st)
            s.take_steps(3, prec)
        assert np.array_equal(a.conserved(), b.conserved()), prec


@pytest.mark.parametrize("name", ["ramp", "tet", "plate"])
def test_cells_that_differ_keep_per_cell_tables(name):
    """Cells that differ keep per-cell least-squares tables; faces keep classes only
    where at most 64 distinct rows exist, and either way the bits do not change."""
    g, c, st = case(name)
    a, b = pair(g, c, st)
    for prec in ("mixed", "mixed_ff", "f64"):
        assert not a.shared_tables(prec)["lsq_shared"], prec
        assert np.array_equal(a.compute_dudt(prec), b.compute_dudt(prec)), prec
    if name == "ramp":
        assert a.shared_tables("mixed")["face_classes"] == 0
