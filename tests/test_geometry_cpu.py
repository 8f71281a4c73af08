"""ibis_gb300.geometry (the grid geometry on numpy arrays, for complex-step
derivatives along vertex displacements) against the engine's own geometry
dumps, and its complex-step derivative against central differences of the
engine's geometry on a displaced grid (no GPU: grids are preprocessed on the
host)."""
import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from ibis_gb300.adjoint import bump_displacements
from ibis_gb300.geometry import GridTopology
from tests.cases import case


@pytest.mark.parametrize("name", ["ramp", "tri", "tiny2d", "tet", "wedge", "pyramid", "box", "box_inout", "plate"])
def test_geometry_equals_the_engine(name):
    g, c, _ = case(name)
    sim = Simulation(c, g)
    face, cell = GridTopology(sim, g).geometry(g.xyz)
    fg, cg = sim.dump("face_geometry"), sim.dump("cell_geometry")
    assert np.abs(face - fg).max() <= 1e-15 * max(1.0, np.abs(fg).max())
    assert np.abs(cell - cg).max() <= 1e-15 * max(1.0, np.abs(cg).max())


def test_complex_step_derivative_of_a_bump():
    bumps = np.random.default_rng(0).uniform(-0.002, 0.002, 16)
    _, c, _ = grids.ramp_bump_case(24, 12, bumps=bumps)
    g = grids.ramp_2d_bumps(24, 12, bumps=bumps)
    topo = GridTopology(Simulation(c, g), g)
    dx = bump_displacements(24, 12)[5]
    df, dc = topo.directional_derivative(g.xyz, dx)
    h = 1e-6
    fp, cp = topo.geometry(g.xyz + h * dx)
    fm, cm = topo.geometry(g.xyz - h * dx)
    assert np.abs(df).max() > 0
    assert np.allclose(df, (fp - fm) / (2 * h), rtol=1e-6, atol=1e-9 * np.abs(df).max())
    assert np.allclose(dc, (cp - cm) / (2 * h), rtol=1e-6, atol=1e-9 * np.abs(dc).max())
