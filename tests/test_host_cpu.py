"""Host side of libibisgb without a GPU: the C ABI exports what include/ibisgb.h
declares, config/grid errors come back as error codes, and the host grid
preprocessing reproduces the reference's numbering and geometry bit for bit
(checked against the oracle and the reference's golden vectors)."""
import os

import numpy as np
import pytest

from ibis_gb300 import Simulation, _lib, grids
from ibis_gb300._lib import IbisgbError
from oracle.oracle import Oracle
from tests.cases import case


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    syms = _lib.header_symbols()
    assert len(syms) >= 16
    for s in syms:
        assert hasattr(L, s), s


@pytest.mark.parametrize("name", ["ramp", "plate", "box", "box_inout", "subsonic", "tri", "tet", "wedge", "pyramid",
                                  "tiny2d", "tiny3d", "bl_plate", "cflux_box"])
def test_numbering_and_geometry_match_oracle(name):
    g, c, _ = case(name)
    sim, o = Simulation(c, g), Oracle(c, g)
    assert (sim.num_cells, sim.num_ghost_cells, sim.num_faces) == (o.N, o.G, o.F)
    conn = o.connectivity()
    for k in ("left", "right"):
        assert np.array_equal(sim.dump(k), conn[k]), k
    assert np.array_equal(sim.dump("cell_faces"), conn["cell_faces"])
    assert np.array_equal(sim.dump("outsigns"), conn["outsigns"])
    assert np.array_equal(sim.dump("neighbours"), conn["neighbours"])
    geo = o.geometry()
    fg, cg = sim.dump("face_geometry"), sim.dump("cell_geometry")
    assert np.array_equal(fg[0:3], geo["normal"]) and np.array_equal(fg[3:6], geo["tan1"])
    assert np.array_equal(fg[6:9], geo["tan2"]) and np.array_equal(fg[9:12], geo["centre"])
    assert np.array_equal(fg[12], geo["area"])
    assert np.array_equal(cg[0:3], geo["centroid"]) and np.array_equal(cg[3], geo["volume"])


def test_golden_vectors_through_the_product(golden):
    bnds = {t: grids.slip_wall() for t in ["slip_wall_bottom", "slip_wall_top", "inflow", "outflow"]}
    sim = Simulation(grids.make_config(2, bnds), grids.unit_square_3x3())
    assert sim.dump("cell_faces").tolist() == golden["grid_cell_faces"]["face_ids"]
    assert sim.dump("outsigns").tolist() == golden["grid_outsigns"]["outsigns"]
    nb = sim.dump("neighbours")
    for c, slot, n in golden["cell_neighbours"]["checks"]:
        assert nb[c, slot] == n
    cg = sim.dump("cell_geometry")
    # ghost ids follow sorted tag order: inflow, outflow, slip_wall_bottom, slip_wall_top
    start = sim.num_cells
    for tag in ["inflow", "outflow", "slip_wall_bottom", "slip_wall_top"]:
        expected = np.array(golden["ghost_cell_centres"][tag])
        assert np.array_equal(cg[0:3, start:start + 3].T, expected), tag
        start += 3


def test_su2_file_and_arrays_agree(tmp_path):
    g, c, _ = case("ramp")
    path = os.path.join(tmp_path, "block_0000.su2")
    g.write(path)
    a, b = Simulation(c, g), Simulation(c, path)
    for k in ("left", "right", "cell_faces", "outsigns", "neighbours", "face_geometry", "cell_geometry"):
        assert np.array_equal(a.dump(k), b.dump(k)), k


def test_periodic_ghost_sources():
    g, c, _ = case("box", n=4)
    sim = Simulation(c, g)
    src = sim.dump("ghost_source")
    cg = sim.dump("cell_geometry")
    N = sim.num_cells
    # a periodic ghost's source is the valid cell one box length away from the ghost
    d = cg[0:3, N:] - cg[0:3, src]
    assert np.allclose(np.sort(np.abs(d), axis=0)[-1], 1.0)


def test_errors_come_back_as_codes(tmp_path):
    g, c, _ = case("ramp")
    bad = dict(c)
    bad["convective_flux"] = dict(c["convective_flux"], flux_calculator={"type": "roe"})
    with pytest.raises(IbisgbError) as e:
        Simulation(bad, g)
    assert e.value.code == -1 and "roe" in str(e.value)
    with pytest.raises(IbisgbError) as e:
        Simulation(c, os.path.join(tmp_path, "missing.su2"))
    assert e.value.code == -2
    missing_bc = dict(c)
    missing_bc["grid"] = dict(c["grid"], boundaries={k: v for k, v in c["grid"]["boundaries"].items() if k != "wall"})
    with pytest.raises(IbisgbError):
        Simulation(missing_bc, g)


def test_flux_and_profile_action_errors():
    """Unknown flux actions and short spline profiles are configuration errors,
    as build_flux_action and the CubicSpline constructor throw (boundary.cpp:481-492,
    cubic_spline.cpp:12-19)."""
    import copy
    g, c, _ = case("bl_plate")
    bad = copy.deepcopy(c)
    bad["grid"]["boundaries"]["north"]["post_convective_flux"][0]["type"] = "shock_fit"
    with pytest.raises(IbisgbError) as e:
        Simulation(bad, g)
    assert e.value.code == -1 and "shock_fit" in str(e.value)
    short = copy.deepcopy(c)
    prof = short["grid"]["boundaries"]["west"]["pre_reconstruction"][0]["profile"]
    for k in ("height", "v", "T"):
        prof[k] = prof[k][:3]
    with pytest.raises(IbisgbError) as e:
        Simulation(short, g)
    assert e.value.code == -1 and "Insufficient points" in str(e.value)


def test_state_calls_before_initial_condition_are_rejected():
    g, c, _ = case("ramp")
    sim = Simulation(c, g)
    with pytest.raises(IbisgbError) as e:
        sim.primitives()
    assert e.value.code == -7
