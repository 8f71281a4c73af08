"""Host side of the internal cell / face numbering (no GPU needed: the grid is
preprocessed on the host when a context is created).

* "rcm" renumbers and every grid dump (connectivity, geometry, ghost maps) in the
  reference's numbering equals the un-renumbered context's, bit for bit;
* the internal order is a permutation and the reverse Cuthill-McKee order
  shortens the cell graph's bandwidth;
* "auto" renumbers tetrahedral grids (shuffled or not) where that halves the
  bandwidth, and leaves quadrilateral and hexahedral grids in their own order;
* an unknown "renumber" value is a config error."""
import copy

import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from ibis_gb300._lib import IbisgbError
from tests.cases import case

DUMPS = ["left", "right", "cell_faces", "outsigns", "neighbours", "ghost_source", "face_geometry",
         "cell_geometry", "ghost_face", "ghost_boundary"]


def with_mode(c, mode):
    c = copy.deepcopy(c)
    c["grid"]["renumber"] = mode
    return c


@pytest.mark.parametrize("name", ["ramp", "tri", "tet", "wedge", "pyramid", "box", "plate", "subsonic", "bl_plate"])
def test_rcm_keeps_every_grid_array_in_the_reference_numbering(name):
    g, c, _ = case(name)
    a, b = Simulation(with_mode(c, "none"), g), Simulation(with_mode(c, "rcm"), g)
    ia, ib = a.numbering(), b.numbering()
    assert not ia["renumbered"] and ib["renumbered"]
    assert ib["bandwidth_reference"] == ia["bandwidth_reference"]
    assert ib["bandwidth_internal"] <= ib["bandwidth_reference"]
    order, forder = b.dump("cell_order"), b.dump("face_order")
    assert np.array_equal(np.sort(order), np.arange(b.num_cells))
    assert np.array_equal(np.sort(forder), np.arange(b.num_faces))
    assert np.array_equal(a.dump("cell_order"), np.arange(a.num_cells))
    for d in DUMPS:
        assert np.array_equal(a.dump(d), b.dump(d)), d


def test_auto_mode():
    g, c, _ = grids.tet_channel_case(8, shuffle_seed=0)
    info = Simulation(c, g).numbering()
    assert info["renumbered"] and 4 * info["bandwidth_internal"] <= info["bandwidth_reference"], info
    for name in ("ramp", "box", "plate"):
        g, c, _ = case(name)
        assert not Simulation(c, g).numbering()["renumbered"], name
    g, c, _ = case("ramp")
    with pytest.raises(IbisgbError):
        Simulation(with_mode(c, "sideways"), g)
