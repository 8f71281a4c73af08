"""Batched ensembles without a GPU: the merged context's numbering is each
case's numbering shifted by the case offsets (valid cells of all cases first,
then all ghost cells), its geometry is the cases' geometry, and inconsistent
batches are refused with the C ABI's error codes."""
import numpy as np
import pytest

from ibis_gb300 import Batch, Simulation, grids
from ibis_gb300._lib import IbisgbError
from tests.cases import case


def _cases():
    ens = grids.ramp_ensemble(3, seed=7, smallest=(8, 4), largest=(24, 12))
    ens.append(grids.ramp_ensemble(1, seed=8, smallest=(16, 8), largest=(16, 8))[0])
    return [Simulation(c, g) for g, c, _, _ in ens]


def _map_ids(ids, c, sims, b):
    """Per-case cell ids (valid, ghost, or -1) to batch ids."""
    ids = np.asarray(ids)
    n = sims[c].num_cells
    return np.where(ids < 0, -1,
                    np.where(ids < n, ids + b.cell_offsets[c], b.num_cells + b.ghost_offsets[c] + ids - n))


def test_batch_layout_and_numbering():
    sims = _cases()
    b = Batch(sims)
    assert b.n_cases == len(sims)
    assert b.cell_offsets.tolist() == np.concatenate([[0], np.cumsum([s.num_cells for s in sims])]).tolist()
    assert b.face_offsets[-1] == sum(s.num_faces for s in sims) == b.num_faces
    assert b.ghost_offsets[-1] == sum(s.num_ghost_cells for s in sims) == b.num_ghost_cells
    assert b.max_faces == max(s.max_faces for s in sims)
    left, right, cf, nb = b.dump("left"), b.dump("right"), b.dump("cell_faces"), b.dump("neighbours")
    os_, gs = b.dump("outsigns"), b.dump("ghost_source")
    fg, cg = b.dump("face_geometry"), b.dump("cell_geometry")
    for c, s in enumerate(sims):
        f0, f1 = b.face_offsets[c], b.face_offsets[c + 1]
        c0, c1 = b.cell_offsets[c], b.cell_offsets[c + 1]
        g0, g1 = b.ghost_offsets[c], b.ghost_offsets[c + 1]
        assert np.array_equal(left[f0:f1], _map_ids(s.dump("left"), c, sims, b))
        assert np.array_equal(right[f0:f1], _map_ids(s.dump("right"), c, sims, b))
        scf = s.dump("cell_faces")
        assert np.array_equal(cf[c0:c1, :scf.shape[1]], np.where(scf < 0, -1, scf + f0))
        assert np.array_equal(nb[c0:c1, :scf.shape[1]], _map_ids(s.dump("neighbours"), c, sims, b))
        assert np.array_equal(os_[c0:c1, :scf.shape[1]], s.dump("outsigns"))
        assert np.array_equal(gs[g0:g1], _map_ids(s.dump("ghost_source"), c, sims, b))
        assert np.array_equal(fg[:, f0:f1], s.dump("face_geometry"))
        scg = s.dump("cell_geometry")
        assert np.array_equal(cg[:, c0:c1], scg[:, :s.num_cells])
        assert np.array_equal(cg[:, b.num_cells + g0:b.num_cells + g1], scg[:, s.num_cells:])


def test_batch_split_and_single_case_layout():
    sims = _cases()
    b = Batch(sims)
    parts = b.split(np.arange(b.num_cells))
    assert [len(p) for p in parts] == [s.num_cells for s in sims]
    one = Batch(sims[:1])
    assert one.n_cases == 1 and one.num_cells == sims[0].num_cells
    assert np.array_equal(one.dump("left"), sims[0].dump("left"))


def test_batch_refuses_inconsistent_cases():
    g1, c1, _ = case("ramp")
    g2, c2, _ = case("ramp", flux="ausmdv")
    with pytest.raises(IbisgbError, match="ERR_CONFIG"):
        Batch([Simulation(c1, g1), Simulation(c2, g2)])
    g3, c3, _ = case("ramp", solver=grids.steady_state())
    with pytest.raises(IbisgbError, match="ERR_CONFIG"):
        Batch([Simulation(c1, g1), Simulation(c3, g3)])
    g4, c4, _ = case("box")
    with pytest.raises(IbisgbError, match="ERR_CONFIG"):
        Batch([Simulation(c1, g1), Simulation(c4, g4)])
    b = Batch([Simulation(c1, g1), Simulation(c1, g1)])
    with pytest.raises(IbisgbError, match="ERR_ARG"):
        Batch([b, Simulation(c1, g1)])
    with pytest.raises(IbisgbError, match="ERR_STATE"):
        b.steady_initialise()
