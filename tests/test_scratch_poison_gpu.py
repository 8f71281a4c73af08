"""No residual or derivative call reads scratch it did not write: with every
scratch buffer of the residual, tangent and adjoint kernels filled with NaN before
each call (ibisgb_set_scratch_poison), the residual in every precision and the
state, geometry and flow-state tangents and adjoints are finite and the same bits
as without -- 2-D and 3-D, first and second order, viscous, constant-flux,
boundary-layer, periodic and renumbered grids."""
import copy

import numpy as np
import pytest

from ibis_gb300 import Simulation
from tests.cases import case
from tests.test_flow_state_cpu import flow_states

pytestmark = pytest.mark.gpu

CASES = [("ramp", {}), ("ramp", {"order": 1}), ("tiny2d", {}), ("tri", {}), ("subsonic", {}), ("bl_plate", {}),
         ("plate", {}), ("cflux_ramp", {}), ("cflux_box", {}), ("box", {}), ("tet", {"renumber": "rcm"}),
         ("wedge", {})]
IDS = ["-".join([n] + [f"{k}={v}" for k, v in kw.items()]) for n, kw in CASES]


def products(sim, c):
    rng = np.random.default_rng(31)
    U = sim.conserved()
    scale = np.abs(U).mean(axis=0)
    v = rng.standard_normal(U.shape) * scale
    w = rng.standard_normal(U.shape) / scale
    fg, cg = sim.dump("face_geometry"), sim.dump("cell_geometry")
    df = rng.standard_normal(fg.shape) * (np.abs(fg).mean(axis=1, keepdims=True) + 1e-3)
    dc = rng.standard_normal(cg.shape) * (np.abs(cg).mean(axis=1, keepdims=True) + 1e-3)
    dc[3, sim.num_cells:] = 0.0
    dfs = {t: rng.standard_normal(7) * 10.0 for t in sim.boundary_tags() if flow_states(c, t)}
    jtw, gadj = sim.vector_jacobian_product(w, ghosts=True)
    out = [sim.compute_dudt(p) for p in ("f64_exact", "f64", "mixed", "mixed_grad", "mixed_ff")]
    out += [sim.matrix_vector_product(v), jtw, gadj, *sim.geometry_adjoint(w), sim.geometry_tangent(df, dc)]
    if dfs:
        out += list(sim.flow_state_adjoint(w).values()) + [sim.flow_state_tangent(dfs)]
    return out


@pytest.mark.parametrize("name,kw", CASES, ids=IDS)
def test_derivatives_read_no_stale_scratch(name, kw):
    kw = dict(kw)
    renumber = kw.pop("renumber", None)
    g, c, st = case(name, **kw)
    if renumber:
        c = copy.deepcopy(c)
        c["grid"]["renumber"] = renumber
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    clean = products(sim, c)
    sim.set_scratch_poison(True)
    for _ in range(2):
        poisoned = products(sim, c)
        for k, (a, b) in enumerate(zip(clean, poisoned)):
            assert np.isfinite(b).all(), k
            assert np.array_equal(a, b), k
