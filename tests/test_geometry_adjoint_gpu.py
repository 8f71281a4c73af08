"""The geometry adjoint (ibisgb_vjp_geometry) and tangent (ibisgb_jvp_geometry):
w^T dR/dgeometry and dR/dgeometry . d against the
oracle's dual-number directional derivative of the residual along a random
perturbation of the geometry (the reference's Dual seeded in the Grid<Dual>
face frame, centres, areas, centroids -- ghosts included -- and volumes, the
least-squares factors recomputed from the dual centroids): the dot-product test
<w, dR/dgeom . d> = <J_geom^T w, d> to 1e-12, on second-order (Barth-Jespersen
and unlimited) and first-order residuals, inviscid and viscous (the flat
plate's no-slip wall, subsonic in/outflow with a fixed-temperature wall), 2-D
and 3-D, every element type, slip walls, supersonic in/out, constant-flux and
periodic boundaries; and the same result with the grid renumbered internally."""
import copy

import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from oracle.oracle import Oracle
from tests.cases import case

pytestmark = pytest.mark.gpu

CASES = [("ramp", {}), ("ramp", {"limiter": "unlimited"}), ("ramp", {"order": 1}), ("ramp", {"flux": "ausmdv"}),
         ("ramp", {"flux": "rusanov"}), ("ramp", {"thermo": "rho_p"}), ("tri", {}), ("tiny2d", {}),
         ("box", {}), ("box_inout", {}), ("tet", {}), ("wedge", {}), ("pyramid", {}),
         ("plate", {}), ("plate", {"order": 1}), ("subsonic", {}), ("bl_plate", {}), ("cflux_ramp", {}),
         ("cflux_box", {})]
IDS = ["-".join([n] + [f"{k}={v}" for k, v in kw.items()]) for n, kw in CASES]
UNREAD_2D = [2, 5, 6, 7, 11]  # n_z, t1_z, t2_x, t2_y, centre z: not inputs of a 2-D residual


def perturbation(sim, rng):
    fg, cg = sim.dump("face_geometry"), sim.dump("cell_geometry")
    df = rng.standard_normal(fg.shape) * (np.abs(fg).mean(axis=1, keepdims=True) + 1e-3)
    dc = rng.standard_normal(cg.shape) * (np.abs(cg).mean(axis=1, keepdims=True) + 1e-3)
    if sim.dim == 2:
        df[UNREAD_2D] = 0.0
        dc[2] = 0.0
    dc[3, sim.num_cells:] = 0.0  # ghost volumes are not inputs
    return df, dc


@pytest.mark.parametrize("name,kw", CASES, ids=IDS)
def test_geometry_adjoint_is_the_transpose_of_the_dual_geometry_derivative(name, kw):
    g, c, st = case(name, **kw)
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    cs = copy.deepcopy(c)
    cs["solver"] = grids.steady_state()
    o = Oracle(cs, g, kind="dual")
    o.set_initial_condition(*st)
    o.steady_initialise()
    U = sim.conserved()
    rng = np.random.default_rng(11)
    w = rng.standard_normal(U.shape) / np.abs(U).mean(axis=0)
    df, dc = perturbation(sim, rng)
    jd = o.geometry_jvp(df, dc)
    fb, cb = sim.geometry_adjoint(w)
    lhs = float(np.sum(w * jd))
    rhs = float(np.sum(fb * df) + np.sum(cb * dc))
    mag = float(np.sum(np.abs(w * jd)))
    assert abs(lhs - rhs) <= 1e-12 * mag, (lhs, rhs, mag)
    # the device's own geometry tangent: equal to the oracle's dual derivative, and
    # the geometry adjoint its transpose
    jg = sim.geometry_tangent(df, dc)
    assert np.abs(jg - jd).max() <= 1e-12 * np.abs(jd).max()
    lhs_g = float(np.sum(w * jg))
    assert abs(lhs_g - rhs) <= 1e-12 * mag, (lhs_g, rhs, mag)


def test_geometry_tangent_and_adjoint_are_independent_of_the_numbering():
    g, c, st = case("tet")
    out = []
    for mode in ("none", "rcm"):
        cc = copy.deepcopy(c)
        cc["grid"]["renumber"] = mode
        sim = Simulation(cc, g)
        sim.set_primitives(*st)
        U = sim.conserved()
        w = np.random.default_rng(2).standard_normal(U.shape) / np.abs(U).mean(axis=0)
        df, dc = perturbation(sim, np.random.default_rng(5))
        out.append(sim.geometry_adjoint(w) + (sim.geometry_tangent(df, dc),))
    for a, b in zip(out[0], out[1]):
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(a).max())
