"""The oracle (CPU restatement of the reference) against the golden vectors of
the reference's own unit tests, and against the free-stream property of its
integration tests."""
import numpy as np
import pytest

from ibis_gb300 import grids
from oracle.oracle import Oracle, dense_gmres


def config_3x3():
    bnds = {t: grids.slip_wall() for t in ["slip_wall_bottom", "slip_wall_top", "inflow", "outflow"]}
    return grids.make_config(2, bnds)


@pytest.fixture(scope="module")
def square():
    return Oracle(config_3x3(), grids.unit_square_3x3())


def test_interfaces_and_cell_faces(square, golden):
    # interface numbering by first appearance (grid.cpp:136-143, 199-215)
    conn = square.connectivity()
    assert conn["cell_faces"].tolist() == golden["grid_cell_faces"]["face_ids"]
    assert conn["outsigns"].tolist() == golden["grid_outsigns"]["outsigns"]
    for c, slot, nb in golden["cell_neighbours"]["checks"]:
        assert conn["neighbours"][c, slot] == nb


def test_face_geometry(square, golden):
    geo = square.geometry()
    n = np.array(golden["interface_normals"]["normals"])
    assert np.abs(geo["normal"][:, : len(n)].T - n).max() < 1e-14
    assert np.abs(geo["centre"][0] - golden["interface_centres"]["x"]).max() < 1e-14
    assert np.abs(geo["centre"][1] - golden["interface_centres"]["y"]).max() < 1e-14
    assert np.abs(geo["area"] - 1.0).max() < 1e-14
    assert np.abs(geo["volume"][: square.N] - 1.0).max() < 1e-14
    assert np.abs(geo["centroid"][0, :9] - golden["cell_centroids_2d"]["x"]).max() < 1e-14
    assert np.abs(geo["centroid"][1, :9] - golden["cell_centroids_2d"]["y"]).max() < 1e-14


def test_ghost_cell_centres(square, golden):
    geo = square.geometry()
    for tag, expected in golden["ghost_cell_centres"].items():
        if tag.startswith("_"):
            continue
        ids, _ = square.ghosts(tag)
        got = geo["centroid"][:, ids].T
        assert np.array_equal(got, np.array(expected)), tag


def test_gradient_of_linear_field(square, golden):
    gv = golden["gradient_linear_field"]
    values = np.zeros(square.N + square.G)
    values[: square.N] = gv["valid"]
    for tag in ["slip_wall_bottom", "slip_wall_top", "inflow", "outflow"]:
        ids, _ = square.ghosts(tag)
        values[ids] = gv[tag]
    g = square.gradient(values)
    assert np.allclose(g[:, 0], gv["expected"][0], rtol=1e-12)
    assert np.allclose(g[:, 1], gv["expected"][1], rtol=1e-12)


def test_cube_volumes_and_orientation(golden):
    bnds = {t: grids.slip_wall() for t in ["bottom", "top", "west", "east", "north", "south"]}
    o = Oracle(grids.make_config(3, bnds), grids.unit_cube_3x3x3())
    geo = o.geometry()
    assert o.N == golden["cube_volumes"]["n_cells"]
    assert np.allclose(geo["volume"][: o.N], golden["cube_volumes"]["volume"], rtol=1e-12)
    for k in ("normal", "tan1", "tan2"):
        assert np.allclose(np.linalg.norm(geo[k], axis=0), 1.0, rtol=1e-12)


def test_gmres_and_fgmres(golden):
    g = golden["gmres"]
    x, info = dense_gmres(np.array(g["A"]), np.array(g["rhs"]), 5, 1e-14)
    assert info["success"] and np.allclose(x, g["x"], rtol=1e-9, atol=1e-12)
    f = golden["fgmres"]
    x, info = dense_gmres(np.array(f["A"]), np.array(f["rhs"]), 5, 1e-14, P=np.array(f["P"]),
                          max_prec_iters=2, prec_tol=1e-1)
    assert info["success"] and np.allclose(x, f["x"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("flux", ["hanel", "ausmdv", "ldfss2", "rusanov"])
@pytest.mark.parametrize("dim", [2, 3])
def test_uniform_stream_is_steady(flux, dim):
    """tests/minimal/uniform_stream{,_3D}: supersonic stream, residual identically 0."""
    gas = grids.ideal_gas()
    inflow = grids.flow_state(gas, 300.0, 1e5, 800.0, 100.0, 50.0 if dim == 3 else 0.0)
    if dim == 2:
        g = grids.structured_2d(*np.meshgrid(np.linspace(0, 1, 9), np.linspace(0, 1, 7), indexing="ij"))
        tags = ["west", "east", "south", "north"]
    else:
        g = grids.box_3d(4)
        tags = ["west", "east", "south", "north", "bottom", "top"]
    bnds = {t: (grids.supersonic_inflow(inflow) if t in ("west", "south", "bottom")
                else grids.supersonic_outflow()) for t in tags}
    o = Oracle(grids.make_config(dim, bnds, flux=flux), g)
    n = o.N
    o.set_initial_condition(np.full(n, 300.0), np.full(n, 1e5), np.full(n, 800.0),
                            np.full(n, 100.0), np.full(n, 50.0) if dim == 3 else None)
    r = o.residual()
    assert np.abs(r).max() < 1e-9 * 1e5 * 800.0


@pytest.mark.parametrize("block", ["cubic_spline", "cubic_spline_2"])
def test_cubic_spline(golden, block):
    """The boundary-layer profile's spline against the reference's spline tests."""
    from oracle.oracle import cubic_spline
    g = golden[block]
    q, expected = np.array(g["evals"]).T
    got = cubic_spline(g["x"], g["y"], q)
    assert np.allclose(got, expected, rtol=1.19e-5, atol=1.19e-5 * 1e-3)


def test_cubic_spline_is_a_natural_spline():
    """Interpolates, has continuous first derivatives at the knots and zero
    curvature at both ends; rejects fewer than 4 points."""
    from oracle.oracle import cubic_spline
    rng = np.random.default_rng(3)
    x = np.cumsum(rng.uniform(0.1, 1.0, 9))
    y = rng.normal(size=9)
    assert np.allclose(cubic_spline(x, y, x[1:-1]), y[1:-1], rtol=0, atol=1e-12)
    h = 1e-6
    for k in range(1, 8):
        left = (cubic_spline(x, y, [x[k]])[0] - cubic_spline(x, y, [x[k] - h])[0]) / h
        right = (cubic_spline(x, y, [x[k] + h])[0] - cubic_spline(x, y, [x[k]])[0]) / h
        assert abs(left - right) < 1e-4 * (1 + abs(left))
    def curvature(c, d):
        f = cubic_spline(x, y, [c - d, c, c + d])
        return (f[0] - 2 * f[1] + f[2]) / d ** 2
    for end, s in ((x[0], 1), (x[-1], -1)):
        # the curvature is linear on the end interval: extrapolate it to the end knot
        d1, d2 = curvature(end + s * 2e-4, 1e-4), curvature(end + s * 4e-4, 1e-4)
        scale = abs(curvature(end + s * 0.05, 1e-3)) + 1.0
        assert abs(2 * d1 - d2) < 1e-3 * scale, (d1, d2)
    with pytest.raises(ValueError):
        cubic_spline([0, 1, 2], [0, 1, 2], [0.5])


def test_flop_counts_fixture_matches_the_counting_oracle():
    """tests/golden/flop_counts.json (the reference algorithm's exact operation
    counts per ssp-rk3 step on the periodic box, used by bench.py for the FP64
    path's roofline) is what the oracle on its counting scalar gives, and the
    per cell-update count follows A + B/n."""
    import json
    import os

    from ibis_gb300 import grids
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(root, "tests", "golden", "flop_counts.json")) as f:
        fx = json.load(f)
    A, B = fx["flops_per_cell_update"]["A"], fx["flops_per_cell_update"]["B"]
    for n in (8, 12):
        g, c = grids.box_case(n)
        o = Oracle(c, g)
        o.set_initial_condition(*grids.box_initial_condition(n, c["gas_model"], seed=0))
        got = o.count_step_flops()
        assert got == fx["counts_per_step"][str(n)]
        arith = sum(got[k] for k in ("add", "mul", "div", "sqrt", "pow"))
        assert arith / (3 * n ** 3) == pytest.approx(A + B / n, rel=1e-12)
