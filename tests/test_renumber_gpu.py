"""Internal reverse Cuthill-McKee cell / face numbering ("renumber": "rcm").

Every array and id that crosses the ABI stays in the reference's numbering, and
each cell keeps its face slots and summation order, so a renumbered context must
give the same bits as one in the grid's own order: residual (every precision),
Runge-Kutta steps, tangent and adjoint products, the adjoint step, primitives,
conserved state and every dump.  "auto" renumbers a shuffled tetrahedral grid
and leaves quadrilateral / hexahedral grids alone; batches of renumbered cases
match the cases run alone."""
import copy

import numpy as np
import pytest

from ibis_gb300 import Batch, Simulation, grids
from tests.cases import case, random_state

pytestmark = pytest.mark.gpu

CASES = [("ramp", {}), ("ramp", {"order": 1}), ("tri", {}), ("tet", {}), ("wedge", {}), ("pyramid", {}),
         ("box", {}), ("box_inout", {}), ("plate", {}), ("subsonic", {}), ("bl_plate", {}), ("cflux_ramp", {})]
IDS = ["-".join([n] + [f"{k}={v}" for k, v in kw.items()]) for n, kw in CASES]
DUMPS = ["left", "right", "cell_faces", "outsigns", "neighbours", "ghost_source", "face_geometry",
         "cell_geometry", "ghost_face", "ghost_boundary"]


def pair(name, kw):
    g, c, st = case(name, **kw)
    out = []
    for mode in ("none", "rcm"):
        cc = copy.deepcopy(c)
        cc["grid"]["renumber"] = mode
        sim = Simulation(cc, g)
        sim.set_primitives(*st)
        out.append(sim)
    assert not out[0].numbering()["renumbered"] and out[1].numbering()["renumbered"]
    return out


@pytest.mark.parametrize("name,kw", CASES, ids=IDS)
def test_renumbered_context_gives_the_same_bits(name, kw):
    a, b = pair(name, kw)
    order = b.dump("cell_order")
    assert sorted(order.tolist()) == list(range(a.num_cells)) and not np.array_equal(order, np.arange(a.num_cells))
    for d in DUMPS:
        assert np.array_equal(a.dump(d), b.dump(d)), d
    for prec in ("f64_exact", "f64", "mixed", "mixed_ff"):
        assert np.array_equal(a.compute_dudt(prec), b.compute_dudt(prec)), prec
    a.compute_dudt("f64_exact")
    b.compute_dudt("f64_exact")
    second_order = a.config["convective_flux"]["reconstruction_order"] == 2
    for d in ("limiter_branches", "limiters", "face_flux") if second_order else ("face_flux",):
        assert np.array_equal(a.dump(d), b.dump(d)), d
    for k in a.primitives():
        assert np.array_equal(a.primitives()[k], b.primitives()[k]), k
    U = a.conserved()
    rng = np.random.default_rng(4)
    scale = np.abs(U).mean(axis=0)
    v = rng.standard_normal(U.shape) * scale
    w = rng.standard_normal(U.shape) / scale
    assert np.array_equal(a.matrix_vector_product(v, 1e3), b.matrix_vector_product(v, 1e3))
    ja, ga = a.vector_jacobian_product(w, ghosts=True)
    jb, gb = b.vector_jacobian_product(w, ghosts=True)
    assert np.allclose(ja, jb, rtol=1e-13, atol=1e-13 * np.abs(ja).max())
    assert np.allclose(ga, gb, rtol=1e-13, atol=1e-13 * max(np.abs(ga).max(), 1e-300))
    # state round trip and a few Runge-Kutta steps
    U2 = U * (1 + 1e-3 * rng.standard_normal(U.shape))
    a.set_conserved(U2)
    b.set_conserved(U2)
    assert np.array_equal(b.conserved(), U2)
    sa, sb = a.take_steps(5, "f64_exact"), b.take_steps(5, "f64_exact")
    assert sa["t"] == sb["t"]
    assert np.array_equal(a.conserved(), b.conserved())


def test_adjoint_step_is_independent_of_the_numbering():
    import torch
    out = []
    for sim in pair("tet", {}):
        U = sim.conserved()
        g = torch.tensor(np.random.default_rng(1).standard_normal(U.shape) / np.abs(U).mean(axis=0),
                         dtype=torch.float64, device="cuda")
        lam = torch.zeros_like(g)
        for _ in range(3):
            st = sim.adjoint_step(g, lam, 5.0)
        out.append((lam.cpu().numpy(), st["scaled_residual_norm"]))
    assert np.allclose(out[0][0], out[1][0], rtol=1e-10, atol=1e-10 * np.abs(out[0][0]).max())
    assert out[0][1] == pytest.approx(out[1][1], rel=1e-10)


def test_auto_renumbers_a_shuffled_tetrahedral_grid_only():
    g, c, inf = grids.tet_channel_case(6, shuffle_seed=0)
    st = random_state(g.num_cells, inf["T"], inf["p"], inf["vx"], 3, seed=4)
    sim = Simulation(c, g)  # no renumber key: auto
    info = sim.numbering()
    assert info["renumbered"] and 2 * info["bandwidth_internal"] <= info["bandwidth_reference"], info
    cc = copy.deepcopy(c)
    cc["grid"]["renumber"] = "none"
    ref = Simulation(cc, g)
    for s in (sim, ref):
        s.set_primitives(*st)
    assert np.array_equal(sim.compute_dudt("f64_exact"), ref.compute_dudt("f64_exact"))
    gq, cq, _ = case("ramp")
    assert not Simulation(cq, gq).numbering()["renumbered"]


def test_batch_of_renumbered_cases_matches_the_cases_alone():
    sims, parts, sts = [], [], []
    for name in ("tri", "ramp"):
        g, c, st = case(name)
        c = copy.deepcopy(c)
        c["grid"]["renumber"] = "rcm"
        s = Simulation(c, g)
        s.set_primitives(*st)
        sims.append(s)
        parts.append(Simulation(c, g))
        sts.append(st)
    b = Batch(parts)
    assert b.numbering()["renumbered"]
    b.set_primitives(*[np.concatenate([st[q] for st in sts]) for q in range(4)])
    for s, r in zip(sims, b.split(b.compute_dudt("f64_exact"))):
        assert np.array_equal(s.compute_dudt("f64_exact"), r)
    for s, r in zip(sims, b.split(b.dump("cell_geometry")[:, :b.num_cells].T)):
        assert np.array_equal(s.dump("cell_geometry")[:, :s.num_cells].T, r)


def test_driver_writes_the_same_flow_files_when_renumbered(tmp_path):
    import subprocess
    from ibis_gb300 import build
    outs = []
    for mode in ("auto", "none"):
        g, c, st = case("tet")
        c = copy.deepcopy(c)
        c["grid"]["renumber"] = mode
        c["solver"] = grids.runge_kutta(max_step=5, plot_every_n_steps=5)
        d = tmp_path / mode
        grids.write_case(str(d), g, c, *st)
        r = subprocess.run([build.DRIVER, "--case", str(d), "--precision", "f64_exact"], capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        outs.append({n: (d / "io" / "flow" / "0001" / n).read_bytes() for n in ("T", "p", "vx", "vy", "vz")})
    g, c, _ = case("tet")
    assert Simulation(c, g).numbering()["renumbered"]  # "auto" renumbers this grid
    assert outs[0] == outs[1]
