"""Parity of the sm_103a residual / Runge-Kutta kernels with the oracle.

Tolerances (per cell, relative to the gross flux through the cell, see
tests/cases.py:gross_flux_scale):
  * f64_exact (reference operation order, no FMA): bitwise, except where the
    reference calls pow() (Sutherland's law in viscous cases, LDFSS2's
    pow(x, 2.0)): CUDA's and glibc's pow may differ in the last bit, <= 1e-14.
  * f64 (FMA contraction allowed): <= 1e-12.
  * mixed (float reconstruction/flux, double accumulation): <= 2e-5.
  * mixed_grad (float gradients/limiters on relative values, double face
    states and fluxes): <= 1e-6 (measured 7e-9 to 3e-7).
  * mixed_ff (float-float gradients, limiters, face states, fluxes, viscous
    terms and ghost normals; double update): <= 1e-11 (measured 4e-15 to 1.4e-12).
Limiter branch selection must be identical in f64_exact; in f64 it may differ
in at most 1% of the cells, where FMA rounding flips a projection that is zero
to rounding or an exact tie between two faces.
"""
import numpy as np
import pytest

from ibis_gb300 import Simulation, grids
from ibis_gb300._lib import IbisgbError
from oracle.oracle import Oracle
from tests.cases import case, gross_flux_scale, per_cell_rel_err

pytestmark = pytest.mark.gpu

CASES = [
    ("ramp", {}),
    ("ramp", {"flux": "ausmdv"}),
    ("ramp", {"flux": "ldfss2"}),
    ("ramp", {"flux": "rusanov"}),
    ("ramp", {"thermo": "rho_p"}),
    ("ramp", {"thermo": "rho_T"}),
    ("ramp", {"thermo": "p_T"}),
    ("ramp", {"limiter": "unlimited"}),
    ("ramp", {"order": 1}),
    ("plate", {}),
    ("box", {}),
    ("box", {"flux": "ausmdv"}),
    ("box_inout", {}),
    ("subsonic", {}),
    ("tri", {}),
    ("tet", {}),
    ("wedge", {}),
    ("pyramid", {}),
    ("pyramid", {"flux": "ausmdv", "thermo": "rho_p"}),
    ("tiny2d", {}),
    ("tiny3d", {}),
    ("bl_plate", {}),
    ("cflux_ramp", {}),
    ("cflux_ramp", {"flux": "ldfss2"}),
    ("cflux_box", {}),
]


def ids(c):
    return c[0] + "-" + "-".join(f"{k}={v}" for k, v in c[1].items())


def pair(name, kw):
    g, c, st = case(name, **kw)
    sim, ref = Simulation(c, g), Oracle(c, g)
    sim.set_primitives(*st)
    ref.set_initial_condition(*st)
    return sim, ref


@pytest.mark.parametrize("name,kw", CASES, ids=[ids(c) for c in CASES])
def test_residual_parity(name, kw):
    sim, ref = pair(name, kw)
    r_ref, br_ref = ref.residual(branches=True)
    scale = gross_flux_scale(ref)
    uses_pow = sim.config["viscous_flux"]["enabled"] or \
        sim.config["convective_flux"]["flux_calculator"]["type"] == "ldfss2"
    limited = sim.config["convective_flux"]["reconstruction_order"] == 2 and \
        sim.config["convective_flux"]["limiter"]["type"] == "barth_jespersen"

    r = sim.compute_dudt("f64_exact")
    if uses_pow:
        assert per_cell_rel_err(r, r_ref, scale).max() <= 1e-14
    else:
        assert np.array_equal(r, r_ref), np.abs(r - r_ref).max()
    if limited:
        assert np.array_equal(sim.dump("limiter_branches"), br_ref)

    r = sim.compute_dudt("f64")
    assert per_cell_rel_err(r, r_ref, scale).max() <= 1e-12
    if limited:
        # FMA contraction can flip a face projection that is zero to rounding, or an
        # exact tie between two faces' ratios (wedge cells have both), so the recorded
        # branch may differ in a few cells; the limiter value, and the residual above,
        # agree to rounding
        differ = np.any(sim.dump("limiter_branches") != br_ref, axis=1)
        assert differ.sum() <= max(1, sim.num_cells // 100), differ.sum()

    r = sim.compute_dudt("mixed")
    assert per_cell_rel_err(r, r_ref, scale).max() <= 2e-5

    r = sim.compute_dudt("mixed_grad")
    assert per_cell_rel_err(r, r_ref, scale).max() <= 1e-6

    r = sim.compute_dudt("mixed_ff")
    assert per_cell_rel_err(r, r_ref, scale).max() <= 1e-11


@pytest.mark.parametrize("name", ["ramp", "plate", "box"])
def test_estimate_dt(name):
    sim, ref = pair(name, {})
    ref.residual()
    sim.compute_dudt("f64")  # viscous dt uses the face states of the last residual
    assert sim.estimate_dt() == pytest.approx(ref.estimate_dt(), rel=1e-13)


@pytest.mark.parametrize("name", ["ramp", "box", "plate", "tri", "tet", "wedge", "pyramid", "tiny2d", "bl_plate",
                                  "cflux_ramp", "cflux_box"])
def test_rk_trajectory(name):
    steps = 6
    sim, ref = pair(name, {})
    ref.rk_initialise()
    o = ref.rk_steps(steps)
    U_ref = ref.conserved()
    st = sim.take_steps(steps, "f64_exact")
    assert st["steps"] == steps
    assert st["dt"] == pytest.approx(o["dt"], rel=1e-14)
    U = sim.conserved()
    scale = np.abs(U_ref).max(axis=0)
    if sim.config["viscous_flux"]["enabled"]:
        assert (np.abs(U - U_ref) / scale).max() <= 1e-13
    else:
        assert np.array_equal(U, U_ref), (np.abs(U - U_ref) / scale).max()
    norms = sim.L2_norms()
    assert np.allclose(norms, o["norms"], rtol=1e-11, atol=1e-300)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-6)])
def test_rk_trajectory_fast_paths(precision, tol):
    """L2 density error of the fast paths against the FP64 oracle after 20 steps
    of the compression ramp from its uniform Mach 2 inflow state."""
    g, c, inf = grids.ramp_case(48, 24)
    sim, ref = Simulation(c, g), Oracle(c, g)
    n = sim.num_cells
    st = (np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    sim.set_primitives(*st)
    ref.set_initial_condition(*st)
    ref.rk_initialise()
    ref.rk_steps(20)
    rho_ref = ref.conserved()[:, 0]
    sim.take_steps(20, precision)
    rho = sim.conserved()[:, 0]
    assert np.linalg.norm(rho - rho_ref) / np.linalg.norm(rho_ref) <= tol


def test_uniform_stream_stays_uniform():
    """tests/minimal/uniform_stream: a uniform supersonic stream is steady."""
    gas = grids.ideal_gas()
    inflow = grids.flow_state(gas, 300.0, 1e5, 800.0, 100.0, 50.0)
    g = grids.box_3d(6)
    b = {t: (grids.supersonic_inflow(inflow) if t in ("west", "south", "bottom") else grids.supersonic_outflow())
         for t in ["west", "east", "south", "north", "bottom", "top"]}
    sim = Simulation(grids.make_config(3, b, gas=gas), g)
    n = sim.num_cells
    sim.set_primitives(np.full(n, 300.0), np.full(n, 1e5), np.full(n, 800.0), np.full(n, 100.0), np.full(n, 50.0))
    for prec in ("f64_exact", "f64", "mixed"):
        assert np.abs(sim.compute_dudt(prec)).max() < 1e-6
    U0 = sim.conserved()
    sim.take_steps(10, "mixed")
    assert np.abs(sim.conserved() - U0).max() <= 1e-9 * np.abs(U0).max()


def test_bad_cells_stop_the_run():
    """count_bad_cells -> Solver::solve returns 1 (solver.cpp:38-43): a NaN placed
    in the host initial state stops the time march with IBISGB_ERR_BAD_CELLS."""
    g, c, st = case("ramp")
    sim = Simulation(c, g)
    T, p, vx, vy, _ = st
    p = p.copy()
    p[7] = np.nan
    sim.set_primitives(T, p, vx, vy)
    with pytest.raises(IbisgbError) as e:
        sim.take_steps(5, "f64")
    assert e.value.code == -4
    assert sim.count_bad_cells() > 0


def test_residual_into_torch_tensor():
    torch = pytest.importorskip("torch")
    sim, ref = pair("box", {})
    out = torch.empty((sim.num_cells, sim.n_conserved), dtype=torch.float64, device="cuda")
    sim.compute_dudt_into(out, "f64_exact", stream=torch.cuda.current_stream())
    assert np.array_equal(out.cpu().numpy(), ref.residual())


@pytest.mark.parametrize("name", ["ramp", "box"])
@pytest.mark.parametrize("precision", ["mixed", "f64"])
def test_launch_variants_are_bit_identical(name, precision):
    """Every launch variant of the autotuner computes the same bits."""
    g, c, st = case(name)
    nv = len(Simulation.launch_variants())
    ref = None
    for w in range(nv):
        sim = Simulation(c, g)
        sim.set_primitives(*st)
        sim.set_launch_variants(precision, w, w, w)
        sim.take_steps(4, precision)
        U = sim.conserved()
        if ref is None:
            ref = U
        assert np.array_equal(U, ref), w
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    sim.set_fused(0)  # the fused stage agrees to rounding only; it has its own tests
    tuned = sim.autotune(precision)
    assert all(0 <= x < nv for x in tuned["variants"].values())
    assert all(len(v) == nv and min(v) > 0 for v in tuned["ms"].values())
    sim.take_steps(4, precision)
    assert np.array_equal(sim.conserved(), ref)


def test_integer_pipe_conversions_match_the_instructions():
    """The mixed update's float -> double conversion (integer bit operations)
    equals the conversion instruction bit for bit."""
    import ctypes as C
    from ibis_gb300 import _lib
    n = C.c_int64()
    assert _lib.load().ibisgb_check_conversions(1 << 24, 12345, C.byref(n)) == 0
    assert n.value == 0


def test_conserved_state_round_trip_pinned_and_pageable():
    """Pinned host buffers are read and written in place by the layout kernels,
    other host memory goes through a staging copy: both give the same bits, and a
    pinned buffer may be overwritten as soon as ibisgb_set_conserved returns."""
    torch = pytest.importorskip("torch")
    g, c, st = case("box")
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    U = sim.conserved()
    pin = torch.empty(U.shape, dtype=torch.float64, pin_memory=True).numpy()
    sim.conserved(out=pin)
    assert np.array_equal(pin, U)
    rng = np.random.default_rng(5)
    U2 = U * (1.0 + 1e-3 * rng.standard_normal(U.shape))
    pin[:] = U2
    sim.set_conserved(pin)
    pin[:] = 0.0
    assert np.array_equal(sim.conserved(), U2)
    sim.set_fused(0)  # the three-kernel stage in both (every launch variant gives the same bits)
    sim.set_cell_flux(0)
    a = sim.take_steps(2, "mixed")
    Ua = sim.conserved()
    other = Simulation(c, g)
    other.set_primitives(*st)
    other.set_conserved(U2.copy())
    other.set_fused(0)
    other.set_cell_flux(0)
    b = other.take_steps(2, "mixed")
    assert np.array_equal(other.conserved(), Ua) and a["t"] == b["t"]
