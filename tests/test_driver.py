"""ibisgb-run, the host driver over the C ABI: reads an ibis case directory
(config/config.json, the SU2 grid, the native initial flow) and writes the
reference's outputs (io/flow/NNNN, io/flow/flows, log/*.dat).  Input errors
are checked on the host; the GPU tests compare its outputs with the engine
driven from Python, bit for bit in the FP64_EXACT build."""
import os
import subprocess

import numpy as np
import pytest

from ibis_gb300 import Simulation, build, grids
from tests.cases import case

DRIVER = build.DRIVER


def _case(tmp_path, fmt="native_binary", solver=None):
    g, c, st = case("ramp")
    c["io"]["flow_format"] = fmt
    if solver is not None:
        c["solver"] = solver
    grids.write_case(str(tmp_path), g, c, *st[:4])
    return g, c, st


def _run(tmp_path, *args):
    return subprocess.run([DRIVER, "--case", str(tmp_path), *args], capture_output=True, text=True, timeout=600)


def test_driver_reports_input_errors(tmp_path):
    assert os.path.exists(DRIVER)
    r = subprocess.run([DRIVER, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    _case(tmp_path)
    os.remove(tmp_path / "io" / "flow" / "0000" / "vy")
    r = _run(tmp_path)
    assert r.returncode == 2 and "Unable to load" in r.stderr and "vy" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["native_binary", "native_text"])
def test_driver_runge_kutta_matches_the_engine(tmp_path, fmt):
    solver = grids.runge_kutta(max_step=10, plot_every_n_steps=5, residuals_every_n_steps=1)
    g, c, st = _case(tmp_path, fmt, solver)
    r = _run(tmp_path, "--precision", "f64_exact")
    assert r.returncode == 0, r.stderr
    flows = (tmp_path / "io" / "flow" / "flows").read_text().split()
    assert flows == ["0001", "0002"]
    sim = Simulation(c, g)
    sim.set_primitives(*st[:4])
    sim.take_steps(10, "f64_exact")
    pr = sim.primitives()
    out = tmp_path / "io" / "flow" / "0002"
    for name in ("T", "p", "vx", "vy"):
        if fmt == "native_binary":
            v = np.fromfile(out / name)
            assert np.array_equal(v, pr[name]), name
        else:
            v = np.loadtxt(out / name)
            assert np.allclose(v, pr[name], rtol=1e-14, atol=1e-12), name
    lines = (tmp_path / "log" / "residuals.dat").read_text().splitlines()
    assert lines[0].split() == ["time", "step", "wall_clock", "global", "mass", "momentum_x", "momentum_y",
                                "momentum_z", "energy"]
    assert len(lines) == 1 + 1 + 10  # header, initial state, every step
    last = np.array(lines[-1].split(), float)
    norms = sim.L2_norms()
    assert np.allclose(last[3:], norms, rtol=1e-5)  # written with 6 significant digits, as the reference does
    import json
    assert json.loads((out / "meta_data.json").read_text())["time"] == pytest.approx(last[0], rel=1e-5)


@pytest.mark.gpu
def test_driver_steady_state(tmp_path):
    cfl = {"type": "residual_based", "growth_threshold": 1.0, "power": 1.0, "start_cfl": 2.0, "max_cfl": 1e12}
    solver = grids.steady_state(cfl=cfl, max_steps=6, max_iters=20, tol=1e-2)
    _case(tmp_path, "native_binary", solver)
    r = _run(tmp_path)
    assert r.returncode == 0, r.stderr
    for name in ("absolute_residuals.dat", "relative_residuals.dat", "gmres_diagnostics.dat"):
        assert (tmp_path / "log" / name).exists(), name
    rel = (tmp_path / "log" / "relative_residuals.dat").read_text().splitlines()
    assert float(rel[1].split()[3]) == 1.0  # step 0: relative residual 1
    ab = (tmp_path / "log" / "absolute_residuals.dat").read_text().splitlines()
    assert float(ab[1].split()[3]) > 0.0
    assert (tmp_path / "io" / "flow" / "flows").read_text().split()[-1] == "0001"
