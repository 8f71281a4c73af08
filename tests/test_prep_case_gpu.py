"""ibisgb-run as a drop-in for `ibis run` on a case directory written by the
reference's own, unchanged prep step (tests/golden/prep_ramp64x32, made by
tests/golden/make_prep_case.py: the CPU-runnable benchmark case on the 64 x 32
ramp, 500 ssp-rk3 steps).

The reference's own driver, run on that directory, wrote io/flow/0001; the
SHA-256 of its T, p, vx and vy files is in prep_ramp64x32_reference.json.
ibisgb-run in the FP64_EXACT build, told to reproduce the reference's aliased
stage derivatives ("stage_derivatives": "aliased" added to the solver block;
see the oracle's notes on RungeKutta), writes byte-identical files, the same
flows index and the same final time.  With the float-float build it writes
flow files within 1e-10 of them."""
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from ibis_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "prep_ramp64x32")
REF = json.load(open(os.path.join(HERE, "golden", "prep_ramp64x32_reference.json")))


def run(tmp_path, precision, aliased=True):
    d = tmp_path / precision
    shutil.copytree(CASE, d)
    cfg_path = d / "config" / "config.json"
    cfg = json.load(open(cfg_path))
    if aliased:
        cfg["solver"]["stage_derivatives"] = "aliased"
    with open(cfg_path, "w") as f:
        json.dump(cfg, f, indent=4)
    r = subprocess.run([build.DRIVER, "--case", str(d), "--precision", precision], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return d


def test_exact_driver_writes_the_reference_flow_files(tmp_path):
    d = run(tmp_path, "f64_exact")
    flows = open(d / "io" / "flow" / "flows").read().split()
    assert flows == REF["flows"]
    last = d / "io" / "flow" / REF["last_flow_dir"]
    assert json.load(open(last / "meta_data.json"))["time"] == REF["meta_data"]["time"]
    for name, digest in REF["sha256"].items():
        assert hashlib.sha256(open(last / name, "rb").read()).hexdigest() == digest, name


def test_float_float_driver_stays_within_1e_minus_10(tmp_path):
    exact = run(tmp_path, "f64_exact") / "io" / "flow" / REF["last_flow_dir"]
    ff = run(tmp_path, "mixed_ff") / "io" / "flow" / REF["last_flow_dir"]
    for name in REF["sha256"]:
        a = np.fromfile(ff / name, np.float64)
        b = np.fromfile(exact / name, np.float64)
        scale = np.linalg.norm(b) if name != "vy" else np.linalg.norm(np.fromfile(exact / "vx", np.float64))
        assert np.linalg.norm(a - b) <= 1e-10 * scale, name
