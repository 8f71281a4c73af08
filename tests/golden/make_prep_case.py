"""An ibis case directory written by the reference's own, unchanged prep step,
and the flow files the reference's own driver writes for it -- for the test
that runs ibisgb-run on the same directory (tests/test_prep_case_gpu.py).

Where an ibis checkout exists and the reference is built with its pybind11
module (python -c "from oracle import ref; ref.build('<checkout>')" and
make -C oracle -f Makefile.ref REF=<checkout> pyapi), run by hand:

    python tests/golden/make_prep_case.py <ibis checkout>

It writes the 64 x 32 compression ramp (15 degrees) as ramp.su2 and a job.py
for the CPU-runnable benchmark case (Mach 2 at 101325 Pa and 300 K, ideal air
R = 287, Hanel, second-order MUSCL with Barth-Jespersen, ssp-rk3 at CFL 0.5 for
500 steps, slip walls), runs prep.py's main(job.py, share) on them
(src/ibis/ibis/commands/prep/prep.py:1178-1251), and keeps what it wrote in
tests/golden/prep_ramp64x32/ (the input ramp.su2 is left out: prep copied it to
io/grid/0000/block_0000.su2).  Then it runs the reference's make_solver +
Solver::solve on a copy (as `ibis run` does) and records the SHA-256 of the
flow files it writes in tests/golden/prep_ramp64x32_reference.json.
"""
import hashlib
import json
import os
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from ibis_gb300 import grids  # noqa: E402
from oracle import ref  # noqa: E402

CASE = os.path.join(HERE, "prep_ramp64x32")
JOB = '''gas_model = IdealGas(R=287.0)
gas_state = GasState()
gas_state.T = 300.0
gas_state.p = 101325.0
gas_model.update_thermo_from_pT(gas_state)
flow_state = FlowState(gas=gas_state, vx=2.0 * gas_model.speed_of_sound(gas_state), vy=0.0)

config.convective_flux = ConvectiveFlux(flux_calculator=Hanel(), reconstruction_order=2)
config.gas_model = gas_model
config.solver = RungeKutta(cfl=0.5, max_step=500, max_time=1.0, plot_frequency=-1.0, print_frequency=100)
config.grid = Block(
    file_name="ramp.su2",
    initial_condition=flow_state,
    boundaries={
        "inflow": supersonic_inflow(flow_state),
        "outflow": supersonic_outflow(),
        "wall": slip_wall(),
        "top": slip_wall(),
    },
)
'''
OUTPUT_FILES = ["T", "p", "vx", "vy"]


def file_hashes(flow_dir):
    return {name: hashlib.sha256(open(os.path.join(flow_dir, name), "rb").read()).hexdigest()
            for name in OUTPUT_FILES}


def main(checkout):
    if os.path.isdir(CASE):
        shutil.rmtree(CASE)
    os.makedirs(CASE)
    grids.ramp_2d(64, 32).write(os.path.join(CASE, "ramp.su2"))
    with open(os.path.join(CASE, "job.py"), "w") as f:
        f.write(JOB)
    ref.run_prep(CASE, checkout)
    os.remove(os.path.join(CASE, "ramp.su2"))  # prep copied it to io/grid/0000/block_0000.su2
    run = tempfile.mkdtemp()
    shutil.copytree(CASE, run, dirs_exist_ok=True)
    rc = ref.run_case(run)
    flows = open(os.path.join(run, "io", "flow", "flows")).read().split()
    last = os.path.join(run, "io", "flow", flows[-1])
    meta = {"generator": "tests/golden/make_prep_case.py", "solve_result": rc, "flows": flows,
            "last_flow_dir": flows[-1], "meta_data": json.load(open(os.path.join(last, "meta_data.json"))),
            "sha256": file_hashes(last)}
    with open(os.path.join(HERE, "prep_ramp64x32_reference.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(meta)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(sys.argv[0])} <path of an ibis checkout>")
    main(sys.argv[1])
