"""Times the reference itself (ibis's own sources compiled unchanged against the
project's subset headers, oracle/_ref, built by oracle.ref.build) on this host's
cores: FiniteVolume::compute_dudt alone (median of several calls after a warm-up)
and whole ssp-rk3 steps (RungeKutta::take_step on a written case directory), on
the benchmark's CPU-runnable configurations (the cube as a channel: the
reference has no periodic boundary), with the Serial and the OpenMP
variant of the Kokkos-subset header, and the oracle's OpenMP restatement beside
them.  Rates are Mcell-updates/s (one valid cell through one Runge-Kutta stage;
a residual evaluation counts as one).  Labelled "reference code on a project
Kokkos-subset OpenMP backend": it is not the Kokkos OpenMP backend.

    python oracle/time_reference.py [--omp-threads 8] [--box 64,96] [--out FILE]
"""
import argparse
import json
import os
import statistics
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)  # the repository root, not this directory (whose oracle.py shadows the package)

import numpy as np  # noqa: E402

from ibis_gb300 import grids  # noqa: E402
from oracle import ref  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402


def cases(boxes):
    g, c, inf = grids.ramp_case(256, 128)
    n = g.num_cells
    yield "ramp 256x128 (Euler, 2nd order, Barth-Jespersen, Hanel)", g, c, \
        (np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    g, c, inf = grids.flat_plate_case(512, 256)
    n = g.num_cells
    yield "flat plate 512x256 (viscous)", g, c, \
        (np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    # the reference has no periodic boundary (boundary.cpp:449-479): the cube as a
    # channel (supersonic in/out, slip walls) with the same cells and kernels
    gas = grids.ideal_gas(287.0)
    inflow = grids.flow_state(gas, 300.0, 1e5, 700.0, 30.0, 20.0)
    bnds = {"west": grids.supersonic_inflow(inflow), "east": grids.supersonic_outflow(),
            "south": grids.slip_wall(), "north": grids.slip_wall(), "bottom": grids.slip_wall(),
            "top": grids.slip_wall()}
    rng = np.random.default_rng(0)
    for b in boxes:
        g = grids.box_3d(b)
        c = grids.make_config(3, bnds, gas=gas)
        n = g.num_cells
        st = tuple(np.full(n, inflow[k]) * (1.0 + 0.02 * rng.standard_normal(n)) for k in ("T", "p", "vx", "vy", "vz"))
        yield f"channel cube {b}^3 (Euler, 2nd order)", g, c, st


def time_residual(make, reps):
    r = make()
    r.residual()
    ts = []
    for _ in range(reps):
        t = time.perf_counter()
        r.residual()
        ts.append(time.perf_counter() - t)
    return statistics.median(ts)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--omp-threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--box", default="64,96")
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--out", default="")
    args = ap.parse_args()
    os.environ.setdefault("OMP_NUM_THREADS", str(args.omp_threads))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    if not ref.available("serial"):
        sys.exit("the reference is not built here: python -c \"from oracle import ref; ref.build('<checkout>')\"")
    boxes = [int(x) for x in args.box.split(",") if x]
    out = {"host_cores": os.cpu_count(), "omp_threads": args.omp_threads, "unit": "Mcell-updates/s",
           "label": "reference code on a project Kokkos-subset backend (not the Kokkos OpenMP backend)", "cases": []}
    for name, g, c, st in cases(boxes):
        n = g.num_cells
        row = {"case": name, "cells": n}
        for kind in ("serial", "openmp"):
            def make(kind=kind):
                r = ref.RefResidual(c, g, kind=kind)
                r.set_initial_condition(*st)
                return r
            row[f"reference_{kind}_residual"] = n / time_residual(make, args.reps) / 1e6
            d = tempfile.mkdtemp()
            grids.write_case(d, g, c, *st)
            rk = ref.RefRungeKutta(d, kind=kind)
            rk.steps(1)
            t = time.perf_counter()
            rk.steps(args.steps)
            row[f"reference_{kind}_rk"] = 3.0 * n * args.steps / (time.perf_counter() - t) / 1e6
        o = Oracle(c, g)
        o.set_initial_condition(*st)
        o.rk_initialise()
        o.rk_steps(1)
        t = time.perf_counter()
        o.rk_steps(args.steps)
        row["oracle_omp_rk"] = 3.0 * n * args.steps / (time.perf_counter() - t) / 1e6
        out["cases"].append(row)
        print(json.dumps(row), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
