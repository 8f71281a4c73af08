"""Benchmark: Mcell-updates/s of the explicit RK residual path on GB300.

Workload (the residual-throughput case): 3-D Euler on a periodic unit box of
n^3 hexahedra (default 256^3 = 16.8M cells), ideal gas gamma=1.4, rho=1 and p=1
plus seeded Fourier modes, divergence-free velocity at rms Mach 0.3; ibis's
default numerics (Hanel flux, 2nd-order MUSCL, Barth-Jespersen, rho_u thermo
pair), ssp-rk3.  One cell-update = one valid cell through one RK stage; one
bench step = one RK step (3 stages).  `value` is the mixed-precision path
(float reconstruction/flux, double accumulation/update); the plain FP64 path
and the mixed path's L2 density error against it are reported alongside.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 256]
Under torchrun each rank advances its own box (weak scaling, no collective on
the data path); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import copy
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic bytes per 3-D cell-update (FP64 state, geometry at the variant's
# precision): read U^(s), U^n, write U^(s+1) + cell geometry + 3.01 faces/cell
B_ALG_3D = {"mixed": 268.0, "f64": 393.0}
KERNELS_PER_STEP = 10  # inviscid ssp-rk3: dt control + (recon, face, update) x 3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="box cells per side")
    ap.add_argument("--cpu-n", type=int, default=96, help="box size of the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-cases", type=int, default=64, help="ramp cases of the batched ensemble (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=200, help="timed RK steps of the batched ensemble")
    ap.add_argument("--batch-accuracy-steps", type=int, default=2000,
                    help="RK steps of the ensemble's accuracy leg (every precision against FP64; 0: skip)")
    ap.add_argument("--adjoint-check", type=int, default=1,
                    help="adjoint gradient vs central differences on the 512x256 steady ramp (0: skip)")
    ap.add_argument("--seq-steps", type=int, default=40, help="timed RK steps per case, one case at a time")
    ap.add_argument("--variants", default="",
                    help="launch variants recon,face,update of the mixed build instead of autotuning (profiling)")
    ap.add_argument("--fused", default="auto", choices=["auto", "on", "off"],
                    help="fused stage for structured blocks: let the autotuner choose, force, or disable")
    ap.add_argument("--march", default="auto", choices=["auto", "on", "off"],
                    help="plane-marching kernel of the fused stage (one 3-D block, TMA-staged planes): let the "
                         "autotuner choose, force, or take the tile kernel")
    ap.add_argument("--march-planes", type=int, default=0, help="planes per CTA of the plane-marching kernel (0: tuned)")
    ap.add_argument("--cell-flux", default="auto", choices=["auto", "on", "off"],
                    help="per-cell flux path (face fluxes recomputed inside the update kernel): let the "
                         "autotuner choose, force, or disable")
    ap.add_argument("--plate-steps", type=int, default=300, help="RK steps of the flat-plate accuracy case (0: skip)")
    ap.add_argument("--renumber-n", type=int, default=56,
                    help="hexahedra per side of the tetrahedral channel of the renumbering leg (6 n^3 cells; 0: skip)")
    ap.add_argument("--renumber-steps", type=int, default=20, help="timed RK steps per ordering of that leg")
    ap.add_argument("--renumber-orders", default="as_generated,shuffled,shuffled_rcm",
                    help="orderings of that leg (comma separated)")
    ap.add_argument("--renumber-only", action="store_true",
                    help="run only the renumbering leg and print its JSON (for profiling its kernels)")
    ap.add_argument("--newton-steps", type=int, default=25, help="Newton steps of the ramp JFNK case (0: skip)")
    ap.add_argument("--first-order-max-steps", type=int, default=400,
                    help="Newton step limit of the first-order ramp's time-to-1e-10 run")
    ap.add_argument("--sweep", default="64,128", help="smaller box sizes timed beside the headline (empty: none)")
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, dist=None, device="cpu"):
    """The job's time: the maximum of x over the ranks of the process group
    (x itself with one process).  The replicas exchange nothing else."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells_per_rank, world, stages, steps, seconds):
    """Mcell-updates/s of the whole job: every rank advances its own replica."""
    return world * cells_per_rank * stages * steps / seconds / 1e6


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# The mixed RK stage in use, its name in the roofline block and the committed ncu
# summary whose stage traffic (traffic_bytes_per_stage_<n>) belongs to it.
STAGE_PATHS = {
    "three_kernel": ("rk_stage (recon + face + update kernels of one stage)", "rk_stage_box128_mixed_full.md"),
    "march": ("k_march_stage (plane-marching fused stage, TMA-staged planes)", "march_stage_box128.md"),
    "tile": ("k_fused_stage (tile-fused stage)", None),
    "cell_flux": ("rk_stage (recon + per-cell flux update kernels of one stage)", None),
}


def stage_path(fused_enabled, march, cell_flux_enabled):
    if fused_enabled:
        return "march" if march else "tile"
    return "cell_flux" if cell_flux_enabled else "three_kernel"


def stage_traffic(summary, n):
    """DRAM bytes of one stage at n^3 from a committed ncu summary, or None."""
    if not summary:
        return None
    path = os.path.join(ROOT, "profiles", summary)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(f"traffic_bytes_per_stage_{n}:"):
            return float(line.split(":")[1].split()[0])
    return None


def f64_flops_per_cell_update(n):
    """FP64 operations per cell-update of the reference algorithm on the n^3
    periodic box: its exact count (tests/golden/flop_counts.json, from the
    restatement instantiated on a counting scalar) is A + B/n."""
    with open(os.path.join(ROOT, "tests", "golden", "flop_counts.json")) as f:
        fit = json.load(f)["flops_per_cell_update"]
    return fit["A"] + fit["B"] / n


def fp64_roofline(value_mcells, n, sm_mhz):
    """The plain FP64 path against the FP64 pipe: algorithmic flops (the
    reference algorithm's count) per second against 2 FP64 FMA lanes per SM per
    clock (ncu's peak_sustained dfma rate on GB300) x 2 flops x SMs x the
    sampled SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    flops = f64_flops_per_cell_update(n)
    achieved = value_mcells * 1e6 * flops / 1e12
    peak = 2 * 2 * sms * sm_mhz * 1e6 / 1e12
    return {"bound": "fp64", "flops_per_cell_update": flops, "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "flops_source": "the reference algorithm (oracle restatement on a counting scalar, "
                            "tests/golden/flop_counts.json); an FMA counts 2, a division or square root 1; "
                            "the FP64 build does fewer (precomputed least-squares weights, one reciprocal per "
                            "cell, two divisions per limited variable), so this is the reference-equivalent rate",
            "peak_kind": f"2 FP64 FMA lanes/SM/clock x 2 flops x {sms} SMs x {sm_mhz:.0f} MHz (sampled)"}


class ClockSampler:
    """nvidia-smi SM clock / throttle samples during the timed region."""

    def __init__(self, device: int):
        self.device, self.samples, self.proc, self.thread = device, [], None, None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_case(n):
    from ibis_gb300 import grids
    grid, config = grids.box_case(n)
    ic = grids.box_initial_condition(n, config["gas_model"], seed=0)
    return grid, config, ic


def cpu_sample(n, steps):
    """The oracle (CPU restatement of the reference) on an n^3 box: Mcell-updates/s."""
    from oracle.oracle import Oracle, num_threads
    grid, config, ic = make_case(n)
    o = Oracle(config, grid)
    o.set_initial_condition(*ic)
    o.rk_initialise()
    o.rk_steps(1)  # warm-up
    t = time.perf_counter()
    o.rk_steps(steps)
    dt = time.perf_counter() - t
    return 3.0 * n ** 3 * steps / dt / 1e6, num_threads(), dt


def batch_measure(args, barrier):
    """Batched ensemble of 2-D compression ramps (grid sizes log-uniform from
    64x32 to 512x256 cells, Mach U[1.5,4], ramp angle U[5,20] deg, T U[200,400] K,
    uniform inflow initial state): all cases advanced together by one CUDA graph
    per RK step, against the same cases run one after another, each through its
    own context (its own graph per step).  Aggregate Mcell-updates/s, and the
    per-case relative L2 density error of the mixed path against the FP64 path."""
    from ibis_gb300 import Batch, Simulation, grids
    ens = grids.ramp_ensemble(args.batch_cases, seed=0)
    sims, ics = [], []
    for g, c, inf, _ in ens:
        sims.append(Simulation(c, g))
        n = g.num_cells
        ics.append([np.full(n, inf[k]) for k in ("T", "p", "vx", "vy")])
    del ens
    cells = sum(s.num_cells for s in sims)
    batch = Batch(sims)
    ic_all = [np.concatenate([ic[q] for ic in ics]) for q in range(4)]

    # batched: every case in the same launches
    batch.set_primitives(*ic_all)
    tune = batch.autotune("mixed")
    fused = batch.fused_info()
    cellf = batch.cell_flux_info()
    batch.take_steps(args.warmup, "mixed")
    barrier()
    t0 = time.perf_counter()
    st = batch.take_steps(args.batch_steps, "mixed")
    barrier()
    wall_b = time.perf_counter() - t0
    ms_b = st["device_ms"]
    rho_mixed = batch.split(batch.conserved()[:, 0].copy())
    batch.set_primitives(*ic_all)
    batch.take_steps(args.warmup + args.batch_steps, "f64")
    rho_f64 = batch.split(batch.conserved()[:, 0].copy())
    errs = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(rho_mixed, rho_f64)]

    # accuracy over the configured run length: every precision for
    # args.batch_accuracy_steps steps against the FP64 path, per case; the FP64
    # path without fused multiply-adds shows how far rounding alone moves a case
    acc = None
    if args.batch_accuracy_steps > 0:
        from ibis_gb300.adjoint import _force, _wall_faces
        n_acc = args.batch_accuracy_steps
        rho_acc, p_acc, U_acc, rate_acc = {}, {}, {}, {}
        for prec in ("f64", "f64_exact", "mixed", "mixed_ff"):
            batch.set_primitives(*ic_all)
            if prec == "mixed_ff":
                batch.autotune(prec)
                batch.set_primitives(*ic_all)
            sa = batch.take_steps(n_acc, prec)
            rate_acc[prec] = cells * 3.0 * n_acc / (sa["device_ms"] / 1e3) / 1e6
            U_all = batch.conserved()
            rho_acc[prec] = batch.split(U_all[:, 0].copy())
            p_acc[prec] = batch.split(batch.primitives()["p"].copy())
            U_acc[prec] = batch.split(U_all)
        # the integrated pressure force on each case's ramp wall (x >= 0.2), from its state
        walls = [(_wall_faces(sm, "wall"), sm.dump("face_geometry")) for sm in sims]

        def force(prec, j):
            (faces, wcells), fg = walls[j]
            return float(_force(sims[j], U_acc[prec][j], fg, faces, wcells, 0.2, 1)[0])
        acc = {"steps": n_acc, "batched_rate": rate_acc,
               "errors": "relative to the FP64 build, per case: L2 and max of density and pressure, and the "
                         "integrated ramp-wall pressure force"}
        for prec in ("f64_exact", "mixed", "mixed_ff"):
            e = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(rho_acc[prec], rho_acc["f64"])]
            em = [float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(rho_acc[prec], rho_acc["f64"])]
            ep = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(p_acc[prec], p_acc["f64"])]
            epm = [float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(p_acc[prec], p_acc["f64"])]
            ef = [abs(force(prec, j) - force("f64", j)) / abs(force("f64", j)) for j in range(len(sims))]
            acc[prec] = {"max": max(e), "median": float(np.median(e)), "cases_above_1e-6": int(sum(x > 1e-6 for x in e)),
                         "rho_max_err_max": max(em), "p_l2_err_max": max(ep), "p_max_err_max": max(epm),
                         "wall_force_err_max": max(ef), "wall_force_err_median": float(np.median(ef))}

    # sequential: one case at a time, each with its own context and graph
    for s, ic in zip(sims, ics):
        s.set_primitives(*ic)
        s.take_steps(args.warmup, "mixed")
    barrier()
    dev_ms = 0.0
    t0 = time.perf_counter()
    for s in sims:
        dev_ms += s.take_steps(args.seq_steps, "mixed")["device_ms"]
    barrier()
    wall_s = time.perf_counter() - t0
    upd_b = cells * 3.0 * args.batch_steps
    upd_s = cells * 3.0 * args.seq_steps
    return {"workload": f"{len(sims)} independent 2-D compression ramps, {cells} cells in all, ssp-rk3, "
                        "Hanel, 2nd-order MUSCL + Barth-Jespersen, mixed precision",
            "cases": len(sims), "cells": cells, "autotune": tune["variants"],
            "fused_stage": {k: fused[k] for k in ("enabled", "fused_ms", "generic_ms")},
            "cell_flux": {k: cellf[k] for k in ("enabled", "variant", "cell_ms", "generic_ms")},
            "batched": {"value": upd_b / (ms_b / 1e3) / 1e6, "unit": "Mcell-updates/s",
                        "steps": args.batch_steps, "ms_per_step": ms_b / args.batch_steps,
                        "wall_value": upd_b / wall_b / 1e6},
            "sequential": {"value": upd_s / wall_s / 1e6, "unit": "Mcell-updates/s",
                           "steps_per_case": args.seq_steps, "ms_per_step_all_cases": wall_s * 1e3 / args.seq_steps,
                           "device_only_value": upd_s / (dev_ms / 1e3) / 1e6},
            "speedup": (upd_b / (ms_b / 1e3)) / (upd_s / wall_s),
            "speedup_vs_device_only": (upd_b / (ms_b / 1e3)) / (upd_s / (dev_ms / 1e3)),
            "rho_rel_l2_err_mixed_vs_f64": {"max": max(errs), "median": float(np.median(errs)),
                                            "steps": args.warmup + args.batch_steps},
            "accuracy": acc}


def sweep_measure(args):
    """The residual-throughput sweep of the box at the smaller sizes (the headline
    size is the main line): mixed and FP64 Mcell-updates/s, 20 timed steps each."""
    from ibis_gb300 import Simulation
    out = {}
    for n in [int(x) for x in args.sweep.split(",") if x.strip()]:
        grid, config, ic = make_case(n)
        sim = Simulation(config, grid)
        del grid
        row = {}
        for prec in ("mixed", "f64"):
            sim.set_primitives(*ic)
            sim.take_steps(3, prec)
            st = sim.take_steps(20, prec)
            row[prec] = sim.num_cells * 3.0 * 20 / (st["device_ms"] / 1e3) / 1e6
        row["fused_stage"] = sim.fused_info()["enabled"]
        row["cell_flux"] = sim.cell_flux_info()["enabled"]
        out[f"{n}^3"] = row
    return out


def plate_measure(args):
    """Laminar flat plate (512 x 256, wall-normal stretching 1.05 from 1e-5 m, Mach 2,
    T 220 K, Re 1e5 per metre, Sutherland air with Pr 0.71, adiabatic no-slip wall
    from x = 0): args.plate_steps RK steps from the uniform inflow state in the
    mixed and FP64 builds; relative L2 and max errors of density, pressure and
    wall skin friction of the mixed build against the FP64 one (which matches
    the FP64 oracle to 1e-12 per cell), and both builds' throughput."""
    from ibis_gb300 import Simulation, grids
    g, c, inf = grids.flat_plate_case(512, 256)
    out = {"workload": "2-D laminar flat plate 512x256, ssp-rk3, Hanel, MUSCL + Barth-Jespersen, viscous",
           "steps": args.plate_steps}
    q_inf = 0.5 * inf["rho"] * inf["vx"] ** 2
    res = {}
    for prec in ("mixed", "f64"):
        sim = Simulation(c, g)
        n = sim.num_cells
        sim.set_primitives(np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
        sim.take_steps(2, prec)
        st = sim.take_steps(args.plate_steps, prec)
        pr = sim.primitives()
        sim.compute_dudt(prec)
        flux = sim.dump("face_flux_mixed" if prec == "mixed" else "face_flux")
        sel = sim.dump("ghost_boundary") == sorted(c["grid"]["boundaries"]).index("wall")
        faces = sim.dump("ghost_face")[sel]
        ny = sim.dump("face_geometry")[1, faces]
        cf = -flux[faces, 1] / (ny * q_inf)  # wall shear / dynamic pressure (flux x-momentum = -tau_xy n_y)
        res[prec] = (pr["rho"], pr["p"], cf)
        out[f"{prec}_value"] = n * 3.0 * args.plate_steps / (st["device_ms"] / 1e3) / 1e6
    for k, name in enumerate(("rho", "p", "cf")):
        a, b = res["mixed"][k], res["f64"][k]
        out[f"{name}_rel_l2_err"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        out[f"{name}_rel_max_err"] = float(np.abs(a - b).max() / np.abs(b).max())
    out["unit"] = "Mcell-updates/s"
    return out


def renumber_measure(args):
    """Cell order and throughput on an unstructured grid: the 3-D tetrahedral
    channel of 6 n^3 cells (grids.tet_channel_case: supersonic in/out, slip walls;
    second order, Hanel, Barth-Jespersen, mixed build) in three orders -- as
    generated (hexahedron by hexahedron), the cells shuffled (seeded), and the
    shuffled grid renumbered by reverse Cuthill-McKee inside the context -- with
    the cell graph's bandwidth and the RK-step throughput of each."""
    from ibis_gb300 import Simulation, grids
    n = args.renumber_n
    g0, c, inf = grids.tet_channel_case(n)
    gs = grids.shuffle_cells(g0, 0)
    rng = np.random.default_rng(7)
    N = g0.num_cells
    st = [np.full(N, inf[k]) * (1.0 + 0.02 * rng.standard_normal(N)) for k in ("T", "p", "vx", "vy", "vz")]
    out = {"workload": f"tetrahedral channel {N} cells (6 x {n}^3), ssp-rk3, Hanel, MUSCL + Barth-Jespersen, "
                       f"mixed build, {args.renumber_steps} timed steps per ordering", "cells": N,
           "unit": "Mcell-updates/s"}
    perm = np.random.default_rng(0).permutation(N)  # shuffle_cells(g0, 0): cell k is cell perm[k] of g0
    for name, grid, mode in (("as_generated", g0, "none"), ("shuffled", gs, "none"), ("shuffled_rcm", gs, "rcm")):
        if name not in args.renumber_orders.split(","):
            continue
        cc = copy.deepcopy(c)
        cc["grid"]["renumber"] = mode
        sim = Simulation(cc, grid)
        sim.set_primitives(*(st if grid is g0 else [a[perm] for a in st]))
        if args.variants:  # fixed launch variants (no autotuning launches)
            sim.set_launch_variants("mixed", *(int(x) for x in args.variants.split(",")))
        sim.take_steps(3, "mixed")
        r = sim.take_steps(args.renumber_steps, "mixed")
        info = sim.numbering()
        out[name] = {"value": N * 3.0 * args.renumber_steps / (r["device_ms"] / 1e3) / 1e6,
                     "renumbered": info["renumbered"], "bandwidth_reference": info["bandwidth_reference"],
                     "bandwidth_internal": info["bandwidth_internal"]}
    return out


def jfnk_measure(args):
    """Steady Jacobian-free Newton-Krylov on the Hicks-Henne ramp (512 x 256,
    15 degrees, 16 bump amplitudes U[-0.002, 0.002] m and inflow Mach U[1.5, 3]
    drawn from seed 0; GMRES of 30 vectors per Newton step, residual-based CFL):
    args.newton_steps steps from the uniform inflow state with their residual
    history, and the rates of the tangent (Jv) and adjoint (J^T w) products and
    of one adjoint continuation step at the final state."""
    import torch
    from ibis_gb300 import Simulation, grids
    from ibis_gb300.adjoint import wall_force
    rng = np.random.default_rng(0)
    mach = float(rng.uniform(1.5, 3.0))
    bumps = rng.uniform(-0.002, 0.002, 16)
    cfl = {"type": "residual_based", "growth_threshold": 1.0, "power": 1.0, "start_cfl": 2.0, "max_cfl": 1e12}
    solver = grids.steady_state(cfl=cfl, max_iters=30, tol=1e-3, max_steps=1000)
    g, c, inf = grids.ramp_bump_case(512, 256, mach=mach, bumps=bumps, solver=solver)
    sim = Simulation(c, g)
    n = sim.num_cells
    sim.set_primitives(np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    sim.steady_initialise("f64")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = [sim.newton_step("f64") for _ in range(args.newton_steps)]
    torch.cuda.synchronize()
    newton_s = time.perf_counter() - t0
    U = torch.tensor(sim.conserved(), dtype=torch.float64, device="cuda")
    v = torch.randn_like(U) * U.abs().mean(dim=0)
    out_t = torch.empty_like(U)

    def rate(fn, reps=20):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return reps / (time.perf_counter() - t)

    stream = torch.cuda.current_stream()
    jv_rate = rate(lambda: sim.matrix_vector_product_into(v, out_t, 1.0, stream=stream))
    vjp_rate = rate(lambda: sim.vector_jacobian_product_into(v, out_t, stream=stream))
    _, dJ = wall_force(sim, x_min=0.2)
    gt = torch.tensor(dJ, dtype=torch.float64, device="cuda")
    lam = torch.zeros_like(gt)
    t = time.perf_counter()
    ast = sim.adjoint_step(gt, lam, 10.0)
    adj_s = time.perf_counter() - t
    rel = [h["relative_residual"] for h in hist]
    # time to a relative residual of 1e-10: the same ramp and solver with first-order
    # reconstruction (the limited second-order residual stalls well above it)
    cfl1 = {"type": "residual_based", "growth_threshold": 1.0, "power": 1.5, "start_cfl": 5.0, "max_cfl": 1e12}
    solver1 = grids.steady_state(cfl=cfl1, max_iters=30, tol=1e-3, max_steps=1000)
    g1, c1, inf1 = grids.ramp_bump_case(512, 256, mach=mach, bumps=bumps, solver=solver1, order=1)
    s1 = Simulation(c1, g1)
    s1.set_primitives(np.full(n, inf1["T"]), np.full(n, inf1["p"]), np.full(n, inf1["vx"]), np.full(n, inf1["vy"]))
    s1.steady_initialise("f64")
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    hist1 = []
    while len(hist1) < args.first_order_max_steps and time.perf_counter() - t1 < 30.0:
        hist1.append(s1.newton_step("f64")["relative_residual"])
        if hist1[-1] < 1e-10:
            break
    torch.cuda.synchronize()
    first = {"workload": "the same ramp with first-order reconstruction, residual-based CFL (power 1.5, start 5), "
                         "GMRES(30), FP64",
             "newton_steps": len(hist1), "seconds": time.perf_counter() - t1, "relative_residual": hist1[-1],
             "reached_1e-10": hist1[-1] < 1e-10,
             "residual_history_every_10": [float(f"{x:.3e}") for x in hist1[::10]]}
    return {"workload": f"2-D Hicks-Henne ramp 512x256 (15 deg, Mach {mach:.3f}, 16 bumps), MUSCL + Barth-Jespersen, "
                        "JFNK with GMRES(30), FP64",
            "newton_steps": len(hist), "ms_per_newton_step": newton_s * 1e3 / len(hist),
            "relative_residual": rel[-1], "residual_history": [float(f"{x:.3e}") for x in rel],
            "gmres_iterations": [h["gmres_iterations"] for h in hist],
            "jv_per_s": jv_rate, "vjp_per_s": vjp_rate,
            "adjoint_step_ms": adj_s * 1e3, "adjoint_step_gmres_iterations": ast["gmres_iterations"],
            "time_to_1e-10_first_order": first}


def headline_config(n, world):
    """The config of the headline line (both arms): the n^3 periodic box."""
    return {"workload": f"3-D Euler periodic box {n}^3 (residual-throughput case), ssp-rk3, "
                        f"Hanel, 2nd-order MUSCL + Barth-Jespersen, rho_u",
            "cells_per_gpu": n ** 3, "faces_per_gpu": 3 * n ** 3 + 3 * n ** 2, "stages_per_step": 3,
            "l2": "inputs larger than L2 (state + geometry several GB per GPU), no flush",
            "parallelism": f"replicas x{world}"}


def run_reference(args, world, rank):
    """--impl reference: the oracle port of the reference's CPU path, all host threads."""
    if rank != 0:
        return
    from oracle.oracle import Oracle, num_threads
    n = args.cpu_n
    grid, config, ic = make_case(n)
    o = Oracle(config, grid)
    o.set_initial_condition(*ic)
    o.rk_initialise()
    o.rk_steps(args.warmup)
    t = time.perf_counter()
    o.rk_steps(args.steps)
    dt = time.perf_counter() - t
    value = 3.0 * n ** 3 * args.steps / dt / 1e6
    sample = (f"oracle port (C++ restatement of ibis's FP64 path, OpenMP) on a {n}^3 periodic box, "
              f"{args.steps} ssp-rk3 steps per timed call (each bench step is one ssp-rk3 step of that box); "
              f"the {args.n}^3 grid does not fit a bounded CPU run")
    line = {"impl": "reference", "metric": "Mcell-updates/s", "value": value, "unit": "Mcell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(headline_config(args.n, world),
                           workload=f"3-D Euler periodic box measured at {n}^3 on the host cores (a bounded "
                                    f"CPU sample of the {args.n}^3 residual-throughput case: ssp-rk3, Hanel, "
                                    f"2nd-order MUSCL + Barth-Jespersen, rho_u; the rate is per cell-update)",
                           measured_cells_per_gpu=n ** 3),
            "cpu_baseline": {"value": value, "unit": "Mcell-updates/s", "cores": num_threads(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from ibis_gb300 import Simulation

    n = args.n
    grid, config, ic = make_case(n)
    sim = Simulation(config, grid)
    N = sim.num_cells
    del grid

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def max_over_ranks_(x):
        return max_over_ranks(x, dist, "cuda")

    # --- headline: mixed precision, device-resident state
    sim.set_primitives(*ic)
    sim.set_fused({"auto": -1, "on": 1, "off": 0}[args.fused])
    if sim.fused_info()["eligible"] and (args.march != "auto" or args.march_planes):
        sim.set_fused_kind({"auto": -1, "on": 1, "off": 0}[args.march], args.march_planes)
    sim.set_cell_flux({"auto": -1, "on": 1, "off": 0}[args.cell_flux])
    if args.variants:
        r, f, u = (int(x) for x in args.variants.split(","))
        sim.set_launch_variants("mixed", r, f, u)
        tune_mixed = {"variants": {"recon": r, "face": f, "update": u}, "ms": None}
    else:
        tune_mixed = sim.autotune("mixed")
    fused = sim.fused_info()
    fkind = sim.fused_kind()
    cellf = sim.cell_flux_info()
    sim.take_steps(args.warmup, "mixed")
    barrier()
    with ClockSampler(local) as clk:
        st = sim.take_steps(args.steps, "mixed")
        barrier()
    ms_mixed = max_over_ranks_(st["device_ms"])
    rho_mixed = sim.conserved()[:, 0].copy()
    p_mixed = sim.primitives()["p"].copy()
    value = whole_job_rate(N, world, 3, args.steps, ms_mixed / 1e3)

    # --- plain FP64 path over the same steps from the same state, and its accuracy reference
    sim.set_primitives(*ic)
    tune_f64 = sim.autotune("f64")
    sim.take_steps(args.warmup, "f64")
    barrier()
    st64 = sim.take_steps(args.steps, "f64")
    barrier()
    ms_f64 = max_over_ranks_(st64["device_ms"])
    rho_f64 = sim.conserved()[:, 0]
    p_f64 = sim.primitives()["p"]
    value_f64 = whole_job_rate(N, world, 3, args.steps, ms_f64 / 1e3)
    l2_err = float(np.linalg.norm(rho_mixed - rho_f64) / np.linalg.norm(rho_f64))
    max_err = float(np.abs(rho_mixed - rho_f64).max() / np.abs(rho_f64).max())
    p_l2_err = float(np.linalg.norm(p_mixed - p_f64) / np.linalg.norm(p_f64))
    p_max_err = float(np.abs(p_mixed - p_f64).max() / np.abs(p_f64).max())

    # --- the float-float path (MIXED_FF) over the same steps from the same state
    sim.set_primitives(*ic)
    tune_ff = sim.autotune("mixed_ff")
    sim.take_steps(args.warmup, "mixed_ff")
    barrier()
    stff = sim.take_steps(args.steps, "mixed_ff")
    barrier()
    ms_ff = max_over_ranks_(stff["device_ms"])
    rho_ff = sim.conserved()[:, 0]
    value_ff = whole_job_rate(N, world, 3, args.steps, ms_ff / 1e3)
    l2_err_ff = float(np.linalg.norm(rho_ff - rho_f64) / np.linalg.norm(rho_f64))

    # --- kernel breakdown of one residual evaluation (CUDA events on the context stream)
    kt = sim.kernel_times("mixed", reps=5)

    # --- end to end through the C ABI with host (pinned) buffers: per step,
    # upload of the conserved state, one RK step, read-back of the new state
    nc = sim.n_conserved
    host_in = torch.empty((N, nc), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty((N, nc), dtype=torch.float64, pin_memory=True).numpy()
    sim.set_primitives(*ic)
    sim.conserved(out=host_in)
    e2e_steps = max(3, args.steps)  # as many steps as the device-timed headline
    for _ in range(2):
        sim.set_conserved(host_in)
        sim.take_steps(1, "mixed")
        sim.conserved(out=host_out)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.set_conserved(host_in)
        sim.take_steps(1, "mixed")
        sim.conserved(out=host_out)
    barrier()
    e2e_seq_s = max_over_ranks_(time.perf_counter() - t0)
    e2e_seq_value = whole_job_rate(N, world, 3, e2e_steps, e2e_seq_s)
    # the same jobs through ibisgb_rk_run_host: each step's upload and read-back on
    # copy streams, overlapping the neighbouring steps' kernels
    host_out2 = torch.empty((N, nc), dtype=torch.float64, pin_memory=True).numpy()
    outs = [host_out if j % 2 == 0 else host_out2 for j in range(e2e_steps)]
    sim.take_steps_host([host_in, host_in], [host_out, host_out2], 1, "mixed")
    barrier()
    t0 = time.perf_counter()
    sim.take_steps_host([host_in] * e2e_steps, outs, 1, "mixed")
    barrier()
    e2e_s = max_over_ranks_(time.perf_counter() - t0)
    e2e_value = whole_job_rate(N, world, 3, e2e_steps, e2e_s)

    peak, peak_kind = measured_peak_hbm()
    stage_ms = ms_mixed / args.steps / 3.0
    achieved = B_ALG_3D["mixed"] * N / (stage_ms / 1e3) / 1e9
    # DRAM bytes of one stage of the path in use, from its committed ncu summary
    stage_kernel, summary = STAGE_PATHS[stage_path(fused["enabled"], fkind["march"], cellf["enabled"])]
    traffic = stage_traffic(summary, n)

    batch = batch_measure(args, barrier) if args.batch_cases > 0 else None
    plate = plate_measure(args) if args.plate_steps > 0 and rank == 0 else None
    renum = renumber_measure(args) if args.renumber_n > 0 and rank == 0 else None
    sweep = sweep_measure(args) if args.sweep and rank == 0 else None
    jfnk = jfnk_measure(args) if args.newton_steps > 0 and rank == 0 else None
    if jfnk is not None and args.adjoint_check:
        from ibis_gb300.adjoint import gradient_check
        t_adj = time.perf_counter()
        gc = gradient_check(512, 256, seed=0, order=1, step=1e-6)
        jfnk["adjoint_gradient_check"] = {
            "workload": "512x256 Hicks-Henne ramp, first order, Mach and 16 bumps from seed 0; adjoint gradient of "
                        "the ramp pressure force vs central differences (step 1e-6) of re-converged states",
            "relative_errors": {"mach": gc["relative_errors"][0],
                                **{f"bump_{k}": e for k, e in enumerate(gc["relative_errors"][1:])}},
            "max_relative_error": max(gc["relative_errors"]),
            "base_relative_residual": gc["base_relative_residual"], "adjoint_steps": gc["adjoint_steps"],
            "adjoint_relative_residual": gc["adjoint_relative_residual"], "seconds": time.perf_counter() - t_adj}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, secs = cpu_sample(args.cpu_n, 4)
        cpu = {"value": v, "unit": "Mcell-updates/s", "cores": cores, "kind": "port",
               "sample": f"oracle (C++ restatement of ibis's FP64 path, OpenMP) on a {args.cpu_n}^3 "
                         f"periodic box, 4 ssp-rk3 steps ({secs:.1f} s)"}

    if rank == 0:
        line = {
            "metric": "Mcell-updates/s", "value": value, "unit": "Mcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mixed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 flux / f64 accumulate+update (mixed)", "data": "synthetic",
            "config": headline_config(n, world),
            "f64": {"value": value_f64, "ms_per_step": ms_f64 / args.steps,
                    "mixed_speedup": value / value_f64,
                    "fp64_roofline": fp64_roofline(value_f64, n, clk.summary()["sm_mhz"] or 2070.0)},
            "accuracy": {"rho_rel_l2_err_mixed_vs_f64": l2_err, "rho_rel_max_err_mixed_vs_f64": max_err,
                         "p_rel_l2_err_mixed_vs_f64": p_l2_err, "p_rel_max_err_mixed_vs_f64": p_max_err,
                         "steps": args.warmup + args.steps},
            "mixed_ff": {"value": value_ff, "ms_per_step": ms_ff / args.steps, "speedup_vs_f64": value_ff / value_f64,
                         "rho_rel_l2_err_vs_f64": l2_err_ff, "autotune": tune_ff["variants"],
                         "arithmetic": "float-float (FP32 pipe) gradients, limiters, face states and fluxes; "
                                       "f64 accumulate/update"},
            "kernel_ms": {k: round(v, 4) for k, v in kt.items()},
            "autotune": {"variants_table": Simulation.launch_variants(), "mixed": tune_mixed, "f64": tune_f64,
                         "fused_stage": dict({k: fused[k] for k in ("enabled", "fused_ms", "generic_ms")},
                                             **{k: fkind[k] for k in ("march", "planes_per_cta", "tile_ms",
                                                                      "march_ms")}),
                         "cell_flux": {k: cellf[k] for k in ("enabled", "variant", "cell_ms", "generic_ms")}},
            "batch": batch,
            "sweep": sweep,
            "plate": plate,
            "renumber": renum,
            "jfnk": jfnk,
            "roofline": {"bound": "hbm", "kernel": stage_kernel,
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "bytes_per_cell_update": B_ALG_3D["mixed"],
                         "traffic": traffic, "traffic_per_cell_update": traffic / N if traffic else None,
                         "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one stage "
                                            f"at 128^3, scaled by 8 (profiles/{summary})") if traffic else None},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "Mcell-updates/s", "h2d_bytes_per_step": 8 * nc * N,
                    "d2h_bytes_per_step": 8 * nc * N, "steps": e2e_steps,
                    "api": "ibisgb_rk_run_host: per step the state from pinned host rows, one ssp-rk3 step, the "
                           "new state to pinned host rows; the next step's upload and the previous step's "
                           "read-back run on copy streams during the step's kernels",
                    "sequential_value": e2e_seq_value,
                    "sequential_api": "ibisgb_set_conserved + ibisgb_rk_run + ibisgb_get_conserved per step, "
                                      "each call synchronous"},
            "gpu_launches": (4 if fused["enabled"] else 7 if cellf["enabled"] else KERNELS_PER_STEP) * args.steps + 2,
            "gpu_launches_note": "kernels of the timed headline call: one graph per step (dt control + 3 fused "
                                 "stages, dt control + 3 x recon/cell-flux update, or dt control + 3 x "
                                 "recon/face/update), plus the call's local-dt prologue",
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.renumber_only:
        if rank == 0:
            import torch
            torch.cuda.set_device(local)
            print(json.dumps({"renumber": renumber_measure(args)}), flush=True)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
