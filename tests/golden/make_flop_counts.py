"""Writes flop_counts.json: the exact floating-point operation counts of one
ssp-rk3 step (with its time-step estimate) of the reference algorithm on the
periodic-box residual-throughput case, from the oracle's restatement
instantiated on a counting scalar (oracle_core.hpp, Cnt).  The per cell-update
count is exactly A + B/n on an n^3 box (cell and face work; faces per cell are
3 + 3/n); A and B come from n = 16 and 32 and are checked at the other sizes.
Run from the repository root after the oracle is built (make -C oracle)."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from ibis_gb300 import grids  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

ARITH = ("add", "mul", "div", "sqrt", "pow")


def count(n):
    g, c = grids.box_case(n)
    o = Oracle(c, g)
    o.set_initial_condition(*grids.box_initial_condition(n, c["gas_model"], seed=0))
    return o.count_step_flops()


def main():
    sizes = (8, 12, 16, 32)
    counts = {n: count(n) for n in sizes}
    per = {n: sum(counts[n][k] for k in ARITH) / (3 * n ** 3) for n in sizes}
    B = (per[16] - per[32]) / (1 / 16 - 1 / 32)
    A = per[32] - B / 32
    for n in sizes:
        assert abs(A + B / n - per[n]) < 1e-9, n
    out = {"workload": "3-D Euler periodic box n^3, Hanel, 2nd-order MUSCL + Barth-Jespersen, rho_u, ssp-rk3 "
                       "(one step = 3 cell-updates per cell), box_initial_condition seed 0",
           "counts_per_step": {str(n): counts[n] for n in sizes},
           "flops_per_cell_update": {"A": A, "B": B, "form": "A + B / n on an n^3 box",
                                     "arithmetic": list(ARITH)}}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "flop_counts.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(path, A, B)


if __name__ == "__main__":
    main()
