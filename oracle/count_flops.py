"""Algorithmic FLOPs per particle-step of the benchmark workloads.

Counts the operations one iteration of the reference's algorithm takes
(oracle/armando_oracle_flops.hpp: the FP64 pair-loop restatement run on an
op-counting real) on each workload's state after its first iteration, and
writes profiles/flops.json, which bench.py reads for its FP32 roof.

  python oracle/count_flops.py [--out profiles/flops.json]

The 3D channel is counted on a 252 x 63 x 63 section of the same channel
(identical spacing, walls and physics): the count per particle is a bulk
property, and the full 8.8M-particle count takes minutes on one core.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from armando_gb300 import cases  # noqa: E402


def count(case, its=2):
    st = O.State(case)
    O.step(st, 1, case.dt)  # the first iteration's half kick; count the next one
    t0 = time.perf_counter()
    tot, search = O.flops(st, its, case.dt)
    return {"particles": case.n, "flop_per_particle": tot / case.n,
            "search_flop_per_particle": search / case.n, "its": its,
            "seconds": round(time.perf_counter() - t0, 2)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(REPO, "profiles", "flops.json"))
    args = ap.parse_args()
    out = {"what": "FLOPs of one iteration of the reference algorithm (link_list, pairs "
                   "j > i once, density, EOS, forces, art. visc/heat, ext. heat, leapfrog) "
                   "per particle, counted by the FP64 pair-loop oracle on an op-counting "
                   "real; +,-,*,/,sqrt,exp = 1 each",
           "command": "python oracle/count_flops.py"}
    out["dambreak2d"] = count(cases.dam_break())
    print("dambreak2d", out["dambreak2d"], flush=True)
    ch = cases.channel(n_x=252, n_yz=63, length=0.2, width=0.05)
    out["channel3d"] = count(ch)
    out["channel3d"]["sample"] = "252 x 63 x 63 section (same dx, walls, physics)"
    print("channel3d", out["channel3d"], flush=True)
    out["dambreak2d_adjoint"] = count(cases.adjoint_dam_break())
    print("adjoint", out["dambreak2d_adjoint"], flush=True)
    json.dump(out, open(args.out, "w"), indent=1)


if __name__ == "__main__":
    main()
