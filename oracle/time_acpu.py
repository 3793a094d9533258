#!/usr/bin/env python
"""Single-thread timing of the reference's own C host path (ArmandoThrust/acpu.c)
on the 2D dam-break geometry of the benchmark (dx = 1 mm, 2,000,000 fluid +
30,018 wall particles, h = 1.3 dx, Wendland C2).

Test infrastructure, like the rest of oracle/: a CPU speed datapoint beside
the FP64 oracle, not an accuracy reference (acpu.c integrates with TVD-RK3 and
the continuity equation, acpu.c:2338-2379, a different scheme from the CERN
leapfrog the GPU step follows).

One reference time step is `RKintegrateHost`'s loop body (acpu.c:2360-2373),
run by oracle/acpu_driver.py: acpu.c's compiled neighbour list and three RK
stages, with a numpy sort and state backup in place of the two pieces bound
to MAXP = 441 particles, whose time is reported separately ("stand-in").

Materials follow acpu.c's `initDamBreak` (acpu.c:1784-1902): fluid material 1
(Tait, hMatType = 4), walls material -1; gravity through hLoad[0].

  make -C oracle ref && python oracle/time_acpu.py [--steps 3] [--dx 0.001]

Prints one JSON object: seconds per step of each part, particle-steps/s, and
the FP64 oracle's single-thread rate on the same host and geometry.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--dx", type=float, default=1.0e-3)
    ap.add_argument("--oracle-steps", type=int, default=2)
    args = ap.parse_args()

    from acpu_driver import AcpuRun
    from armando_gb300 import cases
    import oracle as O

    case = cases.dam_break(dx=args.dx)
    n = case.n
    rho0, c0 = float(case.params.rho0), float(case.params.c0)
    run = AcpuRun(case.x.reshape(n, 2), case.v.reshape(n, 2), case.mass, case.rho, case.p,
                  case.u, case.h, np.where(case.itype > 0, 1, -1), np.full(n, c0, np.float32),
                  {1: (4, [rho0, c0, -1.0e12])}, case.dt, gravity=(0.0, -9.81))
    for s in range(args.steps):
        r0, s0 = run.seconds_ref, run.seconds_stand_in
        run.step()
        print(f"step {s}: acpu.c {run.seconds_ref - r0:.2f} s, stand-in "
              f"{run.seconds_stand_in - s0:.2f} s", file=sys.stderr, flush=True)
    if not np.isfinite(run.a["PosX"]).all():
        raise RuntimeError("acpu.c run produced non-finite positions")

    st = O.State(case)
    O.integrate_gather(st, 1, 1, case.dt, 1)
    t0 = time.perf_counter()
    O.integrate_gather(st, 2, args.oracle_steps, case.dt, 1)
    t_or = (time.perf_counter() - t0) / args.oracle_steps

    per = (run.seconds_ref + run.seconds_stand_in) / args.steps
    out = {
        "workload": f"dam break 2D, {case.n_fluid} fluid + {case.n_wall} wall particles, "
                    f"dx = {args.dx}",
        "host": f"{platform.machine()}, {os.cpu_count()} hardware threads",
        "threads": 1,
        "acpu_steps": args.steps,
        "acpu_s_per_step": run.seconds_ref / args.steps,
        "stand_in_s_per_step": run.seconds_stand_in / args.steps,
        "acpu_particle_steps_per_s": n / per,
        "acpu_force_evaluations_per_step": 3,
        "oracle_steps": args.oracle_steps,
        "oracle_s_per_step": t_or,
        "oracle_particle_steps_per_s": n / t_or,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
