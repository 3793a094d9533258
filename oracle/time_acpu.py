#!/usr/bin/env python
"""Single-thread timing of the reference's own C host path (ArmandoThrust/acpu.c)
on the 2D dam-break geometry of the benchmark (dx = 1 mm, 2,000,000 fluid +
30,018 wall particles, h = 1.3 dx, Wendland C2).

Test infrastructure, like the rest of oracle/: a CPU speed datapoint beside
the FP64 oracle, not an accuracy reference (acpu.c integrates with TVD-RK3 and
the continuity equation, acpu.c:2338-2379, a different scheme from the CERN
leapfrog the GPU step follows).

One reference time step (`RKintegrateHost`'s loop body, acpu.c:2360-2373):
  * neighbour list: `updateHashHost` (acpu.c:2085), a sort by cell hash,
    `updateSetsHost` (acpu.c:2135), `updateListHost` (acpu.c:2201);
  * backup of the step's initial state;
  * `RKstepHost` (acpu.c:2293) three times, alpha = 1, 1/4, 2/3.
acpu.c's own `neighbourListHost` (acpu.c:2245) sorts through a stack array of
MAXP = 441 pairs and `backupDataHost` (acpu.c:1173) copies MAXP entries, so at
two million particles this driver replaces those two pieces:
  * the sort: a stable numpy argsort of the hashes plus the gathers;
  * the backup: numpy copies of the eight arrays.
Their time is reported separately ("stand-in"). Everything else is acpu.c's
compiled code, called through ctypes on arrays this driver owns.

The cell table is padded by one z-plane and one row on each side: acpu.c's
`updateListHost` visits z offsets -1..1 even for 2D grids (nZ = 1), and those
cells read as empty here, as the padding keeps every read in bounds.

Materials follow acpu.c's `initDamBreak` (acpu.c:1784-1902): fluid material 1
(Tait, hMatType = 4), walls material -1; gravity through hLoad[0].

  make -C oracle ref && python oracle/time_acpu.py [--steps 3] [--dx 0.001]

Prints one JSON object: seconds per step of each part, particle-steps/s, and
the FP64 oracle's single-thread rate on the same host and geometry.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

MAXN = 21  # acpu.c:7, neighbour slots per particle
F = C.POINTER(C.c_float)
I = C.POINTER(C.c_int)


class Grid(C.Structure):  # acpu.c:17-21
    _fields_ = [("oX", C.c_float), ("oY", C.c_float), ("oZ", C.c_float), ("size", C.c_float),
                ("nX", C.c_int), ("nY", C.c_int), ("nZ", C.c_int)]


class Simulation(C.Structure):  # acpu.c:23-32
    _fields_ = [(k, C.c_float) for k in ("minX", "maxX", "minY", "maxY", "minZ", "maxZ", "dt")] + \
               [("tsn", C.c_int), ("ssi", C.c_int), ("nsi", C.c_int)]


class Load(C.Structure):  # acpu.c:34-42
    _fields_ = [(k, C.c_float) for k in ("minX", "maxX", "minY", "maxY", "minZ", "maxZ",
                                         "gx", "gy", "gz", "w")]


MODEL_FLOATS = ["Mass", "Smooth", "PosX", "PosY", "PosZ", "VelX", "VelY", "VelZ", "Density",
                "Energy", "Pressure", "Sound", "VelDotX", "VelDotY", "VelDotZ", "DensityDot",
                "EnergyDot", "PosX0", "PosY0", "PosZ0", "VelX0", "VelY0", "VelZ0", "Density0",
                "Energy0"]


class Model(C.Structure):  # acpu.c:69-104, field order kept
    _fields_ = [("pn", C.c_int), ("Material", I)] + [(k, F) for k in MODEL_FLOATS] + \
               [("List", I), ("Hash", I), ("Index", I), ("SetStart", I), ("SetStop", I),
                ("IntDummy", I), ("FloatDummy", F)]


def load_acpu():
    path = os.path.join(HERE, "_ref", "libacpu.so")
    if not os.path.exists(path):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    L = C.CDLL(path)
    L.updateHashHost.argtypes = [C.c_int, Grid, F, F, F, I]
    L.updateSetsHost.argtypes = [C.c_int, I, I, I]
    L.updateListHost.argtypes = [C.c_int, I, I, I, Grid, F, F, F, F]
    L.RKstepHost.argtypes = [C.POINTER(Model), C.c_float]
    return L


def ptr(a, t):
    return a.ctypes.data_as(t)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--dx", type=float, default=1.0e-3)
    ap.add_argument("--oracle-steps", type=int, default=2)
    args = ap.parse_args()

    from armando_gb300 import cases
    import oracle as O

    L = load_acpu()
    case = cases.dam_break(dx=args.dx)
    n = case.n
    xy = case.x.reshape(n, 2)
    fluid = case.itype > 0
    rho0, c0 = float(case.params.rho0), float(case.params.c0)
    h = float(case.h[0])

    mat_type = (C.c_int * 10).in_dll(L, "hMatType")
    mat_prop = ((C.c_float * 10) * 10).in_dll(L, "hMatProp")
    mat_type[1] = 4
    mat_prop[1][0], mat_prop[1][1], mat_prop[1][2] = rho0, c0, -1.0e12
    run = Simulation.in_dll(L, "hRun")
    run.dt = float(case.dt)
    loads = (Load * 10).in_dll(L, "hLoad")
    lo, hi = xy.min(axis=0) - 4 * h, xy.max(axis=0) + 4 * h
    loads[0].minX, loads[0].maxX, loads[0].minY, loads[0].maxY = lo[0], hi[0], lo[1], hi[1]
    loads[0].minZ, loads[0].maxZ, loads[0].gy = -1.0, 1.0, -9.81

    arr = {k: np.zeros(n, np.float32) for k in MODEL_FLOATS}
    arr["Mass"][:] = case.mass
    arr["Smooth"][:] = case.h
    arr["PosX"][:], arr["PosY"][:] = xy[:, 0], xy[:, 1]
    arr["VelX"][:], arr["VelY"][:] = case.v.reshape(n, 2)[:, 0], case.v.reshape(n, 2)[:, 1]
    arr["Density"][:] = case.rho
    arr["Pressure"][:] = case.p
    arr["Sound"][:] = c0
    material = np.where(fluid, 1, -1).astype(np.int32)
    hashes = np.zeros(n, np.int32)
    index = np.zeros(n, np.int32)
    nlist = np.zeros(n * MAXN, np.int32)

    grid = Grid()
    grid.oX, grid.oY, grid.oZ, grid.size = lo[0], lo[1], 0.0, 2.0 * h
    grid.nX = int((hi[0] - lo[0]) / grid.size) + 1
    grid.nY = int((hi[1] - lo[1]) / grid.size) + 1
    grid.nZ = 1
    pad = grid.nX * grid.nY + grid.nX + 1
    cells = grid.nX * grid.nY
    set_start = np.zeros(cells + 2 * pad, np.int32)
    set_stop = np.zeros(cells + 2 * pad, np.int32)
    start_p = C.cast(C.c_void_p(set_start.ctypes.data + 4 * pad), I)
    stop_p = C.cast(C.c_void_p(set_stop.ctypes.data + 4 * pad), I)

    model = Model()
    model.pn = n

    def bind():
        model.Material = ptr(material, I)
        for k in MODEL_FLOATS:
            setattr(model, k, ptr(arr[k], F))
        model.List, model.Hash, model.Index = ptr(nlist, I), ptr(hashes, I), ptr(index, I)
        model.SetStart, model.SetStop = start_p, stop_p

    sorted_keys = ["Mass", "Smooth", "PosX", "PosY", "PosZ", "VelX", "VelY", "VelZ", "Density",
                   "Energy", "Pressure", "Sound"]
    t_ref = t_stand = 0.0
    for s in range(args.steps):
        t0 = time.perf_counter()
        L.updateHashHost(n, grid, ptr(arr["PosX"], F), ptr(arr["PosY"], F), ptr(arr["PosZ"], F),
                         ptr(hashes, I))
        t1 = time.perf_counter()
        perm = np.argsort(hashes, kind="stable")
        hashes[:] = hashes[perm]
        material[:] = material[perm]
        for k in sorted_keys:
            arr[k][:] = arr[k][perm]
        set_start[:] = 0
        set_stop[:] = 0
        bind()
        t2 = time.perf_counter()
        L.updateSetsHost(n, start_p, stop_p, ptr(hashes, I))
        L.updateListHost(n, ptr(nlist, I), start_p, stop_p, grid, ptr(arr["Smooth"], F),
                         ptr(arr["PosX"], F), ptr(arr["PosY"], F), ptr(arr["PosZ"], F))
        t3 = time.perf_counter()
        for a, b in (("PosX0", "PosX"), ("PosY0", "PosY"), ("PosZ0", "PosZ"), ("VelX0", "VelX"),
                     ("VelY0", "VelY"), ("VelZ0", "VelZ"), ("Density0", "Density"),
                     ("Energy0", "Energy")):
            arr[a][:] = arr[b]
        t4 = time.perf_counter()
        for alpha in (1.0, 0.25, 2.0 / 3.0):
            L.RKstepHost(C.byref(model), alpha)
        t5 = time.perf_counter()
        t_ref += (t1 - t0) + (t3 - t2) + (t5 - t4)
        t_stand += (t2 - t1) + (t4 - t3)
        print(f"step {s}: acpu.c {t1 - t0 + t3 - t2 + t5 - t4:.2f} s, stand-in "
              f"{t2 - t1 + t4 - t3:.2f} s", file=sys.stderr, flush=True)
    if not np.isfinite(arr["PosX"]).all():
        raise RuntimeError("acpu.c run produced non-finite positions")

    st = O.State(case)
    O.integrate_gather(st, 1, 1, case.dt, 1)
    t0 = time.perf_counter()
    O.integrate_gather(st, 2, args.oracle_steps, case.dt, 1)
    t_or = (time.perf_counter() - t0) / args.oracle_steps

    per = (t_ref + t_stand) / args.steps
    out = {
        "workload": f"dam break 2D, {case.n_fluid} fluid + {case.n_wall} wall particles, "
                    f"dx = {args.dx}",
        "host": f"{platform.machine()}, {os.cpu_count()} hardware threads",
        "threads": 1,
        "acpu_steps": args.steps,
        "acpu_s_per_step": t_ref / args.steps,
        "stand_in_s_per_step": t_stand / args.steps,
        "acpu_particle_steps_per_s": n / per,
        "acpu_force_evaluations_per_step": 3,
        "oracle_steps": args.oracle_steps,
        "oracle_s_per_step": t_or,
        "oracle_particle_steps_per_s": n / t_or,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
