#!/usr/bin/env python
"""Golden vectors of the GPU-C scheme from the reference's own compiled C host
path (ArmandoThrust/acpu.c, built from the reference sources by
`make -C oracle ref`), driven through oracle/acpu_driver.py.

  python tests/golden/make_gpuc_golden.py     (needs the reference tree)

Writes tests/golden/acpu_rk3.npz:
  * water_*: a small tank in the published dam-break layout (513 particles,
    cases.gpuc_dam_break with fluid (20, 10), tank (54, 16)), water and walls
    Tait (rho0 1000, c0 50), seeded fluid velocities, gravity; the state after
    1 and after 5 TVD-RK3 steps;
  * multi_*: the same tank with the water in three bands of different
    materials (Tait, Mie-Gruneisen shock, Mie-Gruneisen polynomial) and the
    walls of a boundary-type material, u = 100 J/kg;
  * eos_*: known answers of acpu.c's EOS functions (pressure, sound, density
    clamp) for every type on a grid of (rho, u).
and tests/golden/acpu_zones.npz:
  * zones_*: the water tank with two overlapping load zones (acceleration and
    heating, acpu.c:1047-1076) and a fix zone over the left of the water and
    part of the left wall (prescribed velocity, acpu.c:916-926), the zones as
    zones_load (rows lo_x, lo_y, hi_x, hi_y, gx, gy, w) and zones_fix (rows
    lo_x, lo_y, hi_x, hi_y, vx, vy); the state after 1 and after 5 steps.
No neighbour list needs more than the reference's MAXN = 21 entries (checked).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle")]

from acpu_driver import MAXN, AcpuRun, load_acpu  # noqa: E402
from armando_gb300 import cases  # noqa: E402

OUT = os.path.join(HERE, "acpu_rk3.npz")
OUT_ZONES = os.path.join(HERE, "acpu_zones.npz")
INF = float("inf")
LOADS = [((0.10, -INF), (0.24, INF), (3.0, 1.5), 250.0),
         ((0.20, -INF), (0.50, 0.08), (-1.0, 0.0), 40.0)]
FIXES = [((-0.10, -0.03), (0.06, 0.12), (0.5, 0.0))]

TAIT = (4, [1000.0, 50.0, -1.0e12])
SHOCK = (3, [1000.0, 50.0, 0.5, 1.3])
POLY = (2, [1000.0, 2.5e6, 1.0e6, 2.0e5, 0.2, 0.1, 2.5e6, 5.0e5])
WALL = (0, [1000.0, 50.0])
GAS = (1, [1.0, 1.4, 1.0e3])


def sound(t, props, rho, u):
    if t in (0, 3, 4):
        return np.full_like(rho, props[1])
    if t == 2:
        return np.sqrt(np.float32(props[1]) / rho)
    return np.sqrt(np.float32(props[1] * (props[1] - 1.0)) * u)


def tank(seed):
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    rng = np.random.default_rng(seed)
    v = c.v.reshape(-1, 2)
    fl = c.itype > 0
    v[fl] = rng.normal(0.0, 0.05, size=(fl.sum(), 2)).astype(np.float32)
    return c


def run(c, material, materials, u, steps_list, loads=(), fixes=()):
    x = c.x.reshape(-1, 2).astype(np.float32)
    v = c.v.reshape(-1, 2).astype(np.float32)
    snd = np.zeros(c.n, np.float32)
    for k, (t, props) in materials.items():
        sel = np.abs(material) == k
        snd[sel] = sound(t, props, c.rho[sel], u[sel])
    r = AcpuRun(x, v, c.mass, c.rho, c.p, u, c.h, material, snd, materials, c.dt,
                gravity=(0.0, -9.81), loads=loads, fixes=fixes)
    out = {}
    done = 0
    for s in steps_list:
        for _ in range(s - done):
            assert r.in_range_max() <= MAXN  # every list complete
            r.step()
        done = s
        out[s] = r.state()
    return out


def eos_kat():
    L = load_acpu()
    fp = C.POINTER(C.c_float)
    rho = np.linspace(850.0, 1150.0, 13, dtype=np.float32)
    u = np.array([0.0, 10.0, 1000.0], np.float32)
    R, U = np.meshgrid(rho, u, indexing="ij")
    R, U = R.ravel(), U.ravel()
    res = {"rho": R, "u": U}
    for name, (t, props) in (("tait", TAIT), ("shock", SHOCK), ("poly", POLY), ("gas", GAS)):
        pr = (C.c_float * 10)(*(list(props) + [0.0] * (10 - len(props))))
        fam = {4: "Tait", 3: "Shock", 2: "Poly", 1: "Gas"}[t]
        fp_ = getattr(L, "pressure" + fam)
        fs_ = getattr(L, "sound" + fam)
        for f in (fp_, fs_):
            f.argtypes = [fp, C.c_float, C.c_float]
            f.restype = C.c_float
        dens = R.copy()
        if t != 1:
            fd = getattr(L, "density" + fam)
            fd.argtypes = [fp, C.c_float]
            fd.restype = C.c_float
            dens = np.array([fd(pr, float(a)) for a in R], np.float32)
        res[name + "_rho"] = dens
        res[name + "_p"] = np.array([fp_(pr, float(a), float(b)) for a, b in zip(dens, U)], np.float32)
        res[name + "_c"] = np.array([fs_(pr, float(a), float(b)) for a, b in zip(dens, U)], np.float32)
    return res


def main():
    data = {}
    c = tank(11)
    u = np.zeros(c.n, np.float32)
    mats = {1: TAIT}
    out = run(c, c.itype.copy(), mats, u, [1, 5])
    data.update({"water_x0": c.x, "water_v0": c.v, "water_m": c.mass, "water_rho0": c.rho,
                 "water_h": c.h, "water_itype": c.itype, "water_dt": np.float64(c.dt)})
    for s, st in out.items():
        for k, val in st.items():
            data[f"water_{k}_{s}"] = val
    c = tank(12)
    x = c.x.reshape(-1, 2)
    mat = c.itype.copy()
    fl = mat > 0
    mat[fl & (x[:, 0] >= 0.14)] = 2
    mat[fl & (x[:, 0] >= 0.28)] = 4
    mat[~fl] = -3
    u = np.where(fl, 100.0, 0.0).astype(np.float32)
    mats = {1: TAIT, 2: SHOCK, 3: WALL, 4: POLY}
    out = run(c, mat, mats, u, [1, 5])
    data.update({"multi_x0": c.x, "multi_v0": c.v, "multi_m": c.mass, "multi_rho0": c.rho,
                 "multi_h": c.h, "multi_itype": mat, "multi_u0": u, "multi_dt": np.float64(c.dt)})
    for s, st in out.items():
        for k, val in st.items():
            data[f"multi_{k}_{s}"] = val
    for k, val in eos_kat().items():
        data["eos_" + k] = val
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, len(data), "arrays")
    zones = {}
    c = tank(13)
    u = np.zeros(c.n, np.float32)
    out = run(c, c.itype.copy(), {1: TAIT}, u, [1, 5], LOADS, FIXES)
    zones.update({"zones_x0": c.x, "zones_v0": c.v, "zones_m": c.mass, "zones_rho0": c.rho,
                  "zones_h": c.h, "zones_itype": c.itype, "zones_dt": np.float64(c.dt),
                  "zones_load": np.array([list(lo) + list(hi) + list(g) + [w] for lo, hi, g, w in LOADS],
                                         np.float32),
                  "zones_fix": np.array([list(lo) + list(hi) + list(v) for lo, hi, v in FIXES],
                                        np.float32)})
    for s, st in out.items():
        for k, val in st.items():
            zones[f"zones_{k}_{s}"] = val
    np.savez_compressed(OUT_ZONES, **zones)
    print("wrote", OUT_ZONES, len(zones), "arrays")


if __name__ == "__main__":
    main()
