"""Drives the reference's compiled C host path (ArmandoThrust/acpu.c, built by
`make -C oracle ref` into oracle/_ref/libacpu.so) on arrays this module owns.

Test infrastructure, like the rest of oracle/: it generates golden vectors
of the GPU-C scheme and times acpu.c; the product never imports it.

One reference time step is `RKintegrateHost`'s loop body (acpu.c:2360-2373):
  * neighbour list: `updateHashHost` (acpu.c:2085), a sort by cell hash,
    `updateSetsHost` (acpu.c:2135), `updateListHost` (acpu.c:2201);
  * a backup of the step's initial state;
  * `RKstepHost` (acpu.c:2293) three times, alpha = 1, 1/4, 2/3.
acpu.c's own `neighbourListHost` (acpu.c:2245) sorts through a stack array of
MAXP = 441 pairs and `backupDataHost` (acpu.c:1173) copies MAXP entries, so
this driver replaces those two pieces: the sort is a stable numpy argsort of
the hashes plus the gathers, the backup numpy copies. Everything else is
acpu.c's compiled code.

The cell table is padded by one z-plane and one row on each side:
`updateListHost` visits z offsets -1..1 even for 2D grids (nZ = 1), and
those cells read as empty, the padding keeping every read in bounds.
Neighbour lists hold MAXN = 21 entries (acpu.c:7), the particle itself
included; `in_range_max` counts what a row would need, so callers can check
that no list was cut.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAXN = 21
F = C.POINTER(C.c_float)
I = C.POINTER(C.c_int)


class Grid(C.Structure):  # acpu.c:17-21
    _fields_ = [("oX", C.c_float), ("oY", C.c_float), ("oZ", C.c_float), ("size", C.c_float),
                ("nX", C.c_int), ("nY", C.c_int), ("nZ", C.c_int)]


class Simulation(C.Structure):  # acpu.c:23-32
    _fields_ = [(k, C.c_float) for k in ("minX", "maxX", "minY", "maxY", "minZ", "maxZ", "dt")] + \
               [("tsn", C.c_int), ("ssi", C.c_int), ("nsi", C.c_int)]


class Load(C.Structure):  # acpu.c:33-41
    _fields_ = [(k, C.c_float) for k in ("minX", "maxX", "minY", "maxY", "minZ", "maxZ",
                                         "gx", "gy", "gz", "w")]


class Fix(C.Structure):  # acpu.c:43-48
    _fields_ = [(k, C.c_float) for k in ("minX", "maxX", "minY", "maxY", "minZ", "maxZ",
                                         "velX", "velY", "velZ")]


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


def _ptr(a, t):
    return a.ctypes.data_as(t)


class AcpuRun:
    """A 2D particle system stepped by acpu.c. x, v: [n, 2]; materials:
    {index: (type, [props])} set into hMatType / hMatProp; gravity a load zone
    over the whole box (acpu.c:1047-1076 applies it to Material > 0), then
    `loads` [(lo2, hi2, (gx, gy), w)] in hLoad[1:] and `fixes` [(lo2, hi2,
    (vx, vy))] in hFix, z bounds -1, 1 (the 2D system lies at z = 0)."""

    SORTED = ["Mass", "Smooth", "PosX", "PosY", "PosZ", "VelX", "VelY", "VelZ", "Density",
              "Energy", "Pressure", "Sound"]

    def __init__(self, x, v, mass, rho, p, u, h, material, sound, materials, dt, gravity=(0.0, 0.0),
                 loads=(), fixes=()):
        self.L = L = load_acpu()
        n = len(mass)
        self.n = n
        mat_type = (C.c_int * 10).in_dll(L, "hMatType")
        mat_prop = ((C.c_float * 10) * 10).in_dll(L, "hMatProp")
        for k in range(10):
            mat_type[k] = 0
            for q in range(10):
                mat_prop[k][q] = 0.0
        for k, (t, props) in materials.items():
            mat_type[k] = t
            for q, val in enumerate(props):
                mat_prop[k][q] = val
        Simulation.in_dll(L, "hRun").dt = float(dt)
        tab_l = (Load * 10).in_dll(L, "hLoad")
        for k in range(10):
            C.memset(C.byref(tab_l[k]), 0, C.sizeof(Load))
        h0 = float(np.max(h))
        lo, hi = x.min(axis=0) - 8 * h0, x.max(axis=0) + 8 * h0
        tab_l[0].minX, tab_l[0].maxX, tab_l[0].minY, tab_l[0].maxY = lo[0], hi[0], lo[1], hi[1]
        tab_l[0].minZ, tab_l[0].maxZ = -1.0, 1.0
        tab_l[0].gx, tab_l[0].gy = gravity[0], gravity[1]
        assert len(loads) <= 9 and len(fixes) <= 10
        for k, (zlo, zhi, g, w) in enumerate(loads, start=1):
            z = tab_l[k]
            z.minX, z.maxX, z.minY, z.maxY, z.minZ, z.maxZ = zlo[0], zhi[0], zlo[1], zhi[1], -1.0, 1.0
            z.gx, z.gy, z.w = g[0], g[1], w
        tab = (Fix * 10).in_dll(L, "hFix")
        for k in range(10):
            C.memset(C.byref(tab[k]), 0, C.sizeof(Fix))
        for k, (zlo, zhi, vel) in enumerate(fixes):
            z = tab[k]
            z.minX, z.maxX, z.minY, z.maxY, z.minZ, z.maxZ = zlo[0], zhi[0], zlo[1], zhi[1], -1.0, 1.0
            z.velX, z.velY = vel[0], vel[1]
        self.a = {k: np.zeros(n, np.float32) for k in MODEL_FLOATS}
        a = self.a
        a["Mass"][:], a["Smooth"][:] = mass, h
        a["PosX"][:], a["PosY"][:] = x[:, 0], x[:, 1]
        a["VelX"][:], a["VelY"][:] = v[:, 0], v[:, 1]
        a["Density"][:], a["Pressure"][:], a["Energy"][:], a["Sound"][:] = rho, p, u, sound
        self.material = np.asarray(material, np.int32).copy()
        self.ids = np.arange(n)
        self.hashes = np.zeros(n, np.int32)
        self.index = np.zeros(n, np.int32)
        self.nlist = np.zeros(n * MAXN, np.int32)
        g = self.grid = Grid()
        g.oX, g.oY, g.oZ, g.size = lo[0], lo[1], 0.0, 2.0 * h0
        g.nX = int((hi[0] - lo[0]) / g.size) + 1
        g.nY = int((hi[1] - lo[1]) / g.size) + 1
        g.nZ = 1
        self.pad = g.nX * g.nY + g.nX + 1
        cells = g.nX * g.nY
        self.set_start = np.zeros(cells + 2 * self.pad, np.int32)
        self.set_stop = np.zeros(cells + 2 * self.pad, np.int32)
        self.start_p = C.cast(C.c_void_p(self.set_start.ctypes.data + 4 * self.pad), I)
        self.stop_p = C.cast(C.c_void_p(self.set_stop.ctypes.data + 4 * self.pad), I)
        self.model = Model()
        self.model.pn = n
        self.seconds_ref = 0.0
        self.seconds_stand_in = 0.0

    def _bind(self):
        m, a = self.model, self.a
        m.Material = _ptr(self.material, I)
        for k in MODEL_FLOATS:
            setattr(m, k, _ptr(a[k], F))
        m.List, m.Hash, m.Index = _ptr(self.nlist, I), _ptr(self.hashes, I), _ptr(self.index, I)
        m.SetStart, m.SetStop = self.start_p, self.stop_p

    def step(self):
        import time

        L, a, n = self.L, self.a, self.n
        t0 = time.perf_counter()
        L.updateHashHost(n, self.grid, _ptr(a["PosX"], F), _ptr(a["PosY"], F), _ptr(a["PosZ"], F),
                         _ptr(self.hashes, I))
        t1 = time.perf_counter()
        perm = np.argsort(self.hashes, kind="stable")
        self.hashes[:] = self.hashes[perm]
        self.material[:] = self.material[perm]
        self.ids = self.ids[perm]
        for k in self.SORTED:
            a[k][:] = a[k][perm]
        self.set_start[:] = 0
        self.set_stop[:] = 0
        self._bind()
        t2 = time.perf_counter()
        L.updateSetsHost(n, self.start_p, self.stop_p, _ptr(self.hashes, I))
        L.updateListHost(n, _ptr(self.nlist, I), self.start_p, self.stop_p, self.grid,
                         _ptr(a["Smooth"], F), _ptr(a["PosX"], F), _ptr(a["PosY"], F),
                         _ptr(a["PosZ"], F))
        t3 = time.perf_counter()
        for dst, src in (("PosX0", "PosX"), ("PosY0", "PosY"), ("PosZ0", "PosZ"), ("VelX0", "VelX"),
                         ("VelY0", "VelY"), ("VelZ0", "VelZ"), ("Density0", "Density"),
                         ("Energy0", "Energy")):
            a[dst][:] = a[src]
        t4 = time.perf_counter()
        for alpha in (1.0, 0.25, 2.0 / 3.0):
            L.RKstepHost(C.byref(self.model), alpha)
        t5 = time.perf_counter()
        self.seconds_ref += (t1 - t0) + (t3 - t2) + (t5 - t4)
        self.seconds_stand_in += (t2 - t1) + (t4 - t3)

    def in_range_max(self):
        """Largest number of particles within updateListHost's reach of one
        particle (itself included) at the current positions, by brute force
        (small systems): the lists are exact while this is <= MAXN."""
        a = self.a
        x, y, h = a["PosX"], a["PosY"], a["Smooth"]
        dx = x[:, None] - x[None, :]
        dy = y[:, None] - y[None, :]
        dr = np.sqrt(dx * dx + dy * dy)
        return int((dr < (2.0 * h)[:, None]).sum(1).max())

    def state(self):
        """Arrays in the caller's original particle order."""
        inv = np.empty(self.n, np.int64)
        inv[self.ids] = np.arange(self.n)
        a = self.a
        return {
            "x": np.stack([a["PosX"], a["PosY"]], 1)[inv],
            "v": np.stack([a["VelX"], a["VelY"]], 1)[inv],
            "rho": a["Density"][inv], "p": a["Pressure"][inv], "u": a["Energy"][inv],
            "c": a["Sound"][inv], "dv": np.stack([a["VelDotX"], a["VelDotY"]], 1)[inv],
            "drho": a["DensityDot"][inv], "du": a["EnergyDot"][inv],
        }
