"""Generates tests/golden/acpu_pins.npz from the reference's own C host path.

Runs only where the reference sources are mounted: builds
oracle/_ref/libacpu.so from ArmandoThrust/acpu.c (oracle/Makefile, target
`ref`) and records, on a seeded jittered 2D lattice, the outputs of
  kernelWendland / kernelDerivWendland      acpu.c:146-201
  pressureTait                              acpu.c:663-686
  updateHashHost                            acpu.c:2085-2105
  updateSetsHost + updateListHost           acpu.c:2135-2243 (MAXN = 21)
  balanceMassMomentumHost (v = 0, one material: only the pressure action
                           -(P_i + P_j)/(rho_i rho_j) dW/dr (x_i - x_j)/r acts;
                           two materials: plus the boundary repulsion of
                           different-material pairs, acpu.c:424-429;
                           v != 0 at uniform density: plus the momentum
                           shock correction, and the continuity rate)
                                            acpu.c:346-437
The cell tables are padded with empty guard cells because updateListHost
visits cell ids ic +- nX*nY without bounds checks in 2D.

Usage: python tests/golden/make_golden.py [REF_DIR]
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle as O  # noqa: E402

MAXN = 21


class Grid(C.Structure):
    _fields_ = [("oX", C.c_float), ("oY", C.c_float), ("oZ", C.c_float), ("size", C.c_float),
                ("nX", C.c_int), ("nY", C.c_int), ("nZ", C.c_int)]


def fp(a, off=0):
    return C.c_void_p(a.ctypes.data + off * a.itemsize)


def main(ref_dir=os.environ.get("ARMANDO_REF_DIR", "/root/reference")):
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF_DIR={ref_dir}"],
                   check=True)
    L = C.CDLL(os.path.join(REPO, "oracle", "_ref", "libacpu.so"))
    L.kernelWendland.argtypes = [C.c_float, C.c_float]
    L.kernelWendland.restype = C.c_float
    L.kernelDerivWendland.argtypes = [C.c_float, C.c_float]
    L.kernelDerivWendland.restype = C.c_float
    L.pressureTait.argtypes = [C.c_void_p, C.c_float, C.c_float]
    L.pressureTait.restype = C.c_float
    L.updateHashHost.argtypes = [C.c_int, Grid, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.updateSetsHost.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.updateListHost.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, Grid, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_void_p]
    L.balanceMassMomentumHost.argtypes = [C.c_int] + [C.c_void_p] * 17

    out = {}
    # 1. Wendland kernel (2D) over q in [0, 2.2) for two h.
    r = np.linspace(0.0, 2.2, 89)
    wk, dwk, rr, hh = [], [], [], []
    for h in (1.3e-3, 0.25):
        for q in r:
            rv = np.float32(q * h)
            rr.append(rv)
            hh.append(np.float32(h))
            wk.append(L.kernelWendland(float(rv), float(np.float32(h))))
            dwk.append(L.kernelDerivWendland(float(rv), float(np.float32(h))))
    out["wendland_r"] = np.array(rr, np.float32)
    out["wendland_h"] = np.array(hh, np.float32)
    out["wendland_w"] = np.array(wk, np.float32)
    out["wendland_dwdr"] = np.array(dwk, np.float32)

    # 2. Tait pressure.
    props = np.array([1000.0, 62.64184, 0.0], np.float32)
    rho = np.linspace(990.0, 1012.0, 45).astype(np.float32)
    out["tait_props"] = props
    out["tait_rho"] = rho
    out["tait_p"] = np.array([L.pressureTait(fp(props), float(x), 0.0) for x in rho], np.float32)

    # 3-5. Jittered 2D lattice, uniform h = 1.3 dx.
    rng = np.random.default_rng(7)
    nx, ny, dx = 24, 16, 1.0e-3
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    x = np.stack([(i.ravel() + 0.5) * dx, (j.ravel() + 0.5) * dx], 1)
    x += rng.uniform(-0.01, 0.01, x.shape) * dx
    x = x.astype(np.float32)
    n = x.shape[0]
    h = np.full(n, 1.3 * dx, np.float32)
    _, _, _, g = O.link_list(x.ravel(), h, 2, fp32=True)
    grid = Grid(float(g["o"][0]), float(g["o"][1]), 0.0, float(g["size"][0]),
                int(g["n"][0]), int(g["n"][1]), 1)
    px = np.ascontiguousarray(x[:, 0])
    py = np.ascontiguousarray(x[:, 1])
    pz = np.zeros(n, np.float32)
    hsh = np.zeros(n, np.int32)
    L.updateHashHost(n, grid, fp(px), fp(py), fp(pz), fp(hsh))
    out["lattice_x"] = x.ravel()
    out["lattice_h"] = h
    out["lattice_grid"] = np.array([g["o"][0], g["o"][1], g["size"][0], g["n"][0], g["n"][1]],
                                   np.float64)
    out["lattice_hash"] = hsh.copy()

    order = np.argsort(hsh, kind="stable")
    sx, sy, sz, sh = px[order].copy(), py[order].copy(), pz[order].copy(), hsh[order].copy()
    smooth = h[order].copy()
    ncell = grid.nX * grid.nY
    pad = grid.nX * grid.nY + grid.nX + 1
    set_start = np.zeros(ncell + 2 * pad, np.int32)
    set_stop = np.zeros(ncell + 2 * pad, np.int32)
    L.updateSetsHost(n, fp(set_start, pad), fp(set_stop, pad), fp(sh))
    lst = np.zeros(n * MAXN, np.int32)
    L.updateListHost(n, fp(lst), fp(set_start, pad), fp(set_stop, pad), grid, fp(smooth), fp(sx),
                     fp(sy), fp(sz))
    # Neighbour lists in original particle ids (self removed).
    lists = lst.reshape(n, MAXN)
    nb_offs = np.zeros(n + 1, np.int64)
    rows = [None] * n
    for s in range(n):
        ids = sorted(set(int(order[k]) for k in lists[s]) - {int(order[s])})
        rows[int(order[s])] = ids
    for i in range(n):
        nb_offs[i + 1] = nb_offs[i] + len(rows[i])
    out["list_offs"] = nb_offs
    out["list_nbr"] = np.array([k for r_ in rows for k in r_], np.int32)
    out["list_count_with_self"] = np.array([len(set(lists[s])) for s in range(n)], np.int32)

    # Pressure action with v = 0 and one material.
    mass = np.full(n, 1000.0 * dx * dx, np.float32)
    dens = (1000.0 + rng.uniform(-2.0, 2.0, n)).astype(np.float32)
    pres = (5000.0 + 3000.0 * np.sin(40.0 * x[:, 0]) + rng.uniform(-50, 50, n)).astype(np.float32)
    snd = np.full(n, 20.0, np.float32)
    mat = np.ones(n, np.int32)
    z = np.zeros(n, np.float32)
    ddot, vdx, vdy, vdz = (np.zeros(n, np.float32) for _ in range(4))
    # Keep every sorted copy referenced until the call returns (fp() holds no reference).
    msort, masssort = mat[order].copy(), mass[order].copy()
    dsort, psort, csort = dens[order].copy(), pres[order].copy(), snd[order].copy()
    args = [fp(lst), fp(msort), fp(masssort), fp(smooth), fp(sx), fp(sy), fp(sz), fp(z), fp(z),
            fp(z), fp(dsort), fp(psort), fp(csort), fp(ddot), fp(vdx), fp(vdy), fp(vdz)]
    L.balanceMassMomentumHost(n, *args)
    acc = np.zeros((n, 2), np.float32)
    acc[order, 0] = vdx
    acc[order, 1] = vdy
    out["force_mass"] = mass
    out["force_rho"] = dens
    out["force_p"] = pres
    out["force_acc"] = acc.ravel()
    # Uniform density: the pa_sph = 0 and pa_sph = 1 forms coincide.
    dsort[:] = 1000.0
    for a in (ddot, vdx, vdy, vdz):
        a[:] = 0.0
    L.balanceMassMomentumHost(n, *args)
    acc_u = np.zeros((n, 2), np.float32)
    acc_u[order, 0] = vdx
    acc_u[order, 1] = vdy
    out["force_acc_uniform_rho"] = acc_u.ravel()
    # Two materials: the lowest rows of the lattice are material 2.
    y_cut = np.quantile(x[:, 1], 0.25)
    mat2 = np.where(x[:, 1] < y_cut, 2, 1).astype(np.int32)
    msort[:] = mat2[order]
    dsort[:] = dens[order]
    for a in (ddot, vdx, vdy, vdz):
        a[:] = 0.0
    L.balanceMassMomentumHost(n, *args)
    acc_m = np.zeros((n, 2), np.float32)
    acc_m[order, 0] = vdx
    acc_m[order, 1] = vdy
    out["force_mat"] = mat2
    out["force_acc_two_materials"] = acc_m.ravel()
    # Moving particles, one material, uniform density: the continuity rate
    # drho/dt = sum_j m_j (x_i - x_j).(v_i - v_j) dW/dr / r (the mass shock
    # correction vanishes at uniform density) and, beside the pressure action,
    # the momentum shock correction of acpu.c:413-422, which is art_visc with
    # alpha = 0.03, beta = 0, eta = 0.1, c = c0 for uniform h.
    vel = rng.normal(0.0, 0.5, (n, 2)).astype(np.float32)
    vxs, vys = vel[order, 0].copy(), vel[order, 1].copy()
    msort[:] = 1
    dsort[:] = 1000.0
    for a in (ddot, vdx, vdy, vdz):
        a[:] = 0.0
    args_v = [fp(lst), fp(msort), fp(masssort), fp(smooth), fp(sx), fp(sy), fp(sz), fp(vxs),
              fp(vys), fp(z), fp(dsort), fp(psort), fp(csort), fp(ddot), fp(vdx), fp(vdy), fp(vdz)]
    L.balanceMassMomentumHost(n, *args_v)
    acc_v = np.zeros((n, 2), np.float32)
    acc_v[order, 0] = vdx
    acc_v[order, 1] = vdy
    drho_v = np.zeros(n, np.float32)
    drho_v[order] = ddot
    out["moving_v"] = vel.ravel()
    out["moving_acc_uniform_rho"] = acc_v.ravel()
    out["moving_drho_uniform_rho"] = drho_v
    path = os.path.join(HERE, "acpu_pins.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main(*sys.argv[1:])
