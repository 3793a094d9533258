"""The oracle's GPU-C pair rates against the reference's own known-answer test.

ArmandoList/armando2Dlist.cu:2451-2548 (check()) evaluates the reference's GPU
pair kernel (kerInteraction, armando2Dlist.cu:611-686) once on the lattice of
initFree (armando2Dlist.cu:1834-1880) with manufactured p and v, and wrote the
rates to ArmandoList/old.txt (tests/golden/kat_old.npz, made by
tests/golden/make_kat_fixture.py). That kernel's physics is the GPU-C host
path's pair physics (acpu.c:346-437: continuity, pressure -(p_i + p_j) /
(rho_i rho_j), the mass and momentum shock corrections) on one material, no
gravity, which the oracle restates as scheme 1. The rows are in the kernel's
cell order: a stable sort of the lattice by the FP32 cell hash of kerHash
(armando2Dlist.cu:1003-1025). Rows within one cell of the square's edges hold
the analytic rates instead (armando2Dlist.cu:2492-2502), and are checked
against those. The reference computed in FP32 (dv_y/dt is a cancelling sum of
pressure terms of ~1000 Pa); the gate per field is three times the spread
between an IEEE-FP32 restatement of kerInteraction, in its own neighbour-list
order (kerList, armando2Dlist.cu:1071-1110), and the FP64 oracle, plus 1e-6,
of the field's maximum over the interior rows.
"""
import os

import numpy as np

from armando_gb300 import Params

HERE = os.path.dirname(os.path.abspath(__file__))


def kat_case():
    """initFree's lattice in kerInteraction's order, with check()'s fields."""
    dr = 0.01
    jj, ii = np.meshgrid(np.arange(100), np.arange(100), indexing="ij")  # pi = j * 100 + i
    x = (ii.ravel() * dr + 0.0 * dr).astype(np.float32)
    y = (jj.ravel() * dr + 0.0 * dr).astype(np.float32)
    h = np.float32(1.2 * dr)                       # hSmooth (float)
    size = np.float32(2.0 * np.float64(h))         # hGrid.size = 2.0 * hSmooth
    ox = oy = np.float32(-0.5)
    nx = int(np.float32(np.float32(1.5) - np.float32(-0.5)) / size) + 1
    # kerHash divides by the cell size; the GPUs of the time (compute
    # capability 1.x) compiled FP32 division as a product with the reciprocal.
    # That order is the one every analytic edge row of old.txt matches (checked
    # below); a rounded quotient puts 60 lattice lines on cell edges elsewhere.
    r = np.float32(1.0) / size
    ix = np.trunc((x - ox) * r).astype(np.int64)
    iy = np.trunc((y - oy) * r).astype(np.int64)
    order = np.argsort(ix + iy * nx, kind="stable")  # cudppSort: stable radix sort
    x, y = x[order], y[order]
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    yy = (y * y).astype(np.float32)                # hPosY * hPosY in float
    p = (1000.0 * (np.sin(10 * np.pi * x64) + yy.astype(np.float64))).astype(np.float32)
    vx = np.sin(10 * np.pi * x64).astype(np.float32)
    vy = yy
    n = x.size
    return {
        "x": np.stack([x, y], 1).ravel(), "v": np.stack([vx, vy], 1).ravel(),
        "m": np.full(n, np.float32(1000.0 * dr * dr)), "rho": np.full(n, np.float32(1000.0)),
        "p": p, "u": np.zeros(n, np.float32), "h": np.full(n, h), "itype": np.ones(n, np.int32),
        "size": size, "key": (ix + iy * nx)[order], "nx": nx,
    }


def kat_params():
    P = Params.default()
    P.dim = 2
    P.scheme = 1
    P.rho0 = 1000.0
    P.c0 = 50.0
    P.gravity[:] = [0.0, 0.0, 0.0]
    return P


def analytic(x, y):
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    return np.stack([-1000.0 * (10 * np.pi * np.cos(10 * np.pi * x64) + 2.0 * y64),
                     -10 * np.pi * np.cos(10 * np.pi * x64), -2.0 * y64], 1)


def fp32_restatement(k):
    """kerInteraction in IEEE FP32: kerList's neighbour order (the 3 x 3 cells
    row by row, each in cell order, |x_i - x_j| < 2h, at most MAXN = 21, padded
    with the particle itself), then the pair sums in that order."""
    f32 = np.float32
    x, y = k["x"][0::2], k["x"][1::2]
    vx, vy = k["v"][0::2], k["v"][1::2]
    p, rho, m, h = k["p"], k["rho"], k["m"][0], k["h"][0]
    c0 = f32(50.0)
    n = x.size
    key = k["key"]
    cells = {}
    for q in range(n):
        cells.setdefault(int(key[q]), []).append(q)
    lst = np.empty((n, 21), np.int64)
    for q in range(n):
        row = []
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                for j in cells.get(int(key[q]) + di + dj * k["nx"], []):
                    dx, dy = f32(x[q] - x[j]), f32(y[q] - y[j])
                    if np.sqrt(f32(f32(dx * dx) + f32(dy * dy))) < f32(2) * h and len(row) < 21:
                        row.append(j)
        lst[q] = row + [q] * (21 - len(row))
    alpha = f32(7.0 / (4.0 * np.pi)) / (h * h)
    D, AX, AY = (np.zeros(n, f32) for _ in range(3))
    for t in range(21):
        j = lst[:, t]
        dx, dy = x - x[j], y - y[j]
        dr = np.sqrt(dx * dx + dy * dy)
        dr = np.where(dr < f32(0.1) * h, f32(100) * h, dr).astype(f32)
        q = dr / h
        dwdr = np.where(q < 2, f32(5 / 8) * q * (q - f32(2)) ** 3 * alpha / h, f32(0)).astype(f32)
        dvr = dx * (vx - vx[j]) + dy * (vy - vy[j])
        D = D + m * dvr * dwdr / dr
        fp = -(p + p[j]) / (rho * rho[j])
        AX = AX + m * fp * dwdr * dx / dr
        AY = AY + m * fp * dwdr * dy / dr
        D = D + m * ((rho - rho[j]) * (f32(2) * c0 / (rho + rho[j]))) * dwdr
        fv = np.where(dvr < 0, dvr, f32(0)).astype(f32)
        fv = fv * h / (dr * dr + f32(0.01) * h * h) * (f32(2) * c0 / (rho + rho[j])) * f32(0.03)
        AX = AX + m * fv * dwdr * dx / dr
        AY = AY + m * fv * dwdr * dy / dr
    return np.stack([D, AX, AY], 1).astype(np.float64)


def test_oracle_rates_equal_reference_kernel_output(O):
    k = kat_case()
    old = np.load(os.path.join(HERE, "golden", "kat_old.npz"))["rates"].astype(np.float64)
    drho, dv, _ = O.gpuc_rates(kat_params(), k["x"], k["v"], k["m"], k["rho"], k["p"], k["u"],
                               k["h"], k["itype"])
    got = np.stack([drho, dv[0::2], dv[1::2]], 1)
    x, y = k["x"][0::2], k["x"][1::2]
    s = k["size"]
    edge = (x < s) | (y < s) | (x > np.float32(1.0) - s) | (y > np.float32(1.0) - s)
    assert np.count_nonzero(~edge) == 95 * 95
    inner = ~edge
    e32 = fp32_restatement(k)
    for c, name in enumerate(("drho/dt", "dvx/dt", "dvy/dt")):
        scale = np.abs(old[inner, c]).max()
        err = np.abs(got[inner, c] - old[inner, c]).max() / scale
        spread = np.abs(e32[inner, c] - got[inner, c]).max() / scale
        print(name, f"max |oracle - old.txt| / max = {err:.2e} (FP32 spread {spread:.2e})")
        assert err <= 3.0 * spread + 1e-6, (name, err, spread)
    # the edge rows are the analytic rates check() substituted (this pins the order)
    ref = analytic(x, y)
    assert np.allclose(old[edge], ref[edge].astype(np.float32), rtol=1e-6, atol=1e-5)
