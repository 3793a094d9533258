"""The GPU-C scheme of the oracle (armando_params.scheme 1: TVD-RK3, continuity
density, the host path's pair physics) pinned on the reference's own compiled
C host path, ArmandoThrust/acpu.c (golden vectors of
tests/golden/make_gpuc_golden.py: the EOS functions, and 1 and 5 RK3 steps of
two small tanks in the published dam-break layout).

acpu.c computes in FP32 and the oracle in FP64. The integrated state (x, rho,
u) agrees to FP32 rounding (gate 1e-6 normwise relative). Pressure is a stiff
function of the FP32 density: one ulp of rho ~ 1000 (6.1e-5) is c0^2 ulp =
0.15 Pa of Tait pressure, about 1e-4 of the small tank's pressures, and the
velocity rates and velocities inherit it; their gates are 2e-4 (rates,
pressure) and 5e-5 (velocity), the same after one and after five steps.
"""
import os

import numpy as np
import pytest

from armando_gb300 import cases
from armando_gb300._abi import Material

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acpu_rk3.npz")
TOL = {"x": 1e-6, "rho": 1e-6, "u": 1e-6, "v": 5e-5, "p": 2e-4, "dv": 2e-4, "du": 2e-4}

MATS = {
    "tait": Material.make(4, [1000.0, 50.0, -1.0e12]),
    "shock": Material.make(3, [1000.0, 50.0, 0.5, 1.3]),
    "poly": Material.make(2, [1000.0, 2.5e6, 1.0e6, 2.0e5, 0.2, 0.1, 2.5e6, 5.0e5]),
    "gas": Material.make(1, [1.0, 1.4, 1.0e3]),
    "wall": Material.make(0, [1000.0, 50.0]),
}


@pytest.fixture(scope="module")
def G():
    return np.load(GOLD)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    s = np.abs(b).max()
    return np.abs(a - b).max() / s if s > 0 else np.abs(a).max()


@pytest.mark.parametrize("name", ["tait", "shock", "poly", "gas"])
def test_eos_matches_acpu(O, G, name):
    rho, u = G["eos_rho"], G["eos_u"]
    r, p, c = O.gpuc_eos(MATS[name], rho, u)
    np.testing.assert_array_equal(r.astype(np.float32), G[f"eos_{name}_rho"])
    assert rel(p, G[f"eos_{name}_p"]) <= 2e-6, name
    assert rel(c, G[f"eos_{name}_c"]) <= 1e-6, name


def run_oracle(O, G, pre, steps, table):
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    c.x, c.v, c.mass, c.rho = G[pre + "_x0"], G[pre + "_v0"], G[pre + "_m"], G[pre + "_rho0"]
    c.h, c.itype = G[pre + "_h"], G[pre + "_itype"]
    if pre + "_u0" in G:
        c.u = G[pre + "_u0"]
    st = O.State(c)
    dv, du = O.gpuc_step(st, steps, float(G[pre + "_dt"]), materials=table)
    return st, dv.reshape(-1, 2), du


@pytest.mark.parametrize("steps", [1, 5])
def test_water_tank_matches_acpu(O, G, steps):
    table = [MATS["tait"]] * 2
    st, dv, du = run_oracle(O, G, "water", steps, table)
    for f, got in (("x", st.x.reshape(-1, 2)), ("v", st.v.reshape(-1, 2)), ("rho", st.rho),
                   ("p", st.p), ("u", st.u), ("dv", dv), ("du", du)):
        # the water's u is pressure work from u = 0: it carries p's quantization
        tol = TOL["p"] if f == "u" else TOL[f]
        e = rel(got, G[f"water_{f}_{steps}"])
        assert e <= tol, (f, steps, e)


@pytest.mark.parametrize("steps", [1, 5])
def test_four_material_tank_matches_acpu(O, G, steps):
    """Tait, shock and polynomial water bands (repulsion between them) and
    boundary-type walls; u = 100 J/kg enters the shock and polynomial EOS."""
    table = [MATS["wall"], MATS["tait"], MATS["shock"], MATS["wall"], MATS["poly"]]
    st, dv, du = run_oracle(O, G, "multi", steps, table)
    for f, got in (("x", st.x.reshape(-1, 2)), ("v", st.v.reshape(-1, 2)), ("rho", st.rho),
                   ("p", st.p), ("u", st.u), ("dv", dv), ("du", du)):
        e = rel(got, G[f"multi_{f}_{steps}"])
        assert e <= TOL[f], (f, steps, e)


def test_device_variant_gates_pairs_by_material(O, G):
    """Scheme 2 (armando.cu:429-513): water next to boundary walls feels only
    the wall push, so its density rate differs from scheme 1 near the walls
    and not in the tank's interior."""
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    c.v = G["water_v0"].copy()
    c2 = c.copy()
    c2.params.scheme = 2
    a, b = O.State(c), O.State(c2)
    O.gpuc_step(a, 1, c.dt)
    O.gpuc_step(b, 1, c.dt)
    x = c.x.reshape(-1, 2)
    fl = c.itype > 0
    near = fl & (x[:, 1] < 2.4 * c.h[0])
    inner = fl & (x[:, 1] > 6 * c.h[0]) & (x[:, 0] > 6 * c.h[0]) & (x[:, 0] < 0.35)
    assert inner.sum() > 20 and near.sum() > 10
    assert not np.allclose(a.rho[near], b.rho[near], rtol=0, atol=1e-9)
    np.testing.assert_allclose(a.rho[inner], b.rho[inner], rtol=2e-6)


GOLD_ZONES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acpu_zones.npz")


def golden_zones(Z):
    """The load and fix zones of the golden run as C-ABI structs (2D: the z
    bounds do not enter)."""
    from armando_gb300._abi import FixZone, LoadZone

    loads = [LoadZone.make(r[0:2], r[2:4], (r[4], r[5], 0.0), r[6]) for r in Z["zones_load"]]
    fixes = [FixZone.make(r[0:2], r[2:4], (r[4], r[5], 0.0)) for r in Z["zones_fix"]]
    return loads, fixes


@pytest.mark.parametrize("steps", [1, 5])
def test_load_and_fix_zones_match_acpu(O, steps):
    """Two overlapping load zones (acceleration and heating) and a fix zone
    over the left of the water and part of the left wall, which then moves
    (acpu.c resets wall velocities before the fix zones)."""
    Z = np.load(GOLD_ZONES)
    loads, fixes = golden_zones(Z)
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    c.x, c.v, c.mass, c.rho = Z["zones_x0"], Z["zones_v0"], Z["zones_m"], Z["zones_rho0"]
    c.h, c.itype = Z["zones_h"], Z["zones_itype"]
    st = O.State(c)
    dv, du = O.gpuc_step(st, steps, float(Z["zones_dt"]), materials=[MATS["tait"]] * 2,
                         loads=loads, fixes=fixes)
    for f, got in (("x", st.x.reshape(-1, 2)), ("v", st.v.reshape(-1, 2)), ("rho", st.rho),
                   ("p", st.p), ("u", st.u), ("dv", dv.reshape(-1, 2)), ("du", du)):
        # u starts at 0: next to the fixed water its pressure work carries p's
        # quantization, as in the water tank
        tol = TOL["p"] if f == "u" else TOL[f]
        e = rel(got, Z[f"zones_{f}_{steps}"])
        assert e <= tol, (f, steps, e)
    moved = np.abs(st.x.reshape(-1, 2) - c.x.reshape(-1, 2)).max(1) > 1e-6
    assert (moved & (c.itype <= 0)).sum() > 10


def isolated(dim, scheme):
    """Three particles far beyond each other's reach (no pair terms), fluid,
    at rest, no gravity."""
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16), scheme=scheme)
    pts = np.array([[0.1, 0.2, 0.3], [1.1, 0.2, -0.4], [2.1, -0.9, 0.3]])[:, :dim]
    c.params.dim = c.dim = dim
    c.params.gravity[:] = (0.0, 0.0, 0.0)
    keep = np.arange(3)
    for f in ("mass", "rho", "p", "u", "h", "itype", "dudt"):
        setattr(c, f, getattr(c, f)[keep].copy())
    c.itype[:] = 1
    c.x = pts.ravel().astype(np.float32)
    c.v = np.zeros(3 * dim, np.float32)
    c.dvdt = np.zeros(3 * dim, np.float32)
    c.u = np.full(3, 5.0, np.float32)
    return c


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_zone_known_answers(O, dim, scheme):
    """Isolated particles, one RK3 step (exact for constant rates): inside a
    load zone v = dt a, x = x0 + dt^2 a / 2, u = u0 + dt w, overlapping zones
    adding; inside a fix zone v = vel after every stage, so x = x0 + (5/6) dt
    vel from rest; in 3D the z bounds decide (particle 2 lies below the
    load zones' z range); in 2D z does not enter."""
    from armando_gb300._abi import FixZone, LoadZone

    c = isolated(dim, scheme)
    dt = 1e-3
    a1, a2 = np.array([2.0, -1.0, 0.5]), np.array([0.25, 0.5, -4.0])
    loads = [LoadZone.make((0.0, 0.0, -0.1), (1.5, 0.5, 0.5), a1, 300.0),
             LoadZone.make((1.0, 0.0, -0.1), (1.5, 0.5, 0.5), a2, 20.0)]
    vel = np.array([0.7, -0.3, 0.2])
    fixes = [FixZone.make((2.0, -1.0, 0.0), (2.5, -0.5, 0.5), vel)]
    st = O.State(c)
    O.gpuc_step(st, 1, dt, loads=loads, fixes=fixes)
    x0 = c.x.reshape(3, dim).astype(np.float64)
    x, v = st.x.reshape(3, dim), st.v.reshape(3, dim)
    acc = [a1[:dim], (a1 + a2)[:dim]]
    w = [300.0, 320.0]
    if dim == 3:  # particle 2 (z = -0.4) below the z range of the load zones
        acc[1], w[1] = np.zeros(3), 0.0
    for k in range(2):
        np.testing.assert_allclose(v[k], dt * acc[k], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(x[k], x0[k] + 0.5 * dt * dt * acc[k], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(st.u[k], 5.0 + dt * w[k], rtol=1e-12)
    np.testing.assert_allclose(v[2], vel[:dim], rtol=1e-7)
    np.testing.assert_allclose(x[2], x0[2] + dt * 5.0 / 6.0 * vel[:dim], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(st.u[2], 5.0, rtol=1e-12)


def test_pressure_wave_is_symmetric(O):
    """The pressure-wave stand-in (a Gaussian energy deposit at the centre of
    a free square of mercury, polynomial EOS) stays symmetric under the
    square's reflections, and the deposit drives a compression outward."""
    c = cases.gpuc_pressure_wave(41, radius=0.02)
    st = O.State(c)
    O.gpuc_step(st, 10, c.dt, materials=[cases.mercury_poly()] * 2)
    p = st.p.reshape(41, 41)  # [i, j] with x = i dr, y = j dr
    scale = np.abs(p).max()
    assert np.abs(p - p[::-1, :]).max() <= 1e-9 * scale
    assert np.abs(p - p.T).max() <= 1e-9 * scale
    v = st.v.reshape(41, 41, 2)
    assert v[30, 20, 0] > 0 and v[10, 20, 0] < 0  # outward on both sides of the centre


def rk3_relaxation(v_target, tau, dt, steps, x0):
    """The TVD-RK3 step on x' = v, v' = (V - v) / tau from rest: for this
    linear system the step is y + dt f + dt^2/2 A f + dt^3/6 A^2 f, f = A y + b."""
    A = np.array([[0.0, 1.0], [0.0, -1.0 / tau]])
    out = []
    for x, V in zip(x0, v_target):
        y = np.array([x, 0.0])
        b = np.array([0.0, V / tau])
        for _ in range(steps):
            f = A @ y + b
            y = y + dt * f + dt * dt / 2 * (A @ f) + dt ** 3 / 6 * (A @ (A @ f))
        out.append(y)
    return np.array(out)  # [dim, (x, v)]


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_pump_zone_known_answer(O, dim, scheme):
    """A pump zone (a fix zone with tau > 0, Code/armando.cu:1046-1055):
    isolated particle 0 inside relaxes towards vel with dv/dt = (vel - v)/tau,
    which ten RK3 steps integrate exactly as the third-order Taylor step of
    the linear system; particles 1 and 2 lie outside and stay at rest."""
    from armando_gb300._abi import FixZone

    c = isolated(dim, scheme)
    dt, steps = 1e-3, 10
    tau = float(np.float32(5e-3))  # the zone record holds FP32 values
    vel = np.array([0.7, -0.3, 0.2], np.float32).astype(np.float64)
    pumps = [FixZone.make((0.0, 0.0, 0.0), (0.5, 0.5, 0.5), vel, tau)]
    st = O.State(c)
    O.gpuc_step(st, steps, dt, fixes=pumps)
    x0 = c.x.reshape(3, dim).astype(np.float64)
    ref = rk3_relaxation(vel[:dim], tau, dt, steps, x0[0])
    x, v = st.x.reshape(3, dim), st.v.reshape(3, dim)
    np.testing.assert_allclose(v[0], ref[:, 1], rtol=1e-12)
    np.testing.assert_allclose(x[0], ref[:, 0], rtol=1e-12, atol=1e-15)
    assert np.all(v[1:] == 0.0) and np.array_equal(x[1:], x0[1:])
    # approaching vel like 1 - exp(-t / tau)
    np.testing.assert_allclose(v[0], vel[:dim] * (1.0 - np.exp(-steps * dt / tau)), rtol=1e-3)
