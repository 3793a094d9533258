"""The GPU-C schemes (armando_params.scheme 1 and 2: TVD-RK3, continuity
density) on the GPU, against the reference's own compiled C host path
(ArmandoThrust/acpu.c golden vectors, tests/golden/acpu_rk3.npz) and against
the FP64 oracle.

Gates (normwise relative per output; acpu.c and the library compute in FP32):
the integrated state x, rho, u within 1e-6 of the reference's; pressure and
the velocity rates within 2e-4, velocity within 5e-5, because one FP32 ulp of
rho ~ 1000 is 0.15 Pa of Tait pressure (c0 = 50 m/s); the water tank's energy
and its rate, pure pressure work, within 5e-4.
"""
import os

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from armando_gb300._abi import Material

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acpu_rk3.npz")
TOL = {"x": 1e-6, "rho": 1e-6, "u": 1e-6, "v": 5e-5, "p": 2e-4, "dv": 2e-4, "du": 2e-4}

TAIT = Material.make(4, [1000.0, 50.0, -1.0e12])
SHOCK = Material.make(3, [1000.0, 50.0, 0.5, 1.3])
POLY = Material.make(2, [1000.0, 2.5e6, 1.0e6, 2.0e5, 0.2, 0.1, 2.5e6, 5.0e5])
WALL = Material.make(0, [1000.0, 50.0])


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


@pytest.fixture(scope="module")
def G():
    return np.load(GOLD)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    s = np.abs(b).max()
    return np.abs(a - b).max() / s if s > 0 else np.abs(a).max()


def golden_case(G, pre):
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    c.x, c.v, c.mass, c.rho = (G[pre + "_x0"].copy(), G[pre + "_v0"].copy(), G[pre + "_m"].copy(),
                               G[pre + "_rho0"].copy())
    c.h, c.itype = G[pre + "_h"].copy(), G[pre + "_itype"].copy()
    if pre + "_u0" in G:
        c.u = G[pre + "_u0"].copy()
    c.dt = float(G[pre + "_dt"])
    return c


def run_gpu(c, steps, materials=None, tuning=None):
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        if materials is not None:
            ctx.set_materials(materials)
        if tuning is not None:
            ctx.set_tuning(*tuning)
        ctx.integrate(got, c.dt, 1, steps)
    return got


def fields(c):
    return {"x": c.x, "v": c.v, "rho": c.rho, "p": c.p, "u": c.u, "dv": c.dvdt, "du": c.dudt}


@pytest.mark.parametrize("steps", [1, 5])
@pytest.mark.parametrize("pre", ["water", "multi"])
def test_matches_acpu_golden(G, pre, steps):
    c = golden_case(G, pre)
    mats = [TAIT, TAIT] if pre == "water" else [WALL, TAIT, SHOCK, WALL, POLY]
    got = fields(run_gpu(c, steps, mats))
    bad = {}
    for f in ("x", "v", "rho", "p", "u", "dv", "du"):
        ref = G[f"{pre}_{f}_{steps}"]
        # The water's u is pressure work from u = 0: it carries p's quantization,
        # from two FP32 computations here (the library's and acpu.c's).
        tol = 5e-4 if (pre == "water" and f in ("u", "du")) else TOL[f]
        e = rel(got[f].reshape(ref.shape), ref)
        if not e <= tol:
            bad[f] = e
    assert not bad, (pre, steps, bad)


@pytest.mark.parametrize("scheme", [1, 2])
def test_published_dam_break_matches_the_oracle(O, scheme):
    """The published 6,462-particle dam break (Tab.1 case 1), 10 RK3 steps,
    both physics variants."""
    c = cases.gpuc_dam_break(1, scheme=scheme)
    rng = np.random.default_rng(90 + scheme)
    v = c.v.reshape(-1, 2)
    v[c.itype > 0] = rng.normal(0.0, 0.05, size=(c.n_fluid, 2))
    c.v = v.ravel().astype(np.float32)
    ref = O.State(c)
    dv, du = O.gpuc_step(ref, 10, c.dt)
    got = run_gpu(c, 10)
    for f, a, b in (("x", got.x, ref.x), ("v", got.v, ref.v), ("rho", got.rho, ref.rho),
                    ("p", got.p, ref.p), ("dv", got.dvdt, dv)):
        assert rel(a, b) <= TOL[f] * 2, (scheme, f, rel(a, b))


@pytest.mark.parametrize("tuning", [(2, 1, 256, 0), (3, 1, 128, 0), (1, 2, 128, 0), (1, 4, 256, 0),
                                    (2, 4, 128, 0), (2, 1, 128, 20), (1, 2, 256, 40)])
def test_tunings(O, G, tuning):
    """Cell reach, lanes per particle (their sums in another order) and CTA
    size against acpu.c."""
    c = golden_case(G, "multi")
    mats = [WALL, TAIT, SHOCK, WALL, POLY]
    got = fields(run_gpu(c, 5, mats, tuning))
    for f in ("x", "v", "rho", "p", "u"):
        ref = G[f"multi_{f}_5"]
        assert rel(got[f].reshape(ref.shape), ref) <= TOL[f], (tuning, f)


def test_integrate_is_deterministic_and_equals_steps():
    """Bitwise repeatable; one call of 6 steps and 6 calls of one step agree to
    rounding (per call the cell sort starts from caller order, inside a call
    from the last sort, so a particle that changed cell sums in another order)."""
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16), scheme=2)
    a, b, d = c.copy(), c.copy(), c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(a, c.dt, 1, 6)
        ctx.integrate(b, c.dt, 1, 6)
        for its in range(1, 7):
            ctx.step(d, c.dt, its)
    for f in ("x", "v", "rho", "p", "u", "dvdt", "dudt"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
        tol = {"dvdt": TOL["dv"], "dudt": 5e-4, "u": 5e-4}.get(f, TOL.get(f))
        assert rel(getattr(d, f), getattr(a, f)) <= tol, f


def test_itype_outside_the_table_is_an_error():
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    c.itype[c.itype > 0] = 3
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_materials([TAIT, TAIT])
        with pytest.raises(ag.ArmandoError) as e:
            ctx.step(c.copy(), c.dt, 1)
        assert e.value.status == ag._abi.ERR_INVALID_ARG


def test_refusals():
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        with pytest.raises(ag.ArmandoError) as e:
            ctx.forward_checkpointed(c.copy(), c.dt, 1, 4, 2)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED
        with pytest.raises(ag.ArmandoError) as e:
            ctx.set_materials([Material.make(9, [1.0])])
        assert e.value.status == ag._abi.ERR_INVALID_ARG
    with pytest.raises(ag.ArmandoError) as e:
        ag.Batch([c.params, c.params], [c.n_fluid] * 2, [c.n_wall] * 2)
    assert e.value.status == ag._abi.ERR_UNSUPPORTED
    bad = c.params.copy()
    bad.wall_model = 1
    with pytest.raises(ag.ArmandoError) as e:
        ag.Context(bad, c.n_fluid, c.n_wall)
    assert e.value.status == ag._abi.ERR_INVALID_ARG


GOLD_ZONES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acpu_zones.npz")


def zones_of(Z):
    from armando_gb300._abi import FixZone, LoadZone

    loads = [LoadZone.make(r[0:2], r[2:4], (r[4], r[5], 0.0), r[6]) for r in Z["zones_load"]]
    fixes = [FixZone.make(r[0:2], r[2:4], (r[4], r[5], 0.0)) for r in Z["zones_fix"]]
    return loads, fixes


@pytest.mark.parametrize("steps", [1, 5])
def test_zones_match_acpu_golden(steps):
    """Two overlapping load zones and a fix zone over water and part of the
    left wall, against acpu.c (u: pressure work next to the fixed water, gated
    like the water tank's)."""
    Z = np.load(GOLD_ZONES)
    loads, fixes = zones_of(Z)
    c = golden_case(Z, "zones")
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_materials([TAIT, TAIT])
        ctx.set_zones(loads, fixes)
        ctx.integrate(got, c.dt, 1, steps)
    g = fields(got)
    bad = {}
    for f in ("x", "v", "rho", "p", "u", "dv", "du"):
        ref = Z[f"zones_{f}_{steps}"]
        tol = 5e-4 if f in ("u", "du") else TOL[f]
        e = rel(g[f].reshape(ref.shape), ref)
        if not e <= tol:
            bad[f] = e
    assert not bad, (steps, bad)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_zone_known_answers(dim, scheme):
    """Isolated particles, one RK3 step: the load zones' v = dt a, u = u0 + dt w
    (overlapping zones adding; in 3D the z bounds decide), the fix zone's
    x = x0 + (5/6) dt vel from rest."""
    from armando_gb300._abi import FixZone, LoadZone

    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16), scheme=scheme)
    pts = np.array([[0.1, 0.2, 0.3], [1.1, 0.2, -0.4], [2.1, -0.9, 0.3]])[:, :dim]
    c.params.dim = c.dim = dim
    c.params.gravity[:] = (0.0, 0.0, 0.0)
    for f in ("mass", "rho", "p", "u", "h", "itype", "dudt"):
        setattr(c, f, getattr(c, f)[:3].copy())
    c.itype[:] = 1
    c.x = pts.ravel().astype(np.float32)
    c.v = np.zeros(3 * dim, np.float32)
    c.dvdt = np.zeros(3 * dim, np.float32)
    c.u = np.full(3, 5.0, np.float32)
    dt = 1e-3
    a1, a2 = np.array([2.0, -1.0, 0.5]), np.array([0.25, 0.5, -4.0])
    loads = [LoadZone.make((0.0, 0.0, -0.1), (1.5, 0.5, 0.5), a1, 300.0),
             LoadZone.make((1.0, 0.0, -0.1), (1.5, 0.5, 0.5), a2, 20.0)]
    vel = np.array([0.7, -0.3, 0.2])
    fixes = [FixZone.make((2.0, -1.0, 0.0), (2.5, -0.5, 0.5), vel)]
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_zones(loads, fixes)
        ctx.integrate(got, dt, 1, 1)
    x0 = c.x.reshape(3, dim).astype(np.float64)
    x, v = got.x.reshape(3, dim), got.v.reshape(3, dim)
    acc = [a1[:dim], (a1 + a2)[:dim]]
    w = [300.0, 320.0]
    if dim == 3:
        acc[1], w[1] = np.zeros(3), 0.0
    for k in range(2):
        np.testing.assert_allclose(v[k], dt * acc[k], rtol=1e-6, atol=1e-9)
        np.testing.assert_allclose(x[k], x0[k] + 0.5 * dt * dt * acc[k], rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(got.u[k], 5.0 + dt * w[k], rtol=1e-6)
    np.testing.assert_allclose(v[2], vel[:dim], rtol=1e-6)
    np.testing.assert_allclose(x[2], x0[2] + dt * 5.0 / 6.0 * vel[:dim], rtol=1e-6, atol=1e-7)


def test_zones_3d_channel_matches_the_oracle(O):
    """A 3D block of water, device-variant physics, with a heated
    accelerating load zone and a fix zone over its inflow end: 3 RK3 steps
    against the FP64 oracle."""
    from armando_gb300._abi import FixZone, LoadZone

    c = cases.channel(n_x=14, n_yz=6, length=14 * 7.9e-4, width=6 * 7.9e-4, layers=2, jitter=0.01)
    c.params.scheme = 2
    c.params.periodic[:] = (0, 0, 0)
    c.params.heat_external = 0
    c.params.gravity[:] = (0.0, 0.0, -9.81)
    L = 14 * 7.9e-4
    loads = [LoadZone.make((0.4 * L, -1.0, -1.0), (0.8 * L, 1.0, 1.0), (30.0, 0.0, 5.0), 2.0e3)]
    fixes = [FixZone.make((-1.0, -1.0, -1.0), (0.15 * L, 1.0, 1.0), (0.8, 0.0, 0.0))]
    ref = O.State(c)
    dv, du = O.gpuc_step(ref, 3, c.dt, loads=loads, fixes=fixes)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_zones(loads, fixes)
        ctx.integrate(got, c.dt, 1, 3)
    for f, a, b in (("x", got.x, ref.x), ("v", got.v, ref.v), ("rho", got.rho, ref.rho),
                    ("p", got.p, ref.p), ("u", got.u, ref.u), ("dv", got.dvdt, dv)):
        assert rel(a, b) <= TOL[f] * 2, (f, rel(a, b))


def test_zone_refusals():
    from armando_gb300._abi import FixZone, LoadZone

    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    z = LoadZone.make((0.0, 0.0), (1.0, 1.0), (1.0, 0.0), 0.0)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        with pytest.raises(ag.ArmandoError) as e:
            ctx.set_zones([z] * 11, [])
        assert e.value.status == ag._abi.ERR_INVALID_ARG
        with pytest.raises(ag.ArmandoError) as e:
            ctx.set_zones([], [FixZone.make((0.0, 0.0), (1.0, 1.0), (float("nan"), 0.0))])
        assert e.value.status == ag._abi.ERR_INVALID_ARG
        ctx.set_zones([], [])
    p0 = c.params.copy()
    p0.scheme = 0
    with ag.Context(p0, c.n_fluid, c.n_wall) as ctx:
        with pytest.raises(ag.ArmandoError) as e:
            ctx.set_zones([z], [])
        assert e.value.status == ag._abi.ERR_UNSUPPORTED


@pytest.mark.parametrize("scheme", [1, 2])
def test_lazy_sorting_matches_sorting_every_step(scheme):
    """A sort skin: the published 6,462-particle dam break over 40 steps sorts
    on a few of them and agrees with the every-step run to rounding: the
    neighbour lists are the same; only the summation order follows the older
    cells. Gate: 20x the every-step run's own change when its positions move
    by one ulp (u and de/dt are pure pressure work from u = 0 and carry p's
    quantization)."""
    c = cases.gpuc_dam_break(1, scheme=scheme)
    rng = np.random.default_rng(70 + scheme)
    v = c.v.reshape(-1, 2)
    v[c.itype > 0] = rng.normal(0.0, 0.05, size=(c.n_fluid, 2))
    c.v = v.ravel().astype(np.float32)
    every, lazy, twin = c.copy(), c.copy(), c.copy()
    bump = np.where(rng.random(c.x.size) < 0.5, np.inf, -np.inf).astype(np.float32)
    twin.x = np.nextafter(c.x, bump).astype(np.float32)
    for run in (every, twin):
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(2, 1, 128, 0)
            ctx.integrate(run, c.dt, 1, 40)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(2, 1, 128, 20)
        s0 = ctx.stats().sorts_done
        ctx.integrate(lazy, c.dt, 1, 40)
        sorts = ctx.stats().sorts_done - s0
    assert 1 <= sorts < 40
    for f in ("x", "v", "rho", "p", "u", "dvdt", "dudt"):
        cond = rel(getattr(twin, f), getattr(every, f))
        err = rel(getattr(lazy, f), getattr(every, f))
        assert err <= max(20.0 * cond, 1e-6), (f, err, cond)


@pytest.mark.parametrize("scheme", [1, 2])
def test_pressure_wave_matches_the_oracle(O, scheme):
    """The pressure-wave stand-in (polynomial EOS of mercury, free surfaces,
    a Gaussian energy deposit) on a 41 x 41 lattice, 10 RK3 steps. Mercury is
    stiff: one FP32 ulp of rho = 13,540 is 2,200 Pa at c0 = 1,490 m/s, and
    the library rounds its state to FP32 after every stage. Gate: the gates
    above or 20x the oracle's own change when every FP32 input (x, v, rho, u)
    moves by one ulp, whichever is larger."""
    c = cases.gpuc_pressure_wave(41, radius=0.02, scheme=scheme)
    mats = [cases.mercury_poly()] * 2
    ref = O.State(c)
    dv, du = O.gpuc_step(ref, 10, c.dt, materials=mats)
    rng = np.random.default_rng(60 + scheme)
    twin = c.copy()
    for f in ("x", "v", "rho", "u"):
        a = getattr(c, f)
        bump = np.where(rng.random(a.size) < 0.5, np.inf, -np.inf).astype(np.float32)
        setattr(twin, f, np.nextafter(a, bump).astype(np.float32))
    tw = O.State(twin)
    dvt, _ = O.gpuc_step(tw, 10, c.dt, materials=mats)
    got = run_gpu(c, 10, mats)
    for f, a, b, t in (("x", got.x, ref.x, tw.x), ("v", got.v, ref.v, tw.v),
                       ("rho", got.rho, ref.rho, tw.rho), ("p", got.p, ref.p, tw.p),
                       ("u", got.u, ref.u, tw.u), ("dv", got.dvdt, dv, dvt)):
        err, cond = rel(a, b), rel(t, b)
        assert err <= max(TOL[f], 20.0 * cond), (scheme, f, err, cond)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_pump_zone_known_answer(O, dim, scheme):
    """A pump zone relaxing an isolated particle towards vel (dv/dt = (vel - v)
    / tau, Code/armando.cu:1046-1055): ten RK3 steps against the exact RK3
    answer of the linear system and against the oracle; particles outside the
    zone stay at rest."""
    from armando_gb300._abi import FixZone

    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16), scheme=scheme)
    pts = np.array([[0.1, 0.2, 0.3], [1.1, 0.2, -0.4], [2.1, -0.9, 0.3]])[:, :dim]
    c.params.dim = c.dim = dim
    c.params.gravity[:] = (0.0, 0.0, 0.0)
    for f in ("mass", "rho", "p", "u", "h", "itype", "dudt"):
        setattr(c, f, getattr(c, f)[:3].copy())
    c.itype[:] = 1
    c.x = pts.ravel().astype(np.float32)
    c.v = np.zeros(3 * dim, np.float32)
    c.dvdt = np.zeros(3 * dim, np.float32)
    dt, tau, steps = 1e-3, 5e-3, 10
    vel = np.array([0.7, -0.3, 0.2])
    pumps = [FixZone.make((0.0, 0.0, 0.0), (0.5, 0.5, 0.5), vel, tau)]
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_zones([], pumps)
        ctx.integrate(got, dt, 1, steps)
    ref = O.State(c)
    O.gpuc_step(ref, steps, dt, fixes=pumps)
    v, x = got.v.reshape(3, dim), got.x.reshape(3, dim)
    np.testing.assert_allclose(v, ref.v.reshape(3, dim), rtol=2e-6, atol=1e-9)
    np.testing.assert_allclose(x, ref.x.reshape(3, dim), rtol=1e-6, atol=1e-7)
    assert np.all(v[1:] == 0.0)
    np.testing.assert_allclose(v[0], vel[:dim] * (1.0 - np.exp(-steps * dt / tau)), rtol=1e-3)
