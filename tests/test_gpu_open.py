"""Open boundaries of the GPU-C schemes on the GPU (armando_set_open_boundaries,
armando_integrate_open) vs the FP64 oracle: particle counts exactly, the
particles in the same order (survivors in input order, then new ones in
emission order), fields at the RK3 scheme's gates."""
import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from armando_gb300._abi import Inlet, Outlet
from helpers import rel_err

pytestmark = pytest.mark.gpu

CAP = 2000
TOL = {"x": 1e-6, "rho": 1e-6, "u": 1e-6, "v": 5e-5, "p": 2e-4, "dvdt": 2e-4}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def run_gpu(c, n, inlets, outlets, box, steps, loads=(), fixes=()):
    a = {k: v.copy() for k, v in c.arrays().items()}
    with ag.Context(c.params, CAP, 0) as ctx:
        ctx.set_open_boundaries(inlets, outlets, box)
        if loads or fixes:
            ctx.set_zones(list(loads), list(fixes))
        m = ctx.integrate_open(a, c.dt, 1, steps, n)
    return m, a


def compare(O, c, n, inlets, outlets, box, steps, tol_scale=1.0, loads=(), fixes=()):
    m, a = run_gpu(c, n, inlets, outlets, box, steps, loads, fixes)
    ref = O.gpuc_open(c, steps, c.dt, CAP, n=n, inlets=inlets, outlets=outlets, box=box,
                      loads=loads, fixes=fixes)
    assert m == len(ref["mass"])
    assert np.array_equal(a["itype"][:m], ref["itype"])
    bad = {}
    d = c.dim
    for f, g in (("x", a["x"][:d * m]), ("v", a["v"][:d * m]), ("rho", a["rho"][:m]),
                 ("p", a["p"][:m]), ("dvdt", a["dvdt"][:d * m])):
        e = rel_err(g, ref[f])
        if not e <= TOL[f] * tol_scale:
            bad[f] = e
    assert not bad, bad
    return m


def test_one_step_removes_and_emits(O):
    """From identical FP32 inputs: a column already past the outlet leaves, a
    fast inlet emits in the first step."""
    c, n, inl, outl, box = cases.gpuc_open_channel()
    x = c.x.reshape(-1, 2)
    fl = np.arange(CAP) < n
    past = fl & (c.itype > 0) & (x[:, 0] > 0.28)
    x[past, 0] += 0.03  # the last two columns beyond x = 0.3
    c.x = x.ravel()
    I = inl[0]
    fast = Inlet.make(tuple(I.origin), tuple(I.normal), I.radius, 1, I.mass, I.hsml,
                      0.011 / c.dt, I.rho)
    m = compare(O, c, n, [fast], outl, box, 1)
    assert m == n - int(past.sum()) + 11


def test_open_channel_over_100_steps(O):
    """Water at 1 m/s: a column leaves at the outlet (step 42) and a new one
    enters (step 84); counts, order and fields against the oracle."""
    c, n, inl, outl, box = cases.gpuc_open_channel()
    m = compare(O, c, n, inl, outl, box, 100, tol_scale=5.0)
    assert m == n - 10 + 11


def test_device_variant(O):
    """Scheme 2 runs the same open channel; its wall push differs from scheme
    1's and a second column leaves by step 80 (the oracle agrees)."""
    c, n, inl, outl, box = cases.gpuc_open_channel(scheme=2)
    m = compare(O, c, n, inl, outl, box, 100, tol_scale=5.0)
    assert m == n - 20 + 11


def test_disk_inlet_3d(O):
    """A 3D duct with a disk inlet across its start (normal +x) and an outlet
    at its end: the first steps emit disks of the reference's lattice; counts,
    order and fields against the oracle."""
    c = cases.channel(n_x=10, n_yz=4, length=10 * 7.9e-4, width=4 * 7.9e-4, layers=2, jitter=0.01)
    c.params.scheme = 2
    c.params.periodic[:] = (0, 0, 0)
    c.params.heat_external = 0
    n = c.n
    h = float(c.h[0])
    I = Inlet.make((0.0, 0.0016, 0.0016), (1.0, 0.0, 0.0), 1.5 * h, 1, float(c.mass[0]), h,
                   0.6 * h / 1.2 / c.dt, 10500.0, float(c.u[0]))
    L = 10 * 7.9e-4
    outl = [Outlet.make((L - 1.0e-4, 0.0016, 0.0016), (-1.0, 0.0, 0.0), 0.01)]
    box = ((-0.01, -0.01, -0.01), (0.02, 0.02, 0.02))
    padded = c.copy()
    for f, w in (("x", 3), ("v", 3), ("mass", 1), ("rho", 1), ("p", 1), ("u", 1), ("h", 1),
                 ("itype", 1), ("dvdt", 3), ("dudt", 1)):
        a = getattr(c, f)
        out = np.zeros(CAP * w, a.dtype)
        out[:a.size] = a
        setattr(padded, f, out)
    m = compare(O, padded, n, [I], outl, box, 4)
    assert m > n


def test_refusals():
    c, n, inl, outl, box = cases.gpuc_open_channel()
    p0 = c.params.copy()
    p0.scheme = 0
    a = {k: v.copy() for k, v in c.arrays().items()}
    with ag.Context(p0, CAP, 0) as ctx:
        ctx.set_open_boundaries(inl, outl, box)
        with pytest.raises(ag.ArmandoError) as e:
            ctx.integrate_open(a, c.dt, 1, 1, n)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED
    with ag.Context(c.params, CAP, 0) as ctx:
        with pytest.raises(ag.ArmandoError) as e:
            ctx.integrate_open(a, c.dt, 1, 1, n)
        assert e.value.status == ag._abi.ERR_INVALID_ARG
    with ag.Context(c.params, n + 5, 0) as ctx:  # no room for an inflow column
        small = {k: v[:(n + 5) * (2 if k in ("x", "v", "dvdt") else 1)].copy() for k, v in a.items()}
        ctx.set_open_boundaries(inl, [], box)
        with pytest.raises(ag.ArmandoError) as e:
            ctx.integrate_open(small, c.dt, 1, 100, n)
        assert e.value.status == ag._abi.ERR_INVALID_ARG


def test_empty_system_refills(O):
    """Every particle leaves in the first step; steps on no particles launch
    nothing; the inlet refills the system in the third step."""
    c, n, inl, _, _ = cases.gpuc_open_channel()
    I = inl[0]
    o = np.array(I.origin[:2])
    box = (tuple(o - 0.06), tuple(o + 0.06 + [0.02, 0.0]))
    fast = Inlet.make(tuple(I.origin), tuple(I.normal), I.radius, 1, I.mass, I.hsml,
                      0.4 * I.hsml / 1.2 / c.dt, I.rho)
    x = c.x.reshape(-1, 2)
    inside = np.all((x[:n] >= box[0]) & (x[:n] <= box[1]), axis=1)
    c.x[:2 * n] = np.where(np.repeat(inside, 2), c.x[:2 * n] + 1.0, c.x[:2 * n])
    m, _ = run_gpu(c, n, [fast], [], box, 2)
    assert m == 0
    assert compare(O, c, n, [fast], [], box, 3) == 11


def test_open_channel_with_zones(O):
    """The open channel driven like the reference's channel runs: a fix zone
    over the water of the inflow strip (initChannel's hFix) and a heated,
    accelerated band downstream, 20 steps against the oracle. No particle
    comes near a zone's edge in that time: a particle on an edge (a wall
    column at x = 0.04, say) enters or stays out on one ulp of its position."""
    from armando_gb300._abi import FixZone, LoadZone

    c, n, inl, outl, box = cases.gpuc_open_channel()
    fixes = [FixZone.make((-1.0, 0.0), (0.04, 0.1), (1.2, 0.0))]
    loads = [LoadZone.make((0.15, -1.0), (0.22, 1.0), (2.0, 0.0), 500.0)]
    m = compare(O, c, n, inl, outl, box, 20, tol_scale=5.0, loads=loads, fixes=fixes)
    assert m == n
