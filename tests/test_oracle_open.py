"""Open boundaries of the oracle's GPU-C scheme (inlets, outlets and box,
ArmandoThrust/armando.cu:2640-2856): the emission lattice, its timing, the
removal rule and the order of the particles, by hand on small cases."""
import numpy as np

from armando_gb300 import cases
from armando_gb300._abi import Inlet, Outlet


def still_channel(**kw):
    c, n, inl, outl, box = cases.gpuc_open_channel(**kw)
    return c, n, inl, outl, box


def test_segment_inlet_lattice_and_timing(O):
    """2D inlet: a segment of spacing h/1.2 across the normal, |r| < R; it
    emits once its distance passes h/1.2 (speed dt per step)."""
    c, n, inl, _, box = still_channel()
    dr, dt = 0.01, c.dt
    I = inl[0]
    steps = int(np.ceil(dr / (1.0 * dt))) + 1  # the first emission falls in this run
    out = O.gpuc_open(c, steps, dt, 4000, n=n, inlets=[I], outlets=[], box=box, fp32=False)
    # the lattice in FP32 as the reference computes it: spacing h/1.2 (just
    # under 0.01 in FP32, so the ends iu = +-5 fall inside R = 0.05)
    f32 = np.float32
    sp = f32(I.hsml) / f32(1.2)
    nn = int(np.round(f32(1.2) * f32(I.radius) / f32(I.hsml)))
    k = np.arange(-nn, nn + 1)
    r = (k.astype(np.float32) * f32(1.0)) * sp  # u = (-w_y, w_x) = (0, 1)
    k = k[np.abs(r) < f32(I.radius)]
    assert len(out["mass"]) == n + len(k) == n + 11
    # emitted at the start of step 84 (the distance passes h/1.2 there), then
    # carried by steps 84 and 85 at v dt = 1.2e-4 m each
    new = out["x"].reshape(-1, 2)[n:]
    np.testing.assert_allclose(new[:, 1], f32(I.origin[1]) + (k.astype(np.float32) * f32(1.0)) * sp,
                               rtol=0, atol=2e-5)
    np.testing.assert_allclose(new[:, 0], I.origin[0] + 2 * I.speed * dt, rtol=0, atol=2e-5)
    assert np.all(out["itype"][n:] == 1)
    np.testing.assert_allclose(out["v"].reshape(-1, 2)[n:, 0], 1.0, rtol=0.02)  # after two steps
    # one step earlier: nothing yet
    out0 = O.gpuc_open(c, steps - 2, dt, 4000, n=n, inlets=[I], outlets=[], box=box)
    assert len(out0["mass"]) == n


def test_disk_inlet_lattice_3d(O):
    """3D inlet with normal +x: rows along z (the axis of w's smallest
    component, the last on ties) and y; points (iu, iv) sp with |r| < R."""
    c = cases.channel(n_x=10, n_yz=4, length=10 * 7.9e-4, width=4 * 7.9e-4, layers=2)
    c.params.scheme = 1
    c.params.periodic[0] = 0
    h = float(c.h[0])
    R = 3.0 * h
    I = Inlet.make((0.0, 0.0015, 0.0015), (1.0, 0.0, 0.0), R, 1, float(c.mass[0]), h, 1e3,
                   10500.0)
    out = O.gpuc_open(c, 1, 1e-6 * 2, c.n + 500, inlets=[I], outlets=[],
                      box=((-1, -1, -1), (1, 1, 1)))
    sp = np.float32(h) / np.float32(1.2)
    nn = int(np.round(np.float32(1.2) * np.float32(R) / np.float32(h)))
    iu, iv = np.meshgrid(np.arange(-nn, nn + 1), np.arange(-nn, nn + 1), indexing="ij")
    expect = int(np.sum(np.sqrt((iu * sp) ** 2 + (iv * sp) ** 2) < np.float32(R)))
    assert len(out["mass"]) == c.n + expect


def test_outlet_and_box_remove_and_keep_order(O):
    c, n, _, outl, box = still_channel()
    x = c.x.reshape(-1, 2)
    x[3] = (0.305, 0.05)        # behind the outlet, within its radius: leaves
    x[7] = (0.305, 0.2 - 0.05)  # behind the plane but outside the radius: stays
    x[11] = (-0.5, 0.05)        # outside the box: leaves
    c.x = x.ravel()
    out = O.gpuc_open(c, 1, 1e-9, 4000, n=n, inlets=[], outlets=outl, box=box)
    assert len(out["mass"]) == n - 2
    keep = [i for i in range(n) if i not in (3, 11)]
    np.testing.assert_allclose(out["x"].reshape(-1, 2)[:, 1], c.x.reshape(-1, 2)[keep, 1], atol=1e-6)
    assert Outlet is not None


def test_open_channel_flow_counts(O):
    """Water at 1 m/s through the channel: the first column leaves at the
    outlet around step 42, the first new column enters at step 84."""
    c, n, inl, outl, box = still_channel()
    out = O.gpuc_open(c, 100, c.dt, 4000, n=n, inlets=inl, outlets=outl, box=box)
    assert len(out["mass"]) == n - 10 + 11
    assert np.all(np.isfinite(out["x"])) and np.all(np.isfinite(out["rho"]))


def test_empty_system_refills(O):
    """A box that holds none of the particles empties the system in the first
    step; steps on nothing do nothing until the inlet (inside the box) emits."""
    c, n, inl, _, _ = still_channel()
    I = inl[0]
    o = np.array(I.origin[:2])
    box = (tuple(o - 0.06), tuple(o + 0.06 + [0.02, 0.0]))
    fast = Inlet.make(tuple(I.origin), tuple(I.normal), I.radius, 1, I.mass, I.hsml,
                      0.4 * I.hsml / 1.2 / c.dt, I.rho)
    x = c.x.reshape(-1, 2)
    inside = np.all((x[:n] >= box[0]) & (x[:n] <= box[1]), axis=1)
    c.x[:2 * n] = np.where(np.repeat(inside, 2), c.x[:2 * n] + 1.0, c.x[:2 * n])  # move them out
    out = O.gpuc_open(c, 2, c.dt, 4000, n=n, inlets=[fast], outlets=[], box=box)
    assert len(out["mass"]) == 0
    out = O.gpuc_open(c, 3, c.dt, 4000, n=n, inlets=[fast], outlets=[], box=box)
    assert len(out["mass"]) == 11 and np.all(np.isfinite(out["x"]))
