"""Edge cases of the CERN step on the GPU: an empty system, a system of walls
only, a single fluid particle, and a fluid particle with no neighbour beside
a dense block, each against the oracle or its known answer."""
import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def subset(c, keep):
    """The particles `keep` of case c (same parameters)."""
    out = c.copy()
    keep = np.asarray(keep, dtype=np.int64)
    for f in ("mass", "rho", "p", "u", "h", "itype", "dudt"):
        setattr(out, f, getattr(c, f)[keep].copy())
    for f in ("x", "v", "dvdt"):
        setattr(out, f, getattr(c, f).reshape(-1, c.dim)[keep].ravel().copy())
    return out


def test_empty_system():
    c = subset(cases.dam_break(dx=0.1), [])
    with ag.Context(c.params, 0, 0) as ctx:
        ctx.step(c, c.dt, 1)
        ctx.integrate(c, c.dt, 2, 3)
        assert ctx.stats().n_particles == 0


def test_walls_only_are_left_alone():
    """No fluid: every wall keeps its state bit for bit (time_integration.f
    integrates 1..np only)."""
    c0 = cases.dam_break(dx=0.1)
    c = subset(c0, np.flatnonzero(c0.itype <= 0))
    got = c.copy()
    with ag.Context(c.params, 0, c.n) as ctx:
        ctx.integrate(got, c.dt, 1, 3)
    for f in ("x", "v", "rho", "p", "u"):
        np.testing.assert_array_equal(getattr(got, f), getattr(c, f), err_msg=f)


def test_single_fluid_particle(O):
    """One particle alone: density is its self term m W(0, h) (no pmin
    clamp), it falls under gravity; one step against the oracle."""
    c0 = cases.dam_break(dx=0.1)
    c = subset(c0, [int(np.flatnonzero(c0.itype > 0)[0])])
    c.params.pmin = -np.inf  # keep the summed density (p < pmin would reset it to rho0)
    ref = O.State(c)
    O.step(ref, 1, c.dt)
    got = c.copy()
    with ag.Context(c.params, 1, 0) as ctx:
        ctx.step(got, c.dt, 1)
    for f in FIELDS:
        assert rel_err(getattr(got, f), getattr(ref, f)) <= 1e-6, f
    w0 = cases.wendland_w(0.0, float(c.h[0]), 2)
    np.testing.assert_allclose(got.rho[0], c.mass[0] * w0, rtol=1e-6)
    assert got.dvdt[1] == pytest.approx(c.params.gravity[1], rel=1e-6)


def test_isolated_particle_beside_a_block(O):
    """A fluid particle far from a dam-break block: it sees only itself while
    the block's particles keep their neighbours; one step against the oracle."""
    c0 = cases.perturbed(cases.dam_break(dx=0.05), seed=5, dv=0.05)
    c = c0.copy()
    c.params.pmin = -np.inf
    x = c.x.reshape(-1, 2).copy()
    k = int(np.flatnonzero(c.itype > 0)[-1])
    x[k] = x[:, 0].max() + 10 * float(c.h[k]), x[:, 1].max() + 10 * float(c.h[k])
    c.x = x.ravel().astype(np.float32)
    ref = O.State(c)
    O.step(ref, 1, c.dt)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.step(got, c.dt, 1)
    for f in FIELDS:
        assert rel_err(getattr(got, f), getattr(ref, f)) <= 1e-5, f
    w0 = cases.wendland_w(0.0, float(c.h[k]), 2)
    np.testing.assert_allclose(got.rho[k], c.mass[k] * w0, rtol=1e-6)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 0), (3, 1, 256, 10)])
def test_far_outlier_reports_grid_overflow(tuning):
    """One particle 1e4 m out on every axis of a 3D block: the cell count per
    axis is ~5e6, whose product over three axes exceeds every capacity (and a
    64-bit integer). The call must fail with GRID_OVERFLOW, not run on a
    wrapped count."""
    c = cases.channel(n_x=12, n_yz=6, length=12 * 7.9e-4, width=6 * 7.9e-4, layers=1,
                      jitter=0.01)
    c.params.periodic[:] = [0, 0, 0]
    i = int(np.flatnonzero(c.itype > 0)[0])
    c.x.reshape(-1, 3)[i] = [1.0e4, 1.0e4, 1.0e4]
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(*tuning)
        with pytest.raises(ag.ArmandoError) as e:
            ctx.step(c.copy(), c.dt, 1)
        assert e.value.status == ag._abi.ERR_GRID_OVERFLOW
        with pytest.raises(ag.ArmandoError) as e:
            ctx.cell_ids(c.x, c.h)
        assert e.value.status == ag._abi.ERR_GRID_OVERFLOW
