"""Neighbour passes with the CTA's candidates staged in shared memory.

The staged passes (one thread per particle, lean physics, no periodic axis)
must give the same bits as the same passes reading global memory
(ARMANDO_STAGING=0): same candidates in the same order, same arithmetic. That
includes CTAs whose stencil ranges do not fit the shared-memory capacity (a
sparse column below a dense block) and fall back to global memory inside the
staged kernel, and grids thinner than the stencil. Plus one step against the
FP64 oracle on those layouts.
"""
import os

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS, history_state, step_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def _run(c, tuning, steps, staging):
    old = os.environ.get("ARMANDO_STAGING")
    os.environ["ARMANDO_STAGING"] = "1" if staging else "0"
    try:
        out = c.copy()
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(*tuning)
            ctx.integrate(out, c.dt, 1, steps)
        return out
    finally:
        if old is None:
            del os.environ["ARMANDO_STAGING"]
        else:
            os.environ["ARMANDO_STAGING"] = old


def _lattice_2d(points, dx):
    """Fluid particles at `points` (k x 2, metres) with the dam break's physics."""
    base = cases.dam_break(dx=0.05)
    n = len(points)
    rho0 = float(base.params.rho0)
    c = base.copy()
    c.x = np.ascontiguousarray(points, np.float32).ravel()
    c.v = np.zeros(2 * n, np.float32)
    c.mass = np.full(n, rho0 * dx * dx, np.float32)
    c.rho = np.full(n, rho0, np.float32)
    c.p = np.zeros(n, np.float32)
    c.u = np.zeros(n, np.float32)
    c.h = np.full(n, 1.3 * dx, np.float32)
    c.itype = np.ones(n, np.int32)
    c.dvdt = np.zeros(2 * n, np.float32)
    c.dudt = np.zeros(n, np.float32)
    c.dt = 0.2 * 1.3 * dx / float(base.params.c0)
    return c


def _sparse_below_dense(dx=1.0e-3, seed=3):
    """An isolated column of particles 3 dx apart (no neighbours) below a
    2000 x 12 block: the CTA holding the column's top and the block's first
    particles has stencil ranges over several full block rows."""
    rng = np.random.default_rng(seed)
    col = np.stack([np.full(300, 1.0), np.arange(300) * 3 * dx], 1)
    i, j = np.meshgrid(np.arange(2000), np.arange(12), indexing="xy")
    blk = np.stack([i.ravel() * dx, 1.0 + j.ravel() * dx], 1)
    pts = np.concatenate([col, blk]) + rng.uniform(-0.01, 0.01, (300 + blk.shape[0], 2)) * dx
    return _lattice_2d(pts, dx)


def _lean_duct_3d():
    c = cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4, width=12 * 7.9e-4, layers=3,
                      jitter=0.01)
    c.params.periodic[0] = 0
    c.params.heat_art = 0
    c.params.heat_ext = 0
    return cases.perturbed(c, seed=31, dv=0.02)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 0), (2, 1, 256, 0), (3, 1, 128, 0),
                                    (3, 1, 256, 10)])
def test_staged_equals_global_dam_break(tuning):
    c = cases.perturbed(cases.dam_break(dx=0.01), seed=41, dv=0.05)
    a = _run(c, tuning, 6, True)
    b = _run(c, tuning, 6, False)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), (tuning, f)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 0), (3, 1, 256, 0)])
def test_staged_equals_global_with_capacity_fallback(tuning):
    c = _sparse_below_dense()
    a = _run(c, tuning, 3, True)
    b = _run(c, tuning, 3, False)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), (tuning, f)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 0), (2, 1, 128, 0), (3, 1, 128, 0)])
def test_staged_equals_global_3d(tuning):
    c = _lean_duct_3d()
    a = _run(c, tuning, 4, True)
    b = _run(c, tuning, 4, False)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), (tuning, f)


def test_staged_one_step_parity_fallback_layout(O):
    c = history_state(O, _sparse_below_dense(), steps=1)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(3, 1, 128, 0)
        errs, _, _ = step_errors(O, ctx, c, its=2)
    for f in FIELDS:
        assert errs[f] <= 1e-5, (f, errs[f])
