"""The fused predictor of a lazily sorting context.

On the iterations that do not sort, the density and force passes read the
integrated state in place (the slots keep the last sort's order), apply the
leapfrog predictor (time_integration.f:136-154) on load, and the force pass
writes the next state into a second buffer; the reorder copy runs only on the
iterations that sort. Same operations, same order: the results are the same
bits as with a reorder copy every iteration (ARMANDO_FUSED_PREDICTOR=0), over
several calls (the current buffer alternates), the first iteration's half
kick, 2D and 3D, and device-memory calls.
"""
import os

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS, history_state, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


class _Env:
    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update(self.kv)

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def _run(c, tuning, calls, fused):
    with _Env(ARMANDO_FUSED_PREDICTOR="1" if fused else "0"):
        out = c.copy()
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(*tuning)
            for its0, steps in calls:
                ctx.integrate(out, c.dt, its0, steps)
            sorts = ctx.stats().sorts_done
    return out, sorts


def _lean_duct_3d():
    c = cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4, width=12 * 7.9e-4, layers=3,
                      jitter=0.01)
    c.params.periodic[0] = 0
    c.params.heat_artificial = 0
    c.params.heat_external = 0
    return cases.perturbed(c, seed=33, dv=0.05)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 10), (3, 1, 256, 10), (2, 1, 128, 40)])
def test_fused_equals_reorder_copy_2d(tuning):
    c = cases.perturbed(cases.dam_break(dx=0.01), seed=65, dv=0.2)
    calls = [(1, 17), (18, 6), (24, 23)]  # odd lengths: each call starts on another buffer
    a, sa = _run(c, tuning, calls, True)
    b, sb = _run(c, tuning, calls, False)
    assert sa == sb and 3 <= sa < 46
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), (tuning, f)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 20), (3, 1, 128, 20)])
def test_fused_equals_reorder_copy_3d(tuning):
    c = _lean_duct_3d()
    calls = [(1, 9), (10, 12)]
    a, sa = _run(c, tuning, calls, True)
    b, sb = _run(c, tuning, calls, False)
    assert sa == sb and sa < 21
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), (tuning, f)


def test_fused_device_memory_calls():
    import torch

    c = cases.perturbed(cases.dam_break(dx=0.01), seed=66, dv=0.1)
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in c.arrays().items()}
    with ag.Context(c.params, c.n_fluid, c.n_wall, mem=ag.MEM_DEVICE) as ctx:
        ctx.set_tuning(3, 1, 256, 10)
        ctx.integrate(dev, c.dt, 1, 7, wait=False)
        ctx.integrate(dev, c.dt, 8, 8, wait=False)
        ctx.sync()
    ref, _ = _run(c, (3, 1, 256, 10), [(1, 7), (8, 8)], False)
    for f in FIELDS:
        assert np.array_equal(dev[f].cpu().numpy(), getattr(ref, f)), f


def test_fused_iteration_parity(O):
    """An iteration that does not sort, on the fused path, against one FP64
    oracle iteration from the same FP32 state. A call of two iterations sorts
    on the first only; the state after the first is the output of a one-step
    call (integrate equals repeated steps bit for bit), and the oracle steps
    from it."""
    c = history_state(O, cases.perturbed(cases.dam_break(dx=0.01), seed=67, dv=0.05), steps=2)
    mid = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(3, 1, 256, 10)
        ctx.step(mid, c.dt, 3)
    ref = O.State(mid)
    O.step(ref, 4, c.dt)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(3, 1, 256, 10)
        ctx.integrate(got, c.dt, 3, 2)
        assert ctx.stats().sorts_done == 1
    for f in FIELDS:
        err = rel_err(getattr(got, f), getattr(ref, f))
        assert err <= 1e-5, (f, err)
