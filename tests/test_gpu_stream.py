"""Stream order of the device-memory calls.

armando_step / armando_integrate with ARMANDO_MEM_DEVICE enqueue their work on
the context's stream and return; their device status is reported by
armando_sync. armando_set_stream moves the context onto a caller's stream.
Results are compared bit for bit with the synchronous host-memory path.
"""
import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def _host_run(c, calls):
    out = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        for its0, steps in calls:
            ctx.integrate(out, c.dt, its0, steps)
    return out


def test_device_call_returns_before_its_work_completes():
    import torch

    c = cases.dam_break(dx=0.002)  # ~0.5 M particles: tens of ms of GPU work below
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in c.arrays().items()}
    torch.cuda.synchronize()
    with ag.Context(c.params, c.n_fluid, c.n_wall, mem=ag.MEM_DEVICE) as ctx:
        ctx.integrate(dev, c.dt, 1, 2)  # the first call plans the grid and blocks
        s = torch.cuda.ExternalStream(ctx.stream_handle())
        ctx.integrate(dev, c.dt, 3, 60, wait=False)
        busy = not s.query()
        ctx.sync()
        assert s.query()
    assert busy, "the device-memory call waited for its work"
    host = _host_run(c, [(1, 2), (3, 60)])
    for f in FIELDS:
        assert np.array_equal(dev[f].cpu().numpy(), getattr(host, f)), f


def test_device_status_is_reported_by_sync_once():
    import torch

    c = cases.dam_break(dx=0.02)
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in c.arrays().items()}
    with ag.Context(c.params, c.n_fluid, c.n_wall, mem=ag.MEM_DEVICE) as ctx:
        ctx.integrate(dev, c.dt, 1, 2)
        dev["rho"].fill_(float("nan"))
        ctx.integrate(dev, c.dt, 3, 2, wait=False)  # enqueued: no status yet
        with pytest.raises(ag.ArmandoError) as e:
            ctx.sync()
        assert e.value.status == ag._abi.ERR_NONFINITE
        ctx.sync()  # reported once; the context starts clean
        good = {k: torch.from_numpy(v.copy()).cuda() for k, v in c.arrays().items()}
        ctx.integrate(good, c.dt, 1, 2)


def test_context_on_a_caller_stream():
    import torch

    c = cases.dam_break(dx=0.01)
    s = torch.cuda.Stream()
    with ag.Context(c.params, c.n_fluid, c.n_wall, mem=ag.MEM_DEVICE) as ctx:
        ctx.set_stream(s.cuda_stream)
        assert ctx.stream_handle() == s.cuda_stream
        with torch.cuda.stream(s):
            # inputs produced on the caller's stream, outputs consumed there
            dev = {k: torch.from_numpy(v.copy()).pin_memory().to("cuda", non_blocking=True)
                   for k, v in c.arrays().items()}
            ctx.integrate(dev, c.dt, 1, 5, wait=False)
            ctx.integrate(dev, c.dt, 6, 5, wait=False)
            out = {f: dev[f].to("cpu", non_blocking=False) for f in FIELDS}
        ctx.sync()
        ctx.set_stream(0)
        assert ctx.stream_handle() != s.cuda_stream
    host = _host_run(c, [(1, 5), (6, 5)])
    for f in FIELDS:
        assert np.array_equal(out[f].numpy(), getattr(host, f)), f
