"""Host-memory contexts with page-locked caller arrays: the copy kernels read
and write the caller's arrays across the host link (no staging copies); a
one-iteration call (armando_step without a sort skin) loads the inputs other
than the positions on a second stream while the sort runs, and writes the
output density and pressure back while the force pass runs. The results must
be bit-identical to the staged path taken for pageable arrays."""
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


def pinned_copy(case, only=None):
    """A copy of the case whose arrays (or those named in `only`) are page-locked."""
    import torch

    c = case.copy()
    for f in ("x", "v", "mass", "rho", "p", "u", "h", "itype", "dvdt", "dudt"):
        if only is not None and f not in only:
            continue
        a = getattr(c, f)
        t = torch.empty(a.shape, dtype=torch.from_numpy(a).dtype, pin_memory=True)
        t.copy_(torch.from_numpy(a))
        setattr(c, f, t.numpy())
    return c


def small(name):
    if name == "dambreak":
        return cases.perturbed(cases.dam_break(dx=0.02), seed=61, dv=0.05)
    if name == "cavity":  # physical viscosity: the shear pass between the two
        return cases.perturbed(cases.cavity(n_side=24), seed=65, dv=1e-4)
    return cases.perturbed(cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4,
                                         width=12 * 7.9e-4, layers=3, jitter=0.01),
                           seed=62, dv=0.02, du=50.0)


@pytest.mark.parametrize("name", ["dambreak", "channel3d", "cavity"])
@pytest.mark.parametrize("only", [None, ("x", "v", "rho")], ids=["all", "some"])
def test_pinned_host_arrays_match_pageable(name, only):
    c = small(name)
    a = c.copy()
    b = pinned_copy(c, only)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(a, c.dt, 1, 4)
        ctx.step(a, c.dt, 5)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(b, c.dt, 1, 4)
        ctx.step(b, c.dt, 5)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), np.asarray(getattr(b, f))), f


def test_pinned_batch_matches_pageable():
    insts = [cases.perturbed(cases.dam_break(dx=0.04), seed=63, dv=0.05),
             cases.perturbed(cases.cavity(n_side=16), seed=64, dv=1e-4)]
    arrays, offs = cases.pack(insts)
    import torch

    pinned = {}
    for k, v in arrays.items():
        t = torch.empty(v.shape, dtype=torch.from_numpy(v).dtype, pin_memory=True)
        t.copy_(torch.from_numpy(v))
        pinned[k] = t.numpy()
    plain = {k: v.copy() for k, v in arrays.items()}
    dts = [k.dt for k in insts]
    for arr in (plain, pinned):
        with ag.Batch([k.params for k in insts], [k.n_fluid for k in insts],
                      [k.n_wall for k in insts]) as b:
            b.integrate_batch(arr, dts, 1, 3)
    for k in plain:
        assert np.array_equal(plain[k], pinned[k]), k


@pytest.mark.parametrize("name", ["dambreak", "channel3d"])
def test_pinned_step_calls_match_pageable(name):
    """Consecutive one-iteration calls (each loads, steps and stores) on
    page-locked arrays against pageable ones."""
    c = small(name)
    a = c.copy()
    b = pinned_copy(c)
    for arr in (a, b):
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            for its in range(1, 7):
                ctx.step(arr, c.dt, its)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), np.asarray(getattr(b, f))), f


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("name", ["dambreak", "channel3d"])
def test_fluid_input_density_and_pressure_unused(name, pinned):
    """With summation density the step recomputes the fluid particles'
    density and pressure: their input values (NaN here) are not read; the
    walls' are."""
    c = small(name)
    assert c.params.density_form == 0 and c.params.scheme == 0
    bad = c.copy()
    fl = bad.itype > 0
    bad.rho = np.where(fl, np.float32(np.nan), bad.rho).astype(np.float32)
    bad.p = np.where(fl, np.float32(np.nan), bad.p).astype(np.float32)
    a = pinned_copy(c) if pinned else c.copy()
    b = pinned_copy(bad) if pinned else bad.copy()
    for arr in (a, b):
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.step(arr, c.dt, 1)
            ctx.step(arr, c.dt, 2)
    for f in FIELDS:
        assert np.array_equal(np.asarray(getattr(a, f)), np.asarray(getattr(b, f))), f


def test_pinned_step_calls_on_a_caller_stream():
    """The overlapped one-iteration calls with the context on a caller's
    stream: the second stream's copies are ordered by events after the
    caller's earlier work and joined back before the call returns."""
    import torch

    c = small("dambreak")
    a = pinned_copy(c)
    b = pinned_copy(c)
    s = torch.cuda.Stream()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        for its in range(1, 5):
            ctx.step(a, c.dt, its)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_stream(s.cuda_stream)
        for its in range(1, 5):
            ctx.step(b, c.dt, its)
        ctx.set_stream(0)
    for f in FIELDS:
        assert np.array_equal(np.asarray(getattr(a, f)), np.asarray(getattr(b, f))), f
