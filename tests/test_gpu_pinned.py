"""Host-memory contexts with page-locked caller arrays: the copy kernels read
and write the caller's arrays across the host link (no staging copies). The
results must be bit-identical to the staged path taken for pageable arrays."""
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
    return cases.perturbed(cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4,
                                         width=12 * 7.9e-4, layers=3, jitter=0.01),
                           seed=62, dv=0.02, du=50.0)


@pytest.mark.parametrize("name", ["dambreak", "channel3d"])
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
