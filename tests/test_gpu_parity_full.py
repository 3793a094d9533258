"""GPU step vs the FP64 oracle at the benchmark configurations' own sizes.

* 2D dam break, 2,030,018 particles (dx = 1 mm, the throughput workload) and
  3D heated channel, 8,781,696 particles: two oracle iterations give the
  state, rounded to FP32; then one GPU step and one FP64 step from it, per
  output field within 1e-5 normwise (max|gpu - oracle| / max|oracle|), at
  link_list's grid and at the tunings the benchmark runs.
* The benchmark's timed path, armando_integrate with a 10% sort skin (the
  step graph sorts only when a particle has moved half the skin): 20
  iterations against the oracle, bounded like the small drift tests by 20x
  the oracle's own divergence under a one-ulp change of its inputs.
The oracle here is the threaded FP64 gather form (all host cores).
"""
import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS, rel_err

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def _fp32_history(O, case, steps):
    st = O.State(case)
    O.integrate_gather(st, 1, steps, case.dt)
    c = case.copy()
    for f in FIELDS:
        setattr(c, f, getattr(st, f).astype(np.float32))
    return c


def _one_step(O, c, its, tunings):
    ref = O.State(c)
    O.integrate_gather(ref, its, 1, c.dt)
    out = {}
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        for t in tunings:
            ctx.set_tuning(*t)
            got = c.copy()
            ctx.step(got, c.dt, its)
            out[t] = {f: rel_err(getattr(got, f), getattr(ref, f)) for f in FIELDS}
            print(c.name, c.n, t, {f: f"{e:.2e}" for f, e in out[t].items()})
    return out


@pytest.fixture(scope="module")
def dam_break_2m(O):
    c = cases.dam_break()
    assert c.n == 2_030_018
    return _fp32_history(O, c, 2)


def test_dam_break_2m_one_step_parity(O, dam_break_2m):
    errs = _one_step(O, dam_break_2m, 3, [(1, 1, 128, 0), (3, 1, 256, 0), (3, 1, 128, 10),
                                          (2, 1, 256, 0)])
    for t, e in errs.items():
        for f in FIELDS:
            assert e[f] <= TOL_STEP, (t, f, e[f])


def test_channel_8m_one_step_parity(O):
    c = _fp32_history(O, cases.channel(), 2)
    assert c.n == 8_781_696
    errs = _one_step(O, c, 3, [(1, 1, 128, 0), (3, 1, 128, 10)])
    for t, e in errs.items():
        for f in FIELDS:
            assert e[f] <= TOL_STEP, (t, f, e[f])


def test_dam_break_2m_skin_path_20_iterations(O, dam_break_2m):
    """The benchmark's lazily sorting integrate (3, 1, 256, skin 10%) over 20
    iterations from the FP32 state, against the FP64 oracle from the same
    state and from its one-ulp twin."""
    c = dam_break_2m
    rng = np.random.default_rng(52)
    twin = c.copy()
    fl = np.repeat(c.itype > 0, c.dim)
    bump = np.where(rng.random(c.x.size) < 0.5, np.inf, -np.inf).astype(np.float32)
    twin.x = np.where(fl, np.nextafter(c.x, bump), c.x).astype(np.float32)
    ref, pert = O.State(c), O.State(twin)
    O.integrate_gather(ref, 3, 20, c.dt)
    O.integrate_gather(pert, 3, 20, c.dt)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(3, 1, 256, 10)
        ctx.integrate(got, c.dt, 3, 20)
        sorts = ctx.stats().sorts_done
    assert sorts >= 1
    for f in FIELDS:
        g = rel_err(getattr(got, f), getattr(ref, f))
        i = rel_err(getattr(pert, f), getattr(ref, f))
        print("skin path, 20 iterations", f, f"gpu {g:.2e} twin {i:.2e}")
        assert np.isfinite(g) and g <= max(20.0 * i, TOL_STEP), (f, g, i)
