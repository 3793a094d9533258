"""Neighbour lists of a lazily sorting context.

With a sort skin, the iterations that sort build, for every particle, the list
of candidates within h_i + h_j + skin (k_build_list); until the next sort the
passes read the lists instead of walking the cells. A 2D list holds its near
entries (q < 1.5 at the sort) first and its far ones after them. A listed
particle's density pass evaluates each near entry in float-float and each far
one in FP32 with a float-float prefactor, as it reads it (the kernel is zero
beyond its support); its force pass takes the pair forces of the entries that
pass the pair test. The neighbour sets are the cell walk's; the summation
order and (2D) the far pairs' arithmetic differ, so the gates are the oracle
for one iteration and the cell walk to 1e-5 over many. Particles whose list
would exceed its capacity walk their cells (a compressed clump).
"""
import os

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS, history_state, rel_err, step_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def _run(c, tuning, its0, steps, lists):
    old = os.environ.get("ARMANDO_NEIGHBOUR_LISTS")
    os.environ["ARMANDO_NEIGHBOUR_LISTS"] = "1" if lists else "0"
    try:
        out = c.copy()
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(*tuning)
            ctx.integrate(out, c.dt, its0, steps)
            sorts = ctx.stats().sorts_done
        return out, sorts
    finally:
        if old is None:
            del os.environ["ARMANDO_NEIGHBOUR_LISTS"]
        else:
            os.environ["ARMANDO_NEIGHBOUR_LISTS"] = old


@pytest.mark.parametrize("tuning", [(1, 1, 128, 10), (3, 1, 256, 10), (2, 1, 128, 40)])
def test_lists_20_iterations_within_conditioning_2d(O, tuning):
    """20 iterations on the lists (a few sort), against 20 FP64 oracle
    iterations: within 20 times the oracle's own divergence when its FP32
    inputs move by one ulp (the trajectory's conditioning; the perturbed dam
    break amplifies rounding), or 1e-5. The cell walk is held to the same."""
    c = cases.perturbed(cases.dam_break(dx=0.01), seed=61, dv=0.2)
    a, sa = _run(c, tuning, 1, 20, True)
    b, sb = _run(c, tuning, 1, 20, False)
    assert 1 <= sa < 20
    rng = np.random.default_rng(69)
    twin = c.copy()
    fl = np.repeat(c.itype > 0, 2)
    bump = np.where(rng.random(c.x.size) < 0.5, np.inf, -np.inf).astype(np.float32)
    twin.x = np.where(fl, np.nextafter(c.x, bump), c.x).astype(np.float32)
    ref, pert = O.State(c), O.State(twin)
    O.integrate_gather(ref, 1, 20, c.dt)
    O.integrate_gather(pert, 1, 20, c.dt)
    for f in FIELDS:
        cond = rel_err(getattr(pert, f), getattr(ref, f))
        ea, eb = rel_err(getattr(a, f), getattr(ref, f)), rel_err(getattr(b, f), getattr(ref, f))
        print(tuning, f, f"lists {ea:.1e} cell walk {eb:.1e} one-ulp twin {cond:.1e}")
        assert ea <= max(20.0 * cond, 1e-5), (tuning, f, ea, cond)
        assert eb <= max(20.0 * cond, 1e-5), (tuning, f, eb, cond)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 10), (3, 1, 256, 10)])
def test_listed_iteration_parity_2d(O, tuning):
    """One iteration on the lists (it does not sort) against one FP64 oracle
    iteration from the same FP32 state, the output of a first one-step call."""
    c = history_state(O, cases.perturbed(cases.dam_break(dx=0.01), seed=68, dv=0.05), steps=2)
    mid = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(*tuning)
        ctx.step(mid, c.dt, 3)
    ref = O.State(mid)
    O.step(ref, 4, c.dt)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(*tuning)
        ctx.integrate(got, c.dt, 3, 2)
        assert ctx.stats().sorts_done == 1
    for f in FIELDS:
        assert rel_err(getattr(got, f), getattr(ref, f)) <= 1e-5, (tuning, f)


@pytest.mark.parametrize("tuning", [(1, 1, 128, 10), (3, 1, 256, 10)])
def test_listed_iteration_parity_2d_variable_h(O, tuning):
    """Lists over fluid particles whose h differ (seeded, +-10%): the near
    entries' float-float path and the far entries' FP32 path with the pair's
    own h = (h_i + h_j)/2 and prefactor. One iteration on the lists (it does not
    sort) against one FP64 oracle iteration from the same FP32 state."""
    c0 = cases.perturbed(cases.dam_break(dx=0.01), seed=72, dv=0.05)
    rng = np.random.default_rng(73)
    fl = c0.itype > 0
    c0.h = np.where(fl, c0.h * (1.0 + 0.1 * (2.0 * rng.random(c0.n) - 1.0)),
                    c0.h).astype(np.float32)
    c = history_state(O, c0, steps=2)
    mid = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(*tuning)
        ctx.step(mid, c.dt, 3)
    ref = O.State(mid)
    O.step(ref, 4, c.dt)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(*tuning)
        ctx.integrate(got, c.dt, 3, 2)
        assert ctx.stats().sorts_done == 1
    for f in FIELDS:
        err = rel_err(getattr(got, f), getattr(ref, f))
        print(tuning, "variable h", f, f"{err:.2e}")
        assert err <= 1e-5, (tuning, f, err)


def _with_extra_copies(c, idx, offsets):
    """c with copies of particles idx added at each offset (in units of the
    lattice spacing): a locally two- or three-fold denser patch."""
    dx = float(c.h[0]) / 1.3
    out = c.copy()
    x = c.x.reshape(-1, 2)
    add_x = [x[idx] + np.float32(o * dx) for o in offsets]
    out.x = np.concatenate([x] + add_x).ravel().astype(np.float32)
    for f in ("v", "dvdt"):
        a = getattr(c, f).reshape(-1, 2)
        setattr(out, f, np.concatenate([a] + [a[idx]] * len(offsets)).ravel())
    for f in ("mass", "rho", "p", "u", "h", "itype", "dudt"):
        a = getattr(c, f)
        setattr(out, f, np.concatenate([a] + [a[idx]] * len(offsets)))
    return out


def test_lists_with_overflow_patch_2d(O):
    """A patch at three times the lattice density (two shifted copies of 100
    particles): lists there exceed their capacity and those particles walk
    their cells, beside listed ones. One iteration (it sorts and uses the
    lists) against the FP64 oracle, and against the cell walk."""
    c = cases.perturbed(cases.dam_break(dx=0.01), seed=62, dv=0.05)
    fl = np.flatnonzero(c.itype > 0)
    x = c.x.reshape(-1, 2)
    centre = x[fl[len(fl) // 2]]
    patch = fl[np.argsort(np.linalg.norm(x[fl] - centre, axis=1))[:100]]
    c = _with_extra_copies(c, patch, [0.33, 0.66])
    a, _ = _run(c, (1, 1, 128, 40), 1, 1, True)
    b, _ = _run(c, (1, 1, 128, 40), 1, 1, False)
    ref = O.State(c)
    O.step(ref, 1, c.dt)
    for f in FIELDS:
        assert rel_err(getattr(a, f), getattr(ref, f)) <= 1e-5, f
        assert rel_err(getattr(a, f), getattr(b, f)) <= 1e-5, f


def test_lists_3d_channel_against_oracle(O):
    c = history_state(O, cases.perturbed(
        cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4, width=12 * 7.9e-4, layers=3,
                      jitter=0.01), seed=63, dv=0.02, du=50.0), steps=2)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(2, 1, 128, 20)
        errs, _, _ = step_errors(O, ctx, c, its=3)
    for f in FIELDS:
        assert errs[f] <= 1e-5, (f, errs[f])


def test_lists_3d_many_iterations_match_cell_walk_to_rounding():
    """20 iterations of the 3D channel with lists and with the cell walk: the
    same neighbour sets, different summation rounds; the two stay within 1e-5."""
    c = cases.perturbed(cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4, width=12 * 7.9e-4,
                                      layers=3, jitter=0.01), seed=64, dv=0.02, du=50.0)
    a, _ = _run(c, (1, 1, 128, 20), 1, 20, True)
    b, _ = _run(c, (1, 1, 128, 20), 1, 20, False)
    for f in FIELDS:
        assert rel_err(getattr(a, f), getattr(b, f)) <= 1e-5, f
