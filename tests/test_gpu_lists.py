"""Neighbour lists of a lazily sorting context.

With a sort skin, the iterations that sort build, for every particle, the list
of candidates within h_i + h_j + skin (k_build_list); until the next sort the
passes read the lists instead of walking the cells, and the neighbour bits of
the density pass index list entries. The lists hold the candidates in the cell
walk's order, so in 2D (fewer than one round of near and far pairs) the
results are the same bits as walking the cells (ARMANDO_NEIGHBOUR_LISTS=0); in
3D the summation rounds differ and the gate is the oracle. Particles whose
list would exceed its capacity walk their cells (a compressed clump).
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
def test_lists_equal_cell_walk_2d(tuning):
    c = cases.perturbed(cases.dam_break(dx=0.01), seed=61, dv=0.2)
    a, sa = _run(c, tuning, 1, 40, True)
    b, sb = _run(c, tuning, 1, 40, False)
    assert sa == sb and 1 <= sa < 40
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), (tuning, f)


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


def test_lists_with_overflow_patch_2d():
    """A patch at three times the lattice density (two shifted copies of 100
    particles): lists there exceed their capacity and those particles walk
    their cells, beside listed ones; one iteration (it sorts and uses the
    lists), against the cell walk bit for bit."""
    c = cases.perturbed(cases.dam_break(dx=0.01), seed=62, dv=0.05)
    fl = np.flatnonzero(c.itype > 0)
    x = c.x.reshape(-1, 2)
    centre = x[fl[len(fl) // 2]]
    patch = fl[np.argsort(np.linalg.norm(x[fl] - centre, axis=1))[:100]]
    c = _with_extra_copies(c, patch, [0.33, 0.66])
    a, _ = _run(c, (1, 1, 128, 40), 1, 1, True)
    b, _ = _run(c, (1, 1, 128, 40), 1, 1, False)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


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
