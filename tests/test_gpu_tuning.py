"""Tuned neighbour passes (armando_set_tuning / armando_autotune) vs the FP64 oracle.

Every candidate tuning (grid reach 1-3, 1/2/4 threads per particle, 128/256
threads per CTA) must find link_list's exact neighbour sets and pass the
one-step gate TOL_STEP = 1e-5 (normwise relative, every output) that the
default tuning passes; the tuning may change only the rounding of the sums.
"""
import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS, history_state, step_errors

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-5
CANDIDATES = [(r, t, b, 0) for r in (1, 2, 3) for t in (1, 2, 4) for b in (128, 256)]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def wide_h(case, factor=1.6):
    """Smoothing length x factor (masses rescaled to the lattice kernel sum):
    more candidates than the neighbour masks hold (2D: 128 bits)."""
    c = case.copy()
    r0 = float(c.h[0] / c.meta["dx"])
    c.h = (c.h * factor).astype(np.float32)
    c.mass = (c.mass * cases.lattice_kernel_sum(c.dim, r0)
              / cases.lattice_kernel_sum(c.dim, r0 * factor)).astype(np.float32)
    return c


def tuning_cases():
    return {
        "dambreak": cases.perturbed(cases.dam_break(dx=0.02), seed=41, dv=0.05),
        "channel3d": cases.perturbed(
            cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4, width=12 * 7.9e-4, layers=3,
                          jitter=0.01), seed=42, dv=0.02, du=50.0),
        "dambreak_wide_h": wide_h(cases.perturbed(cases.dam_break(dx=0.03), seed=43, dv=0.05)),
    }


@pytest.fixture(scope="module")
def refs(O):
    """Per case: the FP32 input state after two oracle iterations and the
    oracle's third iteration from it."""
    out = {}
    for name, c in tuning_cases().items():
        inp = history_state(O, c, steps=2)
        ref = O.State(inp)
        O.step(ref, 3, inp.dt)
        out[name] = (inp, ref)
    return out


def oracle_rows(O, c):
    pi, pj, _, _ = O.link_list(c.x, c.h, c.dim, fp32=True, params=c.params)
    rows = [[] for _ in range(c.n)]
    for a, b in zip(pi.tolist(), pj.tolist()):
        rows[a].append(b)
        rows[b].append(a)
    offs = np.zeros(c.n + 1, np.int64)
    offs[1:] = np.cumsum([len(r) for r in rows])
    return offs, np.array([k for r in rows for k in sorted(r)], np.int32)


@pytest.mark.parametrize("reach", [1, 2, 3])
@pytest.mark.parametrize("name", ["dambreak", "channel3d", "dambreak_wide_h"])
def test_neighbour_sets_every_reach(O, name, reach):
    c = tuning_cases()[name]
    ref_offs, ref_nbr = oracle_rows(O, c)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(reach=reach)
        offs, nbr = ctx.neighbours(c.x, c.h)
        cid = ctx.cell_ids(c.x, c.h)  # link_list's cells whatever the reach
    _, _, ref_cid, _ = O.link_list(c.x, c.h, c.dim, fp32=True, params=c.params)
    assert np.array_equal(offs, ref_offs)
    assert np.array_equal(nbr, ref_nbr)
    assert np.array_equal(cid.astype(np.int64), ref_cid)


@pytest.mark.parametrize("tuning", CANDIDATES, ids=lambda t: "r%d_t%d_b%d_s%d" % t)
@pytest.mark.parametrize("name", ["dambreak", "channel3d", "dambreak_wide_h"])
def test_one_step_parity_every_tuning(refs, name, tuning):
    inp, ref = refs[name]
    got = inp.copy()
    with ag.Context(inp.params, inp.n_fluid, inp.n_wall) as ctx:
        ctx.set_tuning(*tuning)
        ctx.step(got, inp.dt, 3)
        assert ctx.tuning().as_tuple() == tuning
    for f in FIELDS:
        a = np.asarray(getattr(got, f), np.float64)
        b = np.asarray(getattr(ref, f), np.float64)
        err = np.abs(a - b).max() / np.abs(b).max() if np.abs(b).max() > 0 else np.abs(a).max()
        assert err <= TOL_STEP, (f, err)


def test_tunings_agree_over_many_steps(O):
    """Same trajectory under different tunings up to rounding, 50 iterations:
    tuned vs default within 20x the FP64 oracle's own change when its FP32
    inputs move by one ulp (the trajectory's conditioning), or 1e-5."""
    c = cases.perturbed(cases.dam_break(dx=0.02), seed=44, dv=0.05)
    rng = np.random.default_rng(48)
    c2 = c.copy()
    bump = np.where(rng.random(c.x.size) < 0.5, np.inf, -np.inf).astype(np.float32)
    c2.x = np.where(np.repeat(c.itype > 0, c.dim), np.nextafter(c.x, bump), c.x).astype(np.float32)
    ref, pert = O.State(c), O.State(c2)
    O.integrate_gather(ref, 1, 50, c.dt)
    O.integrate_gather(pert, 1, 50, c.dt)
    runs = {}
    for t in [(1, 1, 128, 0), (2, 2, 128, 0), (3, 4, 256, 0), (2, 1, 256, 0), (1, 1, 128, 20),
              (2, 1, 128, 40)]:
        s = c.copy()
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(*t)
            ctx.integrate(s, c.dt, 1, 50)
        runs[t] = s
    base = runs[(1, 1, 128, 0)]
    for t, s in runs.items():
        for f in FIELDS:
            b = np.asarray(getattr(ref, f), np.float64)
            scale = np.abs(b).max()
            cond = np.abs(np.asarray(getattr(pert, f), np.float64) - b).max() / scale
            diff = np.abs(getattr(s, f).astype(np.float64)
                          - getattr(base, f).astype(np.float64)).max() / scale
            assert diff <= max(20.0 * cond, 1e-5), (t, f, diff, cond)


def test_autotune_picks_a_candidate_and_leaves_inputs(O):
    c = cases.perturbed(cases.dam_break(dx=0.02), seed=45, dv=0.05)
    before = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        best, table = ctx.autotune(c, c.dt, 1, steps_per_trial=3)
        for f in FIELDS + ("mass", "h", "itype"):
            assert np.array_equal(getattr(c, f), getattr(before, f)), f
        assert ctx.tuning().as_tuple() == best
        assert best[:3] + (0,) in CANDIDATES and best[3] in (0, 10, 20, 40)
        assert set(CANDIDATES) <= set(table) and len(table) == 27
        assert all(v > 0 for v in table.values())
        assert table[best] == min(table.values())
        errs, _, _ = step_errors(O, ctx, c, its=1)
    for f in FIELDS:
        assert errs[f] <= TOL_STEP, (f, errs[f])


def test_set_tuning_rejects_bad_values():
    c = cases.dam_break(dx=0.05)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        for bad in [(0, 1, 128), (4, 1, 128), (1, 3, 128), (1, 1, 96), (1, 1, 128, -1),
                    (1, 1, 128, 101)]:
            with pytest.raises(ag.ArmandoError) as e:
                ctx.set_tuning(*bad)
            assert e.value.status == ag._abi.ERR_INVALID_ARG
        assert ctx.tuning().as_tuple() == (1, 1, 128, 0)
    insts = [cases.dam_break(dx=0.05), cases.cavity(n_side=12)]
    with ag.Batch([k.params for k in insts], [k.n_fluid for k in insts],
                  [k.n_wall for k in insts]) as b:
        b.set_tuning(reach=2)
        with pytest.raises(ag.ArmandoError) as e:
            b.set_tuning(reach=1, threads_per_particle=2)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED
        with pytest.raises(ag.ArmandoError) as e:
            b.set_tuning(reach=1, skin=20)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED


def test_batch_with_reach_matches_instances_alone():
    insts = [cases.perturbed(cases.dam_break(dx=0.04), seed=46, dv=0.05),
             cases.perturbed(cases.cavity(n_side=16), seed=47, dv=1e-4)]
    arrays, offs = cases.pack(insts)
    dts = [k.dt for k in insts]
    with ag.Batch([k.params for k in insts], [k.n_fluid for k in insts],
                  [k.n_wall for k in insts]) as b:
        b.set_tuning(reach=2)
        b.integrate_batch(arrays, dts, 1, 5)
    outs = cases.unpack(arrays, offs, insts)
    for k, c in enumerate(insts):
        alone = c.copy()
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(reach=2)
            ctx.integrate(alone, c.dt, 1, 5)
        for f in FIELDS:
            assert np.array_equal(getattr(outs[k], f), getattr(alone, f)), (k, f)
