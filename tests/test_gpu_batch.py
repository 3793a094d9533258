"""Batched multi-instance contexts (armando_batch_create / _integrate).

A batch advances every instance with the kernels of one system plus per-instance
grids and parameters, so each instance must come out bit-identical to the same
instance run alone, and within the one-step tolerance of the FP64 oracle.
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


def _instances_2d():
    a = cases.perturbed(cases.dam_break(dx=0.03), seed=41, dv=0.05)
    b = cases.cavity(n_side=24, length=1.0, lid_u=1.0)
    b.params.c0, b.params.visc, b.params.visc_artificial = 30.0, 0, 1
    b.params.av_alpha, b.params.av_beta = 0.02, 0.0
    b.dt = 0.2 * float(b.h[0]) / 30.0
    c = cases.dam_break(dx=0.04, col_w=0.6, col_h=1.5, tank_w=2.0, tank_h=2.0, seed=43,
                        alpha=0.04, c0=40.0)
    d = cases.cavity(n_side=12)  # physical viscosity instance
    return [a, b, c, d]


def _run_single(c, its0, steps):
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(got, c.dt, its0, steps)
    return got


def _run_batch(insts, its0, steps):
    arrays, offs = cases.pack(insts)
    with ag.Batch([c.params for c in insts], [c.n_fluid for c in insts],
                  [c.n_wall for c in insts]) as b:
        b.integrate_batch(arrays, [c.dt for c in insts], its0, steps)
        assert b.stats().gpu_launches > 0
    return cases.unpack(arrays, offs, insts)


def _packed_ok(insts):
    # the batch assumes each instance's fluid/wall counts describe its slice
    for c in insts:
        assert c.n_fluid + c.n_wall == c.n


@pytest.mark.parametrize("its0,steps", [(1, 1), (1, 6)])
def test_batch_equals_instances_run_alone_2d(its0, steps):
    insts = _instances_2d()
    _packed_ok(insts)
    got = _run_batch(insts, its0, steps)
    for c, g in zip(insts, got):
        ref = _run_single(c, its0, steps)
        for f in FIELDS:
            assert np.array_equal(getattr(g, f), getattr(ref, f)), (c.name, f)


def test_batch_equals_instances_run_alone_3d_periodic():
    insts = []
    for k, (nx, nyz) in enumerate([(24, 8), (30, 10)]):
        c = cases.perturbed(
            cases.channel(n_x=nx, n_yz=nyz, length=nx * 7.9e-4, width=nyz * 7.9e-4, layers=3,
                          jitter=0.01, seed=50 + k), seed=60 + k, dv=0.02, du=30.0)
        insts.append(c)
    got = _run_batch(insts, 1, 4)
    for c, g in zip(insts, got):
        ref = _run_single(c, 1, 4)
        for f in FIELDS:
            assert np.array_equal(getattr(g, f), getattr(ref, f)), (c.name, f)


def test_sweep_instances_match_oracle(O):
    insts = cases.sweep(n_instances=6, seed=44, n_min=400, n_max=3000)
    arrays, offs = cases.pack(insts)
    with ag.Batch([c.params for c in insts], [c.n_fluid for c in insts],
                  [c.n_wall for c in insts]) as b:
        b.integrate_batch(arrays, [c.dt for c in insts], 1, 1)
    got = cases.unpack(arrays, offs, insts)
    for c, g in zip(insts, got):
        ref = O.State(c)
        O.step(ref, 1, c.dt)
        for f in FIELDS:
            e = rel_err(getattr(g, f), getattr(ref, f))
            assert e <= TOL_STEP, (c.name, f, e)


def test_full_sweep_subset_matches_oracle(O):
    """The 512-instance benchmark sweep (22.9 M particles) in one batch: after
    one batched iteration, a second from those FP32 states; the smallest 64
    instances and 16 size-stratified others each within TOL_STEP of the FP64
    oracle's iteration from the same inputs, on every output."""
    insts = cases.sweep()
    subset = cases.sweep_subset(insts)
    assert len(subset) == 80
    arrays, offs = cases.pack(insts)
    dts = [c.dt for c in insts]
    with ag.Batch([c.params for c in insts], [c.n_fluid for c in insts],
                  [c.n_wall for c in insts]) as b:
        b.integrate_batch(arrays, dts, 1, 1)
        first = cases.unpack({k: v.copy() for k, v in arrays.items()}, offs, insts)
        b.integrate_batch(arrays, dts, 2, 1)
    got = cases.unpack(arrays, offs, insts)
    worst = 0.0
    for k in subset:
        ref = O.State(first[k])
        O.step(ref, 2, insts[k].dt)
        for f in FIELDS:
            e = rel_err(getattr(got[k], f), getattr(ref, f))
            worst = max(worst, e)
            assert e <= TOL_STEP, (insts[k].name, insts[k].n, f, e)
    print(f"sweep subset ({len(subset)} of {len(insts)} instances): worst {worst:.2e}")


def test_batch_rejects_single_only_calls():
    insts = _instances_2d()[:2]
    with ag.Batch([c.params for c in insts], [c.n_fluid for c in insts],
                  [c.n_wall for c in insts]) as b:
        with pytest.raises(ag.ArmandoError) as e:  # packed arrays of the batch's size
            b.cell_ids(np.zeros(b.n * b.dim, np.float32), np.ones(b.n, np.float32))
        assert e.value.status == ag._abi.ERR_UNSUPPORTED


def test_batch_of_boundary_models_matches_instances_alone():
    """Instances with different wall models (0, 1, 2) in one batch."""
    insts = _instances_2d()[:3]
    insts[1].params.wall_model = 1
    insts[2].params.wall_model = 2
    _packed_ok(insts)
    outs = _run_batch(insts, 1, 4)
    for k, c in enumerate(insts):
        alone = _run_single(c, 1, 4)
        for f in FIELDS:
            assert np.array_equal(getattr(outs[k], f), getattr(alone, f)), (k, f)


def _lean_sweep():
    insts = cases.sweep(n_instances=8, seed=45, n_min=400, n_max=4000)
    assert all(c.params.visc == 0 and c.params.heat_artificial == 0 for c in insts)
    return insts


def test_lean_batch_equals_instances_run_alone():
    """Every instance lean (the sweep's physics): the batch runs the lean
    passes, still bit-identical to each instance run alone."""
    insts = _lean_sweep()
    got = _run_batch(insts, 1, 5)
    for c, g in zip(insts, got):
        ref = _run_single(c, 1, 5)
        for f in FIELDS:
            assert np.array_equal(getattr(g, f), getattr(ref, f)), (c.name, f)


def test_batch_autotune_times_the_reach_and_keeps_the_fastest():
    insts = _lean_sweep()
    arrays, offs = cases.pack(insts)
    before = {k: v.copy() for k, v in arrays.items()}
    dts = [c.dt for c in insts]
    with ag.Batch([c.params for c in insts], [c.n_fluid for c in insts],
                  [c.n_wall for c in insts]) as b:
        best, table = b.autotune_batch(arrays, dts, 1, 3)
        for k in before:  # the state is not modified
            assert np.array_equal(arrays[k], before[k]), k
        assert sorted(table) == [(1, 1, 128, 0), (2, 1, 128, 0), (3, 1, 128, 0)]
        assert best == min(table, key=table.get)
        assert b.tuning().as_tuple() == best
        b.integrate_batch(arrays, dts, 1, 4)
    got = cases.unpack(arrays, offs, insts)
    for c, g in zip(insts, got):  # the tuned batch equals each instance alone at that tuning
        ref = c.copy()
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(*best)
            ctx.integrate(ref, c.dt, 1, 4)
        for f in FIELDS:
            assert np.array_equal(getattr(g, f), getattr(ref, f)), (c.name, best, f)
