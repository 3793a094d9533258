"""GPU step vs the FP64 CPU oracle, through the C-ABI.

Tolerances (normwise relative, max|gpu - oracle| / max|oracle|, one step from
identical FP32 inputs): TOL_STEP = 1e-5 for x, v, rho, p, u, dv/dt, du/dt.
Cell ids and neighbour sets: bit-exact against the FP32 link_list of the oracle.
"""
import json
import os

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases
from helpers import FIELDS, history_state, rel_err, step_errors

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-5
# Error report of the parity runs (per case and field; drift curves), written
# as parity_report.json into $ARMANDO_REPORT_DIR when that is set.
REPORT_DIR = os.environ.get("ARMANDO_REPORT_DIR")


def _record(name, errs):
    if not REPORT_DIR:
        return
    REPORT = os.path.join(REPORT_DIR, "parity_report.json")
    try:
        os.makedirs(REPORT_DIR, exist_ok=True)
        data = json.load(open(REPORT)) if os.path.exists(REPORT) else {}
        data[name] = errs
        json.dump(data, open(REPORT, "w"), indent=1)
    except OSError:
        pass


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def small_cases():
    return {
        "cavity": cases.cavity(),
        "dambreak": cases.perturbed(cases.dam_break(dx=0.02), seed=21, dv=0.05),
        "dambreak_pa0": cases.perturbed(cases.dam_break(dx=0.03), seed=22, dv=0.05),
        "channel3d": cases.perturbed(
            cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4, width=12 * 7.9e-4, layers=3,
                          jitter=0.01), seed=23, dv=0.02, du=50.0),
    }


def _case(name):
    if name.endswith(("_w1", "_w2")):  # the GPU-C boundary models
        c = small_cases()[name[:-3]]
        c.params.wall_model = int(name[-1])
        return c
    c = small_cases()[name]
    if name == "dambreak_pa0":
        c.params.pa_sph = 0
    return c


@pytest.mark.parametrize("name", ["cavity", "dambreak", "channel3d"])
def test_cell_ids_bit_exact(O, name):
    c = _case(name)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        got = ctx.cell_ids(c.x, c.h)
        st = ctx.stats()
    _, _, cid, g = O.link_list(c.x, c.h, c.dim, fp32=True, params=c.params)
    assert np.array_equal(got.astype(np.int64), cid)
    assert list(st.grid_dims)[:c.dim] == list(g["n"][:c.dim])


@pytest.mark.parametrize("name", ["cavity", "dambreak", "channel3d"])
def test_neighbour_sets_bit_exact(O, name):
    c = _case(name)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        offs, nbr = ctx.neighbours(c.x, c.h)
    pi, pj, _, _ = O.link_list(c.x, c.h, c.dim, fp32=True, params=c.params)
    rows = [[] for _ in range(c.n)]
    for a, b in zip(pi.tolist(), pj.tolist()):
        rows[a].append(b)
        rows[b].append(a)
    ref_offs = np.zeros(c.n + 1, np.int64)
    ref_offs[1:] = np.cumsum([len(r) for r in rows])
    ref_nbr = np.array([k for r in rows for k in sorted(r)], np.int32)
    assert np.array_equal(offs, ref_offs)
    assert np.array_equal(nbr, ref_nbr)
    # FP64 link_list agrees on these inputs too (no pair within rounding of the cutoff).
    qi, qj, _, _ = O.link_list(c.x, c.h, c.dim, params=c.params)
    assert len(qi) == len(pi)


@pytest.mark.parametrize("name", ["cavity", "dambreak", "dambreak_pa0", "channel3d",
                                  "dambreak_w1", "dambreak_w2", "channel3d_w2", "cavity_w1"])
def test_one_step_parity(O, name):
    c = history_state(O, _case(name), steps=2)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        errs, got, ref = step_errors(O, ctx, c, its=3)
    _record(f"one_step/{name}", errs)
    print(name, {k: f"{v:.2e}" for k, v in errs.items()})
    for f in FIELDS:
        assert errs[f] <= TOL_STEP, (f, errs[f])
    walls = c.itype <= 0
    wd = np.repeat(walls, c.dim)
    assert np.array_equal(got.x[wd], c.x[wd]) and np.array_equal(got.v[wd], c.v[wd])
    assert np.array_equal(got.rho[walls], c.rho[walls]) and np.all(got.dvdt[wd] == 0)


@pytest.mark.parametrize("name", ["dambreak", "channel3d"])
def test_first_step_parity(O, name):
    c = _case(name)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        errs, _, _ = step_errors(O, ctx, c, its=1)
    _record(f"first_step/{name}", errs)
    for f in FIELDS:
        assert errs[f] <= TOL_STEP, (f, errs[f])


def test_integrate_equals_repeated_steps_and_is_deterministic():
    c = _case("dambreak")
    a, b, d = c.copy(), c.copy(), c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(a, c.dt, 1, 6)
        for its in range(1, 7):
            ctx.step(b, c.dt, its)
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(d, c.dt, 1, 6)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
        assert np.array_equal(getattr(a, f), getattr(d, f)), f


def one_ulp_twin(c, seed):
    """Copy of `c` whose fluid positions move by one FP32 ulp, randomly up or down."""
    rng = np.random.default_rng(seed)
    c2 = c.copy()
    fl = np.repeat(c.itype > 0, c.dim)
    bump = np.where(rng.random(c.x.size) < 0.5, np.inf, -np.inf).astype(np.float32)
    c2.x = np.where(fl, np.nextafter(c.x, bump), c.x).astype(np.float32)
    return c2


def drift_curve(O, c, checkpoints, seed):
    """GPU and FP64 oracle trajectories from the same FP32 state, plus the
    oracle from the one-ulp twin: {checkpoint: {field: (gpu err, twin err)}}."""
    ref, pert = O.State(c), O.State(one_ulp_twin(c, seed))
    got = c.copy()
    curve = {}
    done = 0
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        for cp in checkpoints:
            ctx.integrate(got, c.dt, done + 1, cp - done)
            O.integrate_gather(ref, done + 1, cp - done, c.dt)
            O.integrate_gather(pert, done + 1, cp - done, c.dt)
            done = cp
            curve[cp] = {f: (rel_err(getattr(got, f), getattr(ref, f)),
                             rel_err(getattr(pert, f), getattr(ref, f))) for f in FIELDS}
    for cp, e in curve.items():
        print("drift", cp, {f: f"{g:.1e}/{i:.1e}" for f, (g, i) in e.items()})
    return curve


def test_multi_step_drift_is_bounded(O):
    """1000 steps: the GPU's divergence from the FP64 oracle is compared with the
    oracle's own divergence when its FP32 inputs are perturbed by one ulp (the
    conditioning of the trajectory). Bound: GPU error <= 20x that, or 1e-5."""
    c = cases.perturbed(cases.dam_break(dx=0.03), seed=31, dv=0.05)
    curve = drift_curve(O, c, (1, 10, 100, 1000), seed=32)
    _record("drift/dambreak", {str(k): v for k, v in curve.items()})
    for f, (g, i) in curve[1000].items():
        assert np.isfinite(g) and g <= max(20.0 * i, 1e-5), (f, g, i)


def test_cavity_full_length_drift_is_bounded(O):
    """The 2D cavity benchmark over its full 3000 steps (1600 fluid + 320 wall
    particles, lid 1e-3 m/s, shear viscosity): the same bound as the dam break
    at every checkpoint."""
    c = cases.cavity()
    curve = drift_curve(O, c, (1, 10, 100, 300, 1000, 3000), seed=33)
    _record("drift/cavity", {str(k): v for k, v in curve.items()})
    for cp, e in curve.items():
        for f, (g, i) in e.items():
            assert np.isfinite(g) and g <= max(20.0 * i, 1e-5), (cp, f, g, i)


def test_device_memory_path_matches_host():
    import torch

    c = _case("channel3d")
    host = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(host, c.dt, 1, 3)
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in c.arrays().items()}
    with ag.Context(c.params, c.n_fluid, c.n_wall, mem=ag.MEM_DEVICE) as ctx:
        ctx.integrate(dev, c.dt, 1, 3)
    for f in FIELDS:
        assert np.array_equal(dev[f].cpu().numpy(), getattr(host, f)), f


def test_status_codes():
    c = _case("dambreak")
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        with pytest.raises(ag.ArmandoError) as e:
            ctx.step(c.copy(), -1.0, 1)
        assert e.value.status == ag._abi.ERR_INVALID_ARG
        bad = c.copy()
        ctx.step(bad, c.dt, 1)  # plans the grid
        far = bad.copy()
        far.x[0] = 1.0e4  # grid now far larger than the planned capacity
        with pytest.raises(ag.ArmandoError) as e:
            ctx.step(far, c.dt, 2)
        assert e.value.status == ag._abi.ERR_GRID_OVERFLOW
        nan = c.copy()
        nan.p[0] = np.nan  # a wall or fluid p feeding every neighbour
        nan.rho[:] = np.nan
        with pytest.raises(ag.ArmandoError) as e:
            ctx.step(nan, c.dt, 2)
        assert e.value.status == ag._abi.ERR_NONFINITE
    with pytest.raises(ag.ArmandoError) as e:
        ag.Context(c.params, -1, 0)
    assert e.value.status == ag._abi.ERR_INVALID_ARG
