"""Mirror ghost particles (wall_model 3) on the GPU vs the FP64 oracle.

Wall particles carry their inward unit normal in v (CERN virtual-particle
files). Gates as for the other boundary models: one step from identical FP32
inputs within TOL_STEP = 1e-5 on every output (normwise relative); the ghost
count equal to the oracle's; many steps within 20x the oracle's one-ulp
conditioning.
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


def ghost_cases():
    dam = cases.perturbed(cases.dam_break(dx=0.02, col_w=0.6, col_h=1.2, tank_w=1.6, tank_h=1.5,
                                          seed=81), seed=82, dv=0.3)
    cav = cases.cavity()
    n = 12
    L = n * 7.9e-4
    ch = cases.perturbed(cases.channel(n_x=30, n_yz=n, length=30 * 7.9e-4, width=L, layers=3,
                                       jitter=0.02, seed=83), seed=84, dv=0.05, du=50.0)
    ch.params.periodic[0] = 0  # a closed duct: walls on y and z, open ends in x
    return {
        "dambreak": cases.with_mirror_ghosts(dam, lo=(0.0, 0.0), hi=(1.6, None)),
        "cavity": cases.with_mirror_ghosts(cav, lo=(0.0, 0.0), hi=(1.0e-3, 1.0e-3)),
        "channel3d": cases.with_mirror_ghosts(ch, lo=(None, 0.0, 0.0), hi=(None, L, L)),
    }


def oracle_steps(O, c, its0, steps):
    st = O.State(c)
    for its in range(its0, its0 + steps):
        O.step(st, its, c.dt, nbr_fp32=True)
    return st


def as_case(c, st):
    out = c.copy()
    for f in FIELDS:
        setattr(out, f, getattr(st, f).astype(np.float32))
    return out


@pytest.mark.parametrize("name", ["dambreak", "cavity", "channel3d"])
@pytest.mark.parametrize("its", [1, 3])
def test_one_step_parity(O, name, its):
    c = ghost_cases()[name]
    inp = c if its == 1 else as_case(c, oracle_steps(O, c, 1, its - 1))
    ref = O.State(inp)
    O.step(ref, its, inp.dt, nbr_fp32=True)
    got = inp.copy()
    with ag.Context(inp.params, inp.n_fluid, inp.n_wall) as ctx:
        ctx.step(got, inp.dt, its)
        ghosts = ctx.stats().ghosts
    owner, _, _, _ = O.ghosts(inp.params, inp.x, inp.v, inp.h, inp.itype)
    assert ghosts == len(owner) > 0
    for f in FIELDS:
        e = rel_err(getattr(got, f), getattr(ref, f))
        assert e <= TOL_STEP, (name, its, f, e)


@pytest.mark.parametrize("tuning", [(2, 1, 256, 0), (3, 2, 128, 0), (1, 4, 128, 0)])
def test_tunings_with_ghosts(O, tuning):
    c = ghost_cases()["dambreak"]
    ref = O.State(c)
    O.step(ref, 1, c.dt, nbr_fp32=True)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.set_tuning(*tuning)
        ctx.step(got, c.dt, 1)
    for f in FIELDS:
        assert rel_err(getattr(got, f), getattr(ref, f)) <= TOL_STEP, (tuning, f)


def test_many_steps_track_the_oracle(O):
    """20 iterations: GPU vs oracle within 20x the oracle's change when its
    fluid positions move by one FP32 ulp, or 1e-5."""
    c = ghost_cases()["dambreak"]
    rng = np.random.default_rng(85)
    c2 = c.copy()
    bump = np.where(rng.random(c.x.size) < 0.5, np.inf, -np.inf).astype(np.float32)
    c2.x = np.where(np.repeat(c.itype > 0, 2), np.nextafter(c.x, bump), c.x).astype(np.float32)
    ref = oracle_steps(O, c, 1, 20)
    pert = oracle_steps(O, c2, 1, 20)
    got = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(got, c.dt, 1, 20)
    for f in FIELDS:
        cond = rel_err(getattr(pert, f), getattr(ref, f))
        err = rel_err(getattr(got, f), getattr(ref, f))
        assert err <= max(20.0 * cond, 1e-5), (f, err, cond)


def test_integrate_equals_steps_and_is_deterministic():
    c = ghost_cases()["channel3d"]
    a, b, d = c.copy(), c.copy(), c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        ctx.integrate(a, c.dt, 1, 4)
        ctx.integrate(b, c.dt, 1, 4)
        for its in range(1, 5):
            ctx.step(d, c.dt, its)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
        assert np.array_equal(getattr(a, f), getattr(d, f)), f


def test_without_walls_in_reach_equals_wall_model_0():
    """Fluid far from every wall: no ghosts, the same bits as wall_model 0."""
    c = ghost_cases()["dambreak"]
    far = c.copy()
    xy = far.x.reshape(-1, 2)
    xy[far.itype <= 0] += np.float32(10.0)  # walls moved out of reach
    far.x = xy.ravel()
    base = far.copy()
    base.params.wall_model = 0
    a, b = far.copy(), base.copy()
    with ag.Context(far.params, far.n_fluid, far.n_wall) as ctx:
        ctx.step(a, far.dt, 1)
        assert ctx.stats().ghosts == 0
    with ag.Context(base.params, base.n_fluid, base.n_wall) as ctx:
        ctx.step(b, base.dt, 1)
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_autotune_keeps_skin_zero():
    c = ghost_cases()["dambreak"]
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        best, table = ctx.autotune(c, c.dt, 1, steps_per_trial=2)
        assert best[3] == 0
        assert all(k[3] == 0 for k, v in table.items() if v > 0)


def test_refusals():
    c = ghost_cases()["dambreak"]
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        with pytest.raises(ag.ArmandoError) as e:
            ctx.set_tuning(1, 1, 128, 20)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED
        with pytest.raises(ag.ArmandoError) as e:
            ctx.forward_checkpointed(c.copy(), c.dt, 1, 4, 2)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED
        ctx.integrate(c.copy(), c.dt, 1, 2)
        with pytest.raises(ag.ArmandoError) as e:
            ctx.profile_phases(1)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED
    plain = c.copy()
    plain.params.wall_model = 0
    with ag.Context(plain.params, plain.n_fluid, plain.n_wall) as ctx:
        with pytest.raises(ag.ArmandoError) as e:
            ctx.set_params(c.params)
        assert e.value.status == ag._abi.ERR_UNSUPPORTED
    with pytest.raises(ag.ArmandoError) as e:
        ag.Batch([c.params, c.params], [c.n_fluid] * 2, [c.n_wall] * 2)
    assert e.value.status == ag._abi.ERR_UNSUPPORTED
    per = cases.channel(n_x=10, n_yz=4, length=10 * 7.9e-4, width=4 * 7.9e-4, layers=2)
    per.params.wall_model = 3
    with pytest.raises(ag.ArmandoError) as e:
        ag.Context(per.params, per.n_fluid, per.n_wall)
    assert e.value.status == ag._abi.ERR_INVALID_ARG


def test_deck_to_step(O, tmp_path):
    """The Fortran virtual_part workflow: a deck with the walls' normals in the
    v_ files, read back and stepped with mirror ghosts."""
    c = ghost_cases()["dambreak"]
    order = np.argsort(c.itype <= 0, kind="stable")
    arrs = {f: (getattr(c, f).reshape(c.n, -1)[order].ravel() if f in ("x", "v")
                else getattr(c, f)[order]) for f in ag.DECK_FIELDS}
    ag.write_deck(tmp_path, 2, c.n_fluid, arrs)
    d = ag.read_deck(tmp_path, 2)
    assert d["n_real"] == c.n_fluid and d["n_virtual"] == c.n_wall
    inp = c.copy()
    for f in ag.DECK_FIELDS:
        setattr(inp, f, d[f])
    inp.dvdt = np.zeros_like(inp.x)
    inp.dudt = np.zeros_like(inp.u)
    ref = O.State(inp)
    O.step(ref, 1, inp.dt, nbr_fp32=True)
    got = inp.copy()
    with ag.Context(inp.params, inp.n_fluid, inp.n_wall) as ctx:
        ctx.step(got, inp.dt, 1)
        assert ctx.stats().ghosts > 0
    for f in FIELDS:
        assert rel_err(getattr(got, f), getattr(ref, f)) <= TOL_STEP, f
