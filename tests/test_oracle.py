"""Self-consistency of the CPU oracle (two reference routines that must agree,
conservation properties of the pair formulas, pair-loop vs gather form)."""
import math

import numpy as np
import pytest

from armando_gb300 import cases
from armando_gb300._abi import Params


def _pairs(pi, pj):
    return set(zip(pi.tolist(), pj.tolist()))


@pytest.mark.parametrize("fp32", [False, True])
def test_link_list_equals_direct_find_2d(O, fp32):
    c = cases.cavity(n_side=20)
    a = O.link_list(c.x, c.h, 2, fp32=fp32)
    b = O.link_list(c.x, c.h, 2, fp32=fp32, direct=True)
    assert len(a[0]) > 0 and _pairs(a[0], a[1]) == _pairs(b[0], b[1])


def test_link_list_equals_direct_find_3d_periodic(O):
    c = cases.channel(n_x=12, n_yz=5, length=12 * 7.9e-4, width=5 * 7.9e-4, layers=2, jitter=0.05)
    for per in (False, True):
        P = c.params if per else None
        a = O.link_list(c.x, c.h, 3, params=P)
        b = O.link_list(c.x, c.h, 3, params=P, direct=True)
        assert _pairs(a[0], a[1]) == _pairs(b[0], b[1])
    # periodic wrap adds pairs across x = 0 / x = L
    a0 = O.link_list(c.x, c.h, 3)
    a1 = O.link_list(c.x, c.h, 3, params=c.params)
    assert len(a1[0]) > len(a0[0])


def test_fp32_pairs_equal_fp64_away_from_threshold(O):
    c = cases.dam_break(dx=0.05)
    a = O.link_list(c.x, c.h, 2)
    b = O.link_list(c.x, c.h, 2, fp32=True)
    assert _pairs(a[0], a[1]) == _pairs(b[0], b[1])


def test_kernel_normalisation(O):
    # Lattice sum of W dx^dim approaches 1 as h/dx grows (Wendland C2 is normalised).
    for dim in (2, 3):
        s = cases.lattice_kernel_sum(dim, 3.0)
        assert abs(s - 1.0) < 2e-3
    w, _ = O.kernel(np.array([0.0]), np.array([1.0]), 2)
    assert abs(w[0] - 7.0 / (4.0 * math.pi)) < 1e-15


def test_pair_loop_equals_gather_form(O):
    for case in (cases.cavity(n_side=16), cases.perturbed(cases.dam_break(dx=0.05), 3, dv=0.1),
                 cases.channel(n_x=12, n_yz=6, length=12 * 7.9e-4, width=6 * 7.9e-4, layers=2)):
        a, b = O.State(case), O.State(case)
        for its in (1, 2, 3):
            O.step(a, its, case.dt)
        O.integrate_gather(b, 1, 3, case.dt, 4)
        for f in ("x", "v", "rho", "p", "u", "dvdt", "dudt"):
            A, B = getattr(a, f), getattr(b, f)
            # summation order only; rounding is amplified by c0^2 through the EOS
            assert np.abs(A - B).max() <= 1e-9 * max(np.abs(A).max(), 1e-30), (case.name, f)


def test_momentum_conservation_without_walls(O):
    # Pairwise antisymmetry of int_force and art_visc: sum m_i a_i = 0 (no gravity, no walls).
    rng = np.random.default_rng(0)
    n, dx = 400, 1e-3
    i, j = np.meshgrid(np.arange(20), np.arange(20), indexing="ij")
    x = np.stack([(i.ravel() + 0.5) * dx, (j.ravel() + 0.5) * dx], 1)
    x += rng.uniform(-0.1, 0.1, x.shape) * dx
    P = Params.default(dim=2, pa_sph=1, visc=1, eta=1e-3, visc_artificial=1, av_alpha=0.1,
                       av_beta=0.0, rho0=1000.0, c0=10.0)
    st = O.State(cases.Case("t", P, 2, x.ravel().astype(np.float32),
                            rng.normal(0, 0.1, 2 * n).astype(np.float32),
                            np.full(n, 1e-3, np.float32), np.full(n, 1000.0, np.float32),
                            np.zeros(n, np.float32), np.zeros(n, np.float32),
                            np.full(n, 1.3e-3, np.float32), np.ones(n, np.int32), 1e-6, 1))
    O.step(st, 1, 1e-6)
    a = st.dvdt.reshape(n, 2)
    total = (st.m[:, None] * a).sum(0)
    scale = (st.m[:, None] * np.abs(a)).sum(0)
    assert np.all(np.abs(total) <= 1e-12 * scale)


def test_tait_clamp_sets_rho0(O):
    p = O.tait(np.array([990.0, 1000.0, 1010.0]), 1000.0, 10.0, pmin=0.0, clamp=True)
    assert p[0] == 0.0 and p[1] == 0.0 and p[2] > 0.0


def test_first_step_half_kick(O):
    # its == 1: v = v + dt/2 a, x = x + dt v (time_integration.f:202-218).
    c = cases.perturbed(cases.dam_break(dx=0.05), 5, dv=0.2)
    s = O.State(c)
    x0, v0 = s.x.copy(), s.v.copy()
    O.step(s, 1, c.dt)
    fl = np.repeat(c.itype > 0, 2)
    assert np.allclose(s.v[fl], v0[fl] + 0.5 * c.dt * s.dvdt[fl], rtol=0, atol=1e-14)
    assert np.allclose(s.x[fl], x0[fl] + c.dt * s.v[fl], rtol=0, atol=1e-14)
    assert np.array_equal(s.x[~fl], x0[~fl]) and np.array_equal(s.v[~fl], v0[~fl])


@pytest.mark.parametrize("name", ["dambreak", "channel3d", "cavity"])
def test_fluid_input_density_and_pressure_unused_under_summation(O, name):
    """Under summation density (density.f:1-62) a step recomputes every fluid
    particle's density and, by the equation of state, its pressure before any
    term reads them: the oracle's step from NaN fluid inputs rho and p equals
    the step from the real ones. (The device step therefore does not read
    them; walls keep theirs.)"""
    if name == "dambreak":
        c = cases.perturbed(cases.dam_break(dx=0.04), seed=81, dv=0.05)
    elif name == "cavity":
        c = cases.perturbed(cases.cavity(n_side=16), seed=82, dv=1e-4)
    else:
        c = cases.perturbed(cases.channel(n_x=12, n_yz=5, length=12 * 7.9e-4,
                                          width=5 * 7.9e-4, layers=2, jitter=0.05),
                            seed=83, dv=0.02, du=50.0)
    assert c.params.density_form == 0 and c.params.scheme == 0
    bad = c.copy()
    fl = bad.itype > 0
    bad.rho = np.where(fl, np.float32(np.nan), bad.rho).astype(np.float32)
    bad.p = np.where(fl, np.float32(np.nan), bad.p).astype(np.float32)
    for its in (1, 2):
        a, b = O.State(c), O.State(bad)
        O.step(a, its, c.dt)
        O.step(b, its, c.dt)
        for f in ("x", "v", "rho", "p", "u", "dvdt", "dudt"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), (name, its, f)
