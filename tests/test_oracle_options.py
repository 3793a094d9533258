"""single_step options of the oracle: continuity and normalised density
(density.f), XSPH (av_vel.f), smoothing-length evolution (hsml.f), and their
place in the leapfrog (time_integration.f). Known answers and the formulas
evaluated by hand on small cases; no reference output exists for them (the
Fortran cannot be built here)."""
import math

import numpy as np
import pytest

from armando_gb300 import cases


def lattice(seed=1, dx=0.02, n=8, jitter=0.1):
    """A block of fluid on a jittered lattice, no walls, no gravity."""
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    x = np.stack([i.ravel(), j.ravel()], 1) * dx + rng.uniform(-jitter, jitter, (n * n, 2)) * dx
    c = cases.dam_break(dx=0.05)
    m = len(x)
    c.x = x.ravel().astype(np.float32)
    c.v = np.zeros(2 * m, np.float32)
    c.mass = np.full(m, 1000.0 * dx * dx, np.float32)
    c.rho = np.full(m, 1000.0, np.float32)
    c.p = np.zeros(m, np.float32)
    c.u = np.zeros(m, np.float32)
    c.h = np.full(m, 1.3 * dx, np.float32)
    c.itype = np.ones(m, np.int32)
    c.dvdt = np.zeros(2 * m, np.float32)
    c.dudt = np.zeros(m, np.float32)
    c.params.gravity[1] = 0.0
    c.params.visc_artificial = 0
    c.params.pmin = -math.inf
    return c


def test_continuity_of_a_uniform_flow_keeps_density(O):
    """Uniform velocity: con_density gives drho/dt = 0 exactly; the step keeps rho."""
    c = lattice()
    c.v[0::2] = 0.7
    c.v[1::2] = -0.2
    c.params.density_form = 1
    st = O.State(c)
    O.step(st, 1, 1e-4)
    assert np.abs(st.drho).max() < 1e-9
    np.testing.assert_allclose(st.rho, 1000.0, rtol=0, atol=1e-9)


def test_continuity_matches_summation_rate(O):
    """drho/dt of con_density against the time derivative of the summation
    density (central difference of sum_density along the velocity field),
    interior particles of a smooth shear-free compression v = -k x."""
    c = lattice(jitter=0.05, n=10)
    x = c.x.reshape(-1, 2).astype(np.float64)
    k = 0.5
    c.v = (-k * (x - x.mean(0))).ravel().astype(np.float32)
    c.params.density_form = 1
    st = O.State(c)
    O.step(st, 1, 1e-7)
    drho = st.drho.copy()

    def summed(shift):
        b = c.copy()
        b.x = (c.x.astype(np.float64) + shift * c.v.astype(np.float64)).astype(np.float32)
        b.params.density_form = 0
        s = O.State(b)
        s.x = c.x.astype(np.float64) + shift * c.v.astype(np.float64)
        O.step(s, 1, 0.0)
        return s.rho

    eps = 1e-5
    fd = (summed(eps) - summed(-eps)) / (2 * eps)
    inner = np.all(np.abs(x - x.mean(0)) < 0.05, axis=1)
    assert inner.sum() >= 16
    np.testing.assert_allclose(drho[inner], fd[inner], rtol=1e-5, atol=1e-3 * np.abs(fd[inner]).max())


def test_normalised_density_is_exact_for_uniform_density(O):
    """nor_density returns a uniform rho unchanged, free surfaces included
    (where summation density falls short)."""
    c = lattice(jitter=0.2)
    c.params.density_form = 2
    st = O.State(c)
    O.step(st, 1, 0.0)
    np.testing.assert_allclose(st.rho, 1000.0, rtol=1e-12)
    c.params.density_form = 0
    s0 = O.State(c)
    O.step(s0, 1, 0.0)
    assert s0.rho.min() < 900.0


def test_xsph_velocity_correction(O):
    """Two particles: av_i = -0.3 m_j / rho_ij (v_i - v_j) W_ij added to v in the
    corrector of the second iteration on (av_vel.f, time_integration.f:195)."""
    c = lattice(n=2, jitter=0.0)
    keep = [0, 1]
    for f in ("mass", "rho", "p", "u", "h", "itype", "dudt"):
        setattr(c, f, getattr(c, f)[keep])
    c.x = np.array([0.0, 0.0, 0.012, 0.0], np.float32)
    c.v = np.array([0.5, 0.1, -0.2, 0.3], np.float32)
    c.dvdt = np.zeros(4, np.float32)
    dt = 1e-6
    a, b = c.copy(), c.copy()
    a.params.average_velocity = 1
    sa, sb = O.State(a), O.State(b)
    O.step(sa, 2, dt)
    O.step(sb, 2, dt)
    h, r = float(c.h[0]), float(c.x[2])  # the FP32 values the oracle reads
    w = cases.wendland_w(r, h, 2)
    m = float(c.mass[0])
    vv = c.v.astype(np.float64).reshape(2, 2)
    dv = vv[0] - vv[1]
    rho_i = sb.rho[0]  # the iteration's summation density (equal for both particles)
    av0 = -0.3 * m / rho_i * dv * w
    np.testing.assert_allclose(sa.v.reshape(2, 2)[0] - sb.v.reshape(2, 2)[0], av0, rtol=1e-9)
    np.testing.assert_allclose(sa.v.reshape(2, 2)[1] - sb.v.reshape(2, 2)[1], -av0, rtol=1e-9)


@pytest.mark.parametrize("dim", [2, 3])
def test_sle1_sets_h_from_density(O, dim):
    c = lattice() if dim == 2 else cases.channel(n_x=10, n_yz=4, length=10 * 7.9e-4,
                                                 width=4 * 7.9e-4, layers=2)
    c.params.sle = 1
    st = O.State(c)
    O.step(st, 1, 1e-6)
    fl = c.itype > 0
    e = float(np.float32(1.0) / np.float32(dim))
    np.testing.assert_allclose(st.h[fl], 2.0 * (st.m[fl] / st.rho[fl]) ** e, rtol=1e-13)
    np.testing.assert_array_equal(st.h[~fl], c.h[~fl].astype(np.float64))


def test_sle2_evolves_h_with_div_v(O):
    """dh/dt = (h/dim) div v: a uniform compression v = -k x shrinks h."""
    c = lattice(jitter=0.0, n=10)
    x = c.x.reshape(-1, 2).astype(np.float64)
    c.v = (-0.5 * (x - x.mean(0))).ravel().astype(np.float32)
    c.params.sle = 2
    dt = 1e-4
    st = O.State(c)
    O.step(st, 1, dt)
    inner = np.all(np.abs(x - x.mean(0)) < 0.05, axis=1)
    # div v = -2 k for v = -k x in 2D (up to the SPH gradient's accuracy)
    dh = (st.h - c.h) / dt
    np.testing.assert_allclose(dh[inner], (c.h[inner] / 2) * (-1.0), rtol=0.05)


def test_continuity_leapfrog_carries_drho(O):
    """its >= 2: rho = rho_min + dt drho with rho_min the iteration's start
    density and the predictor rho + dt/2 drho_prev in the EOS."""
    c = lattice(jitter=0.05)
    x = c.x.reshape(-1, 2).astype(np.float64)
    c.v = (-0.3 * (x - x.mean(0))).ravel().astype(np.float32)
    c.params.density_form = 1
    dt = 1e-5
    st = O.State(c)
    O.step(st, 1, dt)
    rho1, drho1 = st.rho.copy(), st.drho.copy()
    np.testing.assert_allclose(rho1, 1000.0 + 0.5 * dt * drho1, rtol=1e-14)
    O.step(st, 2, dt)
    np.testing.assert_allclose(st.rho, rho1 + dt * st.drho, rtol=1e-14)
    assert np.abs(st.drho - drho1).max() > 0
