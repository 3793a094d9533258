"""Boundary models of the oracle (armando_params.wall_model) on cases small
enough to check against the formulas by hand."""
import math

import numpy as np
import pytest

from armando_gb300._abi import Params


def two_particles(dx, h=0.013, m=0.1, rho=(1000.0, 1010.0)):
    x = np.array([0.0, 0.0, dx, 0.0])
    return dict(x=x, v=np.zeros(4), m=np.full(2, m), rho=np.array(rho), p=np.array([500.0, 800.0]),
                u=np.zeros(2), h=np.full(2, h), itype=np.array([1, 0], np.int32))


def wendland_2d(r, h):
    q = r / h
    return 7.0 / (4.0 * math.pi * h * h) * (1 - q / 2) ** 4 * (1 + 2 * q) if q < 2 else 0.0


def test_wall_model_1_pushes_only(O):
    """armando.cu:507-513: a fluid particle and a wall particle within support
    neither exchange pressure nor viscosity; the fluid one is pushed by
    0.5 W m_j/(rho_j h_j) c0^2 along (x_i - x_j)/r."""
    c0, r, h = 15.0, 0.012, 0.013
    P = Params.default(dim=2, pa_sph=1, rho0=1000.0, c0=c0, visc_artificial=1)
    P.wall_model = 1
    s = two_particles(r, h)
    dv, du = O.forces(P, s["x"], s["v"], s["m"], s["rho"], s["p"], s["u"], s["h"], s["itype"])
    f = 0.5 * wendland_2d(r, h) * s["m"][1] / (s["rho"][1] * h) * c0 ** 2
    assert dv[0] == pytest.approx(-f, rel=1e-12)  # x_0 - x_1 = -r: pushed towards -x
    assert dv[1] == 0.0 and dv[3] == 0.0 and du[0] == 0.0
    # the same pair under wall_model 0 exchanges pressure instead
    P.wall_model = 0
    dv0, _ = O.forces(P, s["x"], s["v"], s["m"], s["rho"], s["p"], s["u"], s["h"], s["itype"])
    assert dv0[0] != pytest.approx(-f, rel=1e-3)


def test_wall_model_2_adds_push_to_pressure(O):
    c0, r, h = 15.0, 0.012, 0.013
    P = Params.default(dim=2, pa_sph=1, rho0=1000.0, c0=c0)
    s = two_particles(r, h)
    args = (s["x"], s["v"], s["m"], s["rho"], s["p"], s["u"], s["h"], s["itype"])
    P.wall_model = 0
    dv0, _ = O.forces(P, *args)
    P.wall_model = 2
    dv2, _ = O.forces(P, *args)
    push = 0.02 * wendland_2d(r, h) / wendland_2d(0.0, h) * c0 * c0 / r * 0.5
    assert dv2[0] - dv0[0] == pytest.approx(-push, rel=1e-12)


def test_gather_form_refuses_wall_models(O):
    from armando_gb300 import cases

    c = cases.dam_break(dx=0.1)
    c.params.wall_model = 1
    with pytest.raises(RuntimeError):
        O.integrate_gather(O.State(c), 1, 1, c.dt)
