"""The FP64 tangent-linear oracle (dual numbers) against FP64 central finite
differences of the same loss: the reference the GPU adjoint is checked on."""
import numpy as np
import pytest

from armando_gb300 import cases


def _case():
    c = cases.perturbed(cases.dam_break(dx=0.05), seed=3, dv=0.1)
    c.params.av_beta = 0.3
    c.params.heat_external = 1
    c.params.heat_q0 = 1.0e6
    c.params.heat_sigma = 0.3
    c.params.set("heat_center", (0.5, 1.0, 0.0))
    return c


@pytest.mark.parametrize("name,k", [("av_alpha", 0), ("av_beta", 1), ("c0", 2), ("heat_q0", 3)])
def test_tangent_linear_matches_central_differences_params(O, name, k):
    c = _case()
    st = O.State(c)
    spec = O.LossSpec.make(w_ke=1.0, w_p=1e-4, w_u=0.1, c=(0.9, 0.3), radius=0.4)
    dp = [0.0] * 4
    dp[k] = 1.0
    _, dL = O.tangent(st, 1, 10, c.dt, spec, dparam=dp)
    a = getattr(c.params, name)
    p1, p2 = c.params.copy(), c.params.copy()
    setattr(p1, name, a * (1 + 1e-5))
    setattr(p2, name, a * (1 - 1e-5))
    h = float(getattr(p1, name)) - float(getattr(p2, name))  # FP32 parameters
    fd = (O.loss(st, 1, 10, c.dt, spec, p1) - O.loss(st, 1, 10, c.dt, spec, p2)) / h
    assert abs(dL - fd) <= 1e-5 * abs(fd) + 1e-12, (dL, fd)


def test_tangent_linear_matches_central_differences_velocity(O):
    c = _case()
    st = O.State(c)
    spec = O.LossSpec.make(w_ke=1.0, w_p=1e-4, w_u=0.1, c=(0.9, 0.3), radius=0.4)
    rng = np.random.default_rng(0)
    dv = rng.standard_normal(st.v.size) * np.repeat(c.itype > 0, 2)
    _, dL = O.tangent(st, 1, 10, c.dt, spec, dv0=dv)
    e = 1e-6
    s1, s2 = O.State(c), O.State(c)
    s1.v = st.v + e * dv
    s2.v = st.v - e * dv
    fd = (O.loss(s1, 1, 10, c.dt, spec) - O.loss(s2, 1, 10, c.dt, spec)) / (2 * e)
    assert abs(dL - fd) <= 1e-5 * abs(fd), (dL, fd)


def visc_case():
    """The lid-driven cavity (physical viscosity, internal_force.f:75-171) with
    a perturbed velocity field, so the shear tensors and their heating carry
    gradient everywhere."""
    return cases.perturbed(cases.cavity(), seed=5, dv=2e-4)


def test_tangent_linear_with_viscosity_matches_central_differences(O):
    c = visc_case()
    st = O.State(c)
    spec = O.LossSpec.make(w_ke=1.0, w_p=1e-6, w_u=1.0, c=(5e-4, 5e-4), radius=3e-4)
    rng = np.random.default_rng(1)
    dv = rng.standard_normal(st.v.size) * np.repeat(c.itype > 0, 2)
    _, dL = O.tangent(st, 1, 5, c.dt, spec, dv0=dv)
    e = 1e-7
    s1, s2 = O.State(c), O.State(c)
    s1.v = st.v + e * dv
    s2.v = st.v - e * dv
    fd = (O.loss(s1, 1, 5, c.dt, spec) - O.loss(s2, 1, 5, c.dt, spec)) / (2 * e)
    assert abs(dL - fd) <= 1e-5 * abs(fd), (dL, fd)
