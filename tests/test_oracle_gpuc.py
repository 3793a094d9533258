"""The GPU-C scheme of the oracle (armando_params.scheme 1: TVD-RK3, continuity
density, the host path's pair physics) pinned on the reference's own compiled
C host path, ArmandoThrust/acpu.c (golden vectors of
tests/golden/make_gpuc_golden.py: the EOS functions, and 1 and 5 RK3 steps of
two small tanks in the published dam-break layout).

acpu.c computes in FP32 and the oracle in FP64. The integrated state (x, rho,
u) agrees to FP32 rounding (gate 1e-6 normwise relative). Pressure is a stiff
function of the FP32 density: one ulp of rho ~ 1000 (6.1e-5) is c0^2 ulp =
0.15 Pa of Tait pressure, about 1e-4 of the small tank's pressures, and the
velocity rates and velocities inherit it; their gates are 2e-4 (rates,
pressure) and 5e-5 (velocity), the same after one and after five steps.
"""
import os

import numpy as np
import pytest

from armando_gb300 import cases
from armando_gb300._abi import Material

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acpu_rk3.npz")
TOL = {"x": 1e-6, "rho": 1e-6, "u": 1e-6, "v": 5e-5, "p": 2e-4, "dv": 2e-4, "du": 2e-4}

MATS = {
    "tait": Material.make(4, [1000.0, 50.0, -1.0e12]),
    "shock": Material.make(3, [1000.0, 50.0, 0.5, 1.3]),
    "poly": Material.make(2, [1000.0, 2.5e6, 1.0e6, 2.0e5, 0.2, 0.1, 2.5e6, 5.0e5]),
    "gas": Material.make(1, [1.0, 1.4, 1.0e3]),
    "wall": Material.make(0, [1000.0, 50.0]),
}


@pytest.fixture(scope="module")
def G():
    return np.load(GOLD)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    s = np.abs(b).max()
    return np.abs(a - b).max() / s if s > 0 else np.abs(a).max()


@pytest.mark.parametrize("name", ["tait", "shock", "poly", "gas"])
def test_eos_matches_acpu(O, G, name):
    rho, u = G["eos_rho"], G["eos_u"]
    r, p, c = O.gpuc_eos(MATS[name], rho, u)
    np.testing.assert_array_equal(r.astype(np.float32), G[f"eos_{name}_rho"])
    assert rel(p, G[f"eos_{name}_p"]) <= 2e-6, name
    assert rel(c, G[f"eos_{name}_c"]) <= 1e-6, name


def run_oracle(O, G, pre, steps, table):
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    c.x, c.v, c.mass, c.rho = G[pre + "_x0"], G[pre + "_v0"], G[pre + "_m"], G[pre + "_rho0"]
    c.h, c.itype = G[pre + "_h"], G[pre + "_itype"]
    if pre + "_u0" in G:
        c.u = G[pre + "_u0"]
    st = O.State(c)
    dv, du = O.gpuc_step(st, steps, float(G[pre + "_dt"]), materials=table)
    return st, dv.reshape(-1, 2), du


@pytest.mark.parametrize("steps", [1, 5])
def test_water_tank_matches_acpu(O, G, steps):
    table = [MATS["tait"]] * 2
    st, dv, du = run_oracle(O, G, "water", steps, table)
    for f, got in (("x", st.x.reshape(-1, 2)), ("v", st.v.reshape(-1, 2)), ("rho", st.rho),
                   ("p", st.p), ("u", st.u), ("dv", dv), ("du", du)):
        # the water's u is pressure work from u = 0: it carries p's quantization
        tol = TOL["p"] if f == "u" else TOL[f]
        e = rel(got, G[f"water_{f}_{steps}"])
        assert e <= tol, (f, steps, e)


@pytest.mark.parametrize("steps", [1, 5])
def test_four_material_tank_matches_acpu(O, G, steps):
    """Tait, shock and polynomial water bands (repulsion between them) and
    boundary-type walls; u = 100 J/kg enters the shock and polynomial EOS."""
    table = [MATS["wall"], MATS["tait"], MATS["shock"], MATS["wall"], MATS["poly"]]
    st, dv, du = run_oracle(O, G, "multi", steps, table)
    for f, got in (("x", st.x.reshape(-1, 2)), ("v", st.v.reshape(-1, 2)), ("rho", st.rho),
                   ("p", st.p), ("u", st.u), ("dv", dv), ("du", du)):
        e = rel(got, G[f"multi_{f}_{steps}"])
        assert e <= TOL[f], (f, steps, e)


def test_device_variant_gates_pairs_by_material(O, G):
    """Scheme 2 (armando.cu:429-513): water next to boundary walls feels only
    the wall push, so its density rate differs from scheme 1 near the walls
    and not in the tank's interior."""
    c = cases.gpuc_dam_break(1, fluid=(20, 10), tank=(54, 16))
    c.v = G["water_v0"].copy()
    c2 = c.copy()
    c2.params.scheme = 2
    a, b = O.State(c), O.State(c2)
    O.gpuc_step(a, 1, c.dt)
    O.gpuc_step(b, 1, c.dt)
    x = c.x.reshape(-1, 2)
    fl = c.itype > 0
    near = fl & (x[:, 1] < 2.4 * c.h[0])
    inner = fl & (x[:, 1] > 6 * c.h[0]) & (x[:, 0] > 6 * c.h[0]) & (x[:, 0] < 0.35)
    assert inner.sum() > 20 and near.sum() > 10
    assert not np.allclose(a.rho[near], b.rho[near], rtol=0, atol=1e-9)
    np.testing.assert_allclose(a.rho[inner], b.rho[inner], rtol=2e-6)
