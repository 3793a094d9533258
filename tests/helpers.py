"""Shared helpers of the parity tests (test infrastructure)."""
import numpy as np

FIELDS = ("x", "v", "rho", "p", "u", "dvdt", "dudt")


def rel_err(a, b):
    """Normwise relative error max|a - b| / max|b| (0 when both vanish)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.abs(b).max() if b.size else 0.0
    num = np.abs(a - b).max() if b.size else 0.0
    if den == 0.0:
        return 0.0 if num == 0.0 else float("inf")
    return float(num / den)


def history_state(O, case, steps=2):
    """Runs the FP64 oracle `steps` iterations and returns a copy of `case` holding
    that state rounded to FP32 (the identical FP32 input of a parity step)."""
    st = O.State(case)
    for its in range(1, steps + 1):
        O.step(st, its, case.dt)
    c = case.copy()
    for f in FIELDS:
        setattr(c, f, getattr(st, f).astype(np.float32))
    return c


def step_errors(O, ctx, case, its):
    """One GPU step and one FP64 oracle step from identical FP32 inputs;
    returns {field: normwise relative error} and the two states."""
    ref = O.State(case)
    got = case.copy()
    ctx.step(got, case.dt, its)
    O.step(ref, its, case.dt)
    errs = {f: rel_err(getattr(got, f), getattr(ref, f)) for f in FIELDS}
    return errs, got, ref


def probe_weight(x, dim, c, radius):
    """w = (1 - |x - c|^2/R^2)^3 inside R and its gradient (oracle LossSpec probe)."""
    X = np.asarray(x, np.float64).reshape(-1, dim)
    e = X - np.asarray(c[:dim], np.float64)
    t = 1.0 - (e * e).sum(1) / radius ** 2
    inside = t > 0
    w = np.where(inside, t ** 3, 0.0)
    gw = np.where(inside[:, None], 3.0 * t[:, None] ** 2 * (-2.0 * e / radius ** 2), 0.0)
    return w, gw


def loss_and_cotangents(state, dim, mass, itype, spec):
    """The oracle's loss (w_ke KE + w_p probe-pressure + w_u probe-energy, fluid
    particles, final state) and its cotangents with respect to the final x, v, u
    and the last iteration's pressure output, evaluated on a GPU result."""
    fl = np.asarray(itype) > 0
    m = np.asarray(mass, np.float64)
    v = np.asarray(state["v"], np.float64).reshape(-1, dim)
    p = np.asarray(state["p"], np.float64)
    u = np.asarray(state["u"], np.float64)
    w, gw = probe_weight(state["x"], dim, list(spec.c), spec.radius)
    w = np.where(fl, w, 0.0)
    gw = np.where(fl[:, None], gw, 0.0)
    L = (spec.w_ke * 0.5 * (m[fl, None] * v[fl] ** 2).sum()
         + spec.w_p / spec.w_ref * (w * p).sum() + spec.w_u / spec.w_ref * (w * u).sum())
    xb = (spec.w_p * p + spec.w_u * u)[:, None] / spec.w_ref * gw
    vb = np.where(fl[:, None], spec.w_ke * m[:, None] * v, 0.0)
    return L, {"x_bar": xb.ravel(), "v_bar": vb.ravel(), "u_bar": spec.w_u / spec.w_ref * w,
               "p_bar": spec.w_p / spec.w_ref * w}
