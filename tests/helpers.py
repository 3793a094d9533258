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
