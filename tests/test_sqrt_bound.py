"""The neighbour test of the GPU-C stage kernel compares r^2 with a per-particle
bound t instead of sqrt_rn(r^2) with lim = 2 h (gpuc.cuh, sqrt_less_bound):
t is the smallest FP32 value with sqrt_rn(t) >= lim, found from lim^2 rounded
by at most four steps up and four down. numpy's float32 square root and
product are IEEE correctly rounded like __fsqrt_rn and __fmul_rn; this checks
that one step always suffices and that the bound reproduces the square-root
test exactly."""
import numpy as np

F = np.float32


def bound(lim):
    t = (lim * lim).astype(F)
    up = np.sqrt(t) < lim
    t = np.where(up, np.nextafter(t, F(np.inf)), t)
    assert np.all(np.sqrt(t) >= lim)  # one step up is enough
    d = np.nextafter(t, F(0))
    down = np.sqrt(d) >= lim
    t = np.where(down, d, t)
    assert np.all(np.sqrt(np.nextafter(t, F(0))) < lim)  # one step down is enough
    return t


def test_one_step_from_the_rounded_square():
    rng = np.random.default_rng(7)
    lims = np.concatenate([rng.uniform(1e-4, 1.0, 200_000),
                           10.0 ** rng.uniform(-30, 19, 200_000)]).astype(F)
    t = bound(lims)
    assert np.all(np.sqrt(t) >= lims)


def test_bound_reproduces_the_square_root_test():
    rng = np.random.default_rng(8)
    lim = rng.uniform(1e-3, 1e-1, 2000).astype(F)
    t = bound(lim)
    # r^2 values around lim^2, within a few ulps, and far from it
    r2 = (lim[:, None] ** 2).astype(F) * (1 + rng.uniform(-1e-6, 1e-6, (2000, 64))).astype(F)
    r2 = np.concatenate([r2, rng.uniform(0, 0.02, (2000, 64)).astype(F)], 1).astype(F)
    np.testing.assert_array_equal(np.sqrt(r2) < lim[:, None], r2 < t[:, None])
