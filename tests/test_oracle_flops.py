"""The oracle's operation counter (the algorithmic FLOPs of the two-roof figure)."""
import numpy as np
import pytest

from armando_gb300 import cases
from armando_gb300._abi import Params


def isolated_state(O, n, dim, seed=3):
    """n fluid particles on a coarse lattice, each alone in its 3^dim stencil."""
    rng = np.random.default_rng(seed)
    h = 0.01
    k = int(np.ceil(n ** (1.0 / dim)))
    idx = np.stack(np.unravel_index(np.arange(n), (k,) * dim), 1).astype(np.float64)
    x = idx * 10 * h + rng.uniform(-h, h, size=idx.shape)
    c = cases.Case("isolated", Params.default(dim=dim, visc_artificial=1), dim,
                   x.ravel().astype(np.float32), np.zeros(n * dim, np.float32),
                   np.full(n, 1e-4, np.float32), np.full(n, 1000.0, np.float32),
                   np.zeros(n, np.float32), np.zeros(n, np.float32),
                   np.full(n, h, np.float32), np.ones(n, np.int32), dt=1e-5, steps=1)
    return O.State(c)


@pytest.mark.parametrize("dim", [2, 3])
def test_neighbour_search_count_of_isolated_particles(O, dim):
    # link_list on particles without neighbours: the grid (2 mh, then per axis
    # lo, hi, extent / cell), and each particle's cell coordinates twice
    # ((x - o) / size per axis, for the counting sort and for its stencil).
    n = 50
    st = isolated_state(O, n, dim)
    _, search = O.flops(st, 2, 1e-5)
    assert search == 1 + 4 * dim + 4 * dim * n


def test_dambreak_count_is_plausible_and_deterministic(O):
    c = cases.dam_break(dx=0.02)
    st = O.State(c)
    O.step(st, 1, c.dt)
    a = O.flops(st, 2, c.dt)
    b = O.flops(st, 2, c.dt)
    assert a == b
    per = a[0] / c.n
    # ~20 neighbours, pairs j > i once: a few hundred flop per particle for the
    # search, ~1-3 kflop for the iteration
    assert 1000 < per < 3000 and 100 < a[1] / c.n < 400
    # the count does not modify the state
    x0 = st.x.copy()
    O.flops(st, 2, c.dt)
    assert np.array_equal(st.x, x0)
