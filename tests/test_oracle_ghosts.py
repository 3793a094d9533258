"""Mirror ghost particles of the oracle (wall_model 3, CERNsource/ghost.f).

Checked three ways: against a loop-by-loop Python restatement of ghost.f on
the oracle's own pair list, against the mirror geometry of a flat wall by
hand, and through the step (ghosts only change particles within reach of a
wall)."""
import numpy as np
import pytest

from armando_gb300 import cases
from helpers import FIELDS


def small_tank(seed=3):
    c = cases.dam_break(dx=0.05, col_w=0.5, col_h=0.6, tank_w=1.0, tank_h=0.8, seed=seed,
                        jitter=0.05)
    return cases.with_mirror_ghosts(cases.perturbed(c, seed=seed + 1, dv=0.3), lo=(0.0, 0.0),
                                    hi=(1.0, None))


def ghost_f_restated(O, c):
    """ghost.f:34-84 as loops over the oracle's FP64 pair list of the current
    positions; the nearest wall on the FP64 squared distance, ties to the
    lower index."""
    dim = c.dim
    x = c.x.astype(np.float64).reshape(-1, dim)
    v = c.v.astype(np.float64).reshape(-1, dim)
    pi, pj, _, _ = O.link_list(c.x, c.h, dim, fp32=False, params=c.params)
    fluid = c.itype > 0
    best = {}
    for a, b in zip(pi.tolist(), pj.tolist()):
        for i, j in ((a, b), (b, a)):
            if fluid[i] and not fluid[j]:
                dd = sum((x[j, d] - x[i, d]) ** 2 for d in range(dim))
                if i not in best or dd < best[i][0] or (dd == best[i][0] and j < best[i][1]):
                    best[i] = (dd, j)
    owner, wall, xg, vg = [], [], [], []
    for i in range(c.n):
        if i not in best:
            continue
        j = best[i][1]
        dd1 = sum((x[i, d] - x[j, d]) * v[j, d] for d in range(dim))
        dd2 = sum(v[i, d] * v[j, d] for d in range(dim))
        owner.append(i)
        wall.append(j)
        xg.append([x[i, d] - 2.0 * v[j, d] * dd1 for d in range(dim)])
        vg.append([v[i, d] - 2.0 * v[j, d] * dd2 for d in range(dim)])
    return np.array(owner), np.array(wall), np.array(xg), np.array(vg)


def test_ghosts_match_loop_restatement(O):
    c = small_tank()
    owner, wall, xg, vg = O.ghosts(c.params, c.x, c.v, c.h, c.itype, fp32=False)
    r_owner, r_wall, r_xg, r_vg = ghost_f_restated(O, c)
    assert len(owner) > 10
    assert np.array_equal(owner, r_owner) and np.array_equal(wall, r_wall)
    np.testing.assert_allclose(xg, r_xg, rtol=0, atol=1e-15)
    np.testing.assert_allclose(vg, r_vg, rtol=0, atol=1e-15)


def test_fp32_selection_agrees_on_this_case(O):
    """The GPU mirror (nearest wall on FP32 coordinates) picks the same walls."""
    c = small_tank(seed=9)
    a = O.ghosts(c.params, c.x, c.v, c.h, c.itype, fp32=False)
    b = O.ghosts(c.params, c.x, c.v, c.h, c.itype, fp32=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])


def test_flat_wall_mirror_by_hand(O):
    """Fluid above a wall row y = 0 with normal (0, 1): ghost at (x, -y), the
    normal velocity component reversed, nearest wall particle chosen."""
    h = 0.013
    xs = np.array([[0.001, 0.004], [0.0205, 0.009], [0.05, 0.03]])  # third: out of reach
    wx = np.arange(-3, 8) * 0.01
    walls = np.stack([wx, np.zeros_like(wx)], 1)
    x = np.concatenate([xs, walls])
    v = np.concatenate([[[0.3, -0.2], [-0.1, 0.5], [0.0, 0.0]], np.tile([0.0, 1.0], (len(wx), 1))])
    itype = np.array([1, 1, 1] + [0] * len(wx), np.int32)
    P = cases.Params.default(dim=2, rho0=1000.0, c0=10.0)
    P.wall_model = 3
    owner, wall, xg, vg = O.ghosts(P, x.ravel(), v.ravel(), np.full(len(x), h), itype)
    assert owner.tolist() == [0, 1]
    assert wall.tolist() == [3 + 3, 3 + 5]  # walls at x = 0.00 and 0.02
    np.testing.assert_allclose(xg, [[0.001, -0.004], [0.0205, -0.009]], atol=1e-15)
    np.testing.assert_allclose(vg, [[0.3, 0.2], [-0.1, -0.5]], atol=1e-15)


def test_step_changes_only_particles_near_walls(O):
    """One iteration with and without ghosts: particles farther than two
    supports from every wall particle come out identical."""
    c = small_tank(seed=5)
    base = c.copy()
    base.params.wall_model = 0
    a, b = O.State(c), O.State(base)
    O.step(a, 1, c.dt)
    O.step(b, 1, c.dt)
    x = c.x.reshape(-1, 2).astype(np.float64)
    walls = x[c.itype <= 0]
    dist = np.sqrt(((x[:, None, :] - walls[None, :, :]) ** 2).sum(-1)).min(1)
    far = (dist > 4.0 * c.h.max()) & (c.itype > 0)
    near = (dist < 1.0 * c.h.max()) & (c.itype > 0)
    assert far.sum() > 10 and near.sum() > 10
    for f in ("rho", "p"):
        assert np.array_equal(getattr(a, f)[far], getattr(b, f)[far]), f
        assert not np.allclose(getattr(a, f)[near], getattr(b, f)[near]), f
    assert np.array_equal(a.v.reshape(-1, 2)[far], b.v.reshape(-1, 2)[far])


def test_ghost_density_sees_the_mirror_image(O):
    """A fluid particle next to a wall gains its ghost neighbours' mass in the
    summation density (Tait clamp off): larger exactly for the owners within
    the support of their own ghost, no smaller for any other."""
    c = small_tank(seed=6)
    c.params.pmin = -np.inf
    base = c.copy()
    base.params.wall_model = 0
    a, b = O.State(c), O.State(base)
    O.step(a, 1, c.dt)
    O.step(b, 1, c.dt)
    owner, _, xg, _ = O.ghosts(c.params, c.x, c.v, c.h, c.itype)
    x = c.x.reshape(-1, 2).astype(np.float64)[owner]
    reach = np.sqrt(((x - xg) ** 2).sum(1)) < 2.0 * c.h[owner]
    assert reach.sum() > 10
    assert np.all(a.rho[owner][reach] > b.rho[owner][reach])
    assert np.all(a.rho[owner] >= b.rho[owner])


def test_periodic_systems_refused(O):
    c = cases.channel(n_x=10, n_yz=4, length=10 * 7.9e-4, width=4 * 7.9e-4, layers=2)
    c.params.wall_model = 3
    with pytest.raises(RuntimeError):
        O.ghosts(c.params, c.x, c.v, c.h, c.itype)
    st = O.State(c)
    with pytest.raises(RuntimeError):
        O.step(st, 1, c.dt)
    assert FIELDS  # the shared field list stays importable
