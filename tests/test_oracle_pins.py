"""The oracle against golden outputs of the reference's own C host path
(ArmandoThrust/acpu.c), recorded by tests/golden/make_golden.py."""
import numpy as np

from armando_gb300._abi import Params


def test_wendland_matches_acpu(O, golden):
    w, dw = O.kernel(golden["wendland_r"].astype(np.float64),
                     golden["wendland_h"].astype(np.float64), 2)
    assert np.abs(w - golden["wendland_w"]).max() <= 1e-6 * np.abs(w).max()
    assert np.abs(dw - golden["wendland_dwdr"]).max() <= 1e-6 * np.abs(dw).max()


def test_tait_matches_acpu(O, golden):
    pr = golden["tait_props"]
    p = O.tait(golden["tait_rho"], float(pr[0]), float(pr[1]))
    # acpu.c evaluates powf(rho/rho0, 7) - 1 in FP32 (cancellation ~1e-6 of B).
    assert np.abs(p - golden["tait_p"]).max() <= 2e-5 * np.abs(p).max()


def test_cell_hash_matches_acpu_bit_exact(O, golden):
    _, _, cid, g = O.link_list(golden["lattice_x"], golden["lattice_h"], 2, fp32=True)
    gg = golden["lattice_grid"]
    assert np.allclose([g["o"][0], g["o"][1], g["size"][0], g["n"][0], g["n"][1]], gg, rtol=0, atol=0)
    assert np.array_equal(cid, golden["lattice_hash"].astype(np.int64))


def test_neighbour_lists_match_acpu(O, golden):
    n = golden["lattice_h"].size
    pi, pj, _, _ = O.link_list(golden["lattice_x"], golden["lattice_h"], 2)
    rows = [set() for _ in range(n)]
    for a, b in zip(pi, pj):
        rows[a].add(b)
        rows[b].add(a)
    offs, nbr = golden["list_offs"], golden["list_nbr"]
    # acpu.c keeps at most MAXN = 21 entries (self included): no row may be truncated.
    assert golden["list_count_with_self"].max() <= 21
    for i in range(n):
        assert set(nbr[offs[i]:offs[i + 1]].tolist()) == rows[i]


def test_pressure_force_pa_sph0_matches_acpu(O, golden):
    n = golden["lattice_h"].size
    x = golden["lattice_x"]
    P = Params.default(dim=2, pa_sph=0, rho0=1000.0, c0=20.0)
    dv, _ = O.forces(P, x, np.zeros_like(x), golden["force_mass"], golden["force_rho"],
                     golden["force_p"], np.zeros(n), golden["lattice_h"], np.ones(n, np.int32))
    assert np.abs(dv - golden["force_acc"]).max() <= 2e-6 * np.abs(dv).max()


def test_pressure_force_pa_sph1_matches_acpu_uniform_rho(O, golden):
    n = golden["lattice_h"].size
    x = golden["lattice_x"]
    P = Params.default(dim=2, pa_sph=1, rho0=1000.0, c0=20.0)
    dv, _ = O.forces(P, x, np.zeros_like(x), golden["force_mass"], np.full(n, 1000.0),
                     golden["force_p"], np.zeros(n), golden["lattice_h"], np.ones(n, np.int32))
    assert np.abs(dv - golden["force_acc_uniform_rho"]).max() <= 2e-6 * np.abs(dv).max()


def test_art_visc_matches_acpu_momentum_shock_correction(O, golden):
    """Moving particles at uniform density: acpu.c's momentum shock correction
    (acpu.c:413-422) is art_visc (art_visc.f:55-101) with alpha = 0.03,
    beta = 0, eta = 0.1 and c = c0 at uniform h, so the oracle's pa_sph 0
    pressure action plus art_visc must equal the compiled host path's rate."""
    n = golden["lattice_h"].size
    x, v = golden["lattice_x"], golden["moving_v"]
    P = Params.default(dim=2, pa_sph=0, rho0=1000.0, c0=20.0)
    P.visc_artificial = 1
    P.av_alpha, P.av_beta, P.av_eta = 0.03, 0.0, 0.1
    dv, _ = O.forces(P, x, v, golden["force_mass"], np.full(n, 1000.0), golden["force_p"],
                     np.zeros(n), golden["lattice_h"], np.ones(n, np.int32))
    ref = golden["moving_acc_uniform_rho"]
    assert np.abs(dv - ref).max() <= 2e-6 * np.abs(ref).max()
    # the viscous term is a visible part of the result, not rounding
    assert np.abs(ref - golden["force_acc_uniform_rho"]).max() > 1e-2 * np.abs(ref).max()
    P.visc_artificial = 0
    dv0, _ = O.forces(P, x, v, golden["force_mass"], np.full(n, 1000.0), golden["force_p"],
                      np.zeros(n), golden["lattice_h"], np.ones(n, np.int32))
    assert np.abs(dv0 - ref).max() > 1e-2 * np.abs(ref).max()


def test_con_density_matches_acpu_continuity_rate(O, golden):
    """con_density (density.f:161-218) against acpu.c's drho/dt at uniform
    density, where its mass shock correction vanishes (acpu.c:396, 407-411)."""
    n = golden["lattice_h"].size
    P = Params.default(dim=2, rho0=1000.0, c0=20.0)
    drho = O.con_density(P, golden["lattice_x"], golden["moving_v"], golden["force_mass"],
                         np.full(n, 1000.0), golden["lattice_h"], np.ones(n, np.int32))
    ref = golden["moving_drho_uniform_rho"]
    assert np.abs(drho - ref).max() <= 2e-6 * np.abs(ref).max()


def test_boundary_repulsion_matches_acpu_two_materials(O, golden):
    """wall_model 2 (acpu.c:424-429): pressure action of every pair plus the
    repulsion 0.02 (W/W0) c_i c_j m_j / ((m_i + m_j) r) between particles of
    different material, against the reference's own compiled host path."""
    n = golden["lattice_h"].size
    x = golden["lattice_x"]
    mat = golden["force_mat"].astype(np.int32)
    P = Params.default(dim=2, pa_sph=0, rho0=1000.0, c0=20.0)
    P.wall_model = 2
    dv, _ = O.forces(P, x, np.zeros_like(x), golden["force_mass"], golden["force_rho"],
                     golden["force_p"], np.zeros(n), golden["lattice_h"], mat)
    ref = golden["force_acc_two_materials"]
    assert np.abs(dv - ref).max() <= 2e-6 * np.abs(dv).max()
    # the repulsion is a visible part of the result, not rounding
    assert np.abs(ref - golden["force_acc"]).max() > 1e-2 * np.abs(ref).max()
