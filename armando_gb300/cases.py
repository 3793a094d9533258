"""Seeded synthetic workloads of the benchmark configurations.

The reference generates its inputs the same way (hard-coded lattices in
CERNsource/test_cases.f:577-761 and ArmandoThrust/acpu.c:1784-1902); no
dataset is involved. Every generator returns a :class:`Case` whose arrays are
FP32/int32 in the C-ABI layout (particle-major, ``x[i*dim + d]``).

Configurations (sizes are parameters so tests can shrink them):
  * :func:`cavity`      -- 2D shear-driven cavity, physical viscosity.
  * :func:`dam_break`   -- 2D dam break, artificial viscosity, gravity.
  * :func:`channel`     -- 3D heated channel, periodic x, art. visc + art. heat
                            + Gaussian volumetric source.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from ._abi import Params

G = 9.81


@dataclasses.dataclass
class Case:
    name: str
    params: Params
    dim: int
    x: np.ndarray        # float32 [n*dim]
    v: np.ndarray        # float32 [n*dim]
    mass: np.ndarray     # float32 [n]
    rho: np.ndarray      # float32 [n]
    p: np.ndarray        # float32 [n]
    u: np.ndarray        # float32 [n]
    h: np.ndarray        # float32 [n]
    itype: np.ndarray    # int32 [n]; > 0 fluid, <= 0 wall
    dt: float
    steps: int
    dvdt: np.ndarray = None  # float32 [n*dim] rates carried between steps
    dudt: np.ndarray = None  # float32 [n]
    meta: dict = dataclasses.field(default_factory=dict)

    def __post_init__(self):
        if self.dvdt is None:
            self.dvdt = np.zeros_like(self.x)
        if self.dudt is None:
            self.dudt = np.zeros_like(self.u)

    @property
    def n(self) -> int:
        return int(self.mass.shape[0])

    @property
    def n_fluid(self) -> int:
        return int(np.count_nonzero(self.itype > 0))

    @property
    def n_wall(self) -> int:
        return self.n - self.n_fluid

    def copy(self) -> "Case":
        c = dataclasses.replace(self)
        for f in ("x", "v", "mass", "rho", "p", "u", "h", "itype", "dvdt", "dudt"):
            setattr(c, f, getattr(self, f).copy())
        c.params = self.params.copy()
        c.meta = dict(self.meta)
        return c

    def arrays(self) -> dict:
        return {f: getattr(self, f) for f in
                ("x", "v", "mass", "rho", "p", "u", "h", "itype", "dvdt", "dudt")}


def wendland_w(r, h, dim, legacy3d=0):
    """Wendland C2 W(r, h) in FP64 (same formula as the library)."""
    q = np.asarray(r, dtype=np.float64) / h
    if dim == 2:
        a = 7.0 / (4.0 * math.pi * h * h)
    else:
        a = (15.0 if legacy3d else 21.0) / (16.0 * math.pi * h ** 3)
    t = np.clip(1.0 - 0.5 * q, 0.0, None)
    return np.where(q < 2.0, a * t ** 4 * (1.0 + 2.0 * q), 0.0)


def lattice_kernel_sum(dim: int, h_over_dx: float, legacy3d: int = 0) -> float:
    """sum_k W(|k| dx, h) dx^dim over a perfect lattice (self included), dx = 1."""
    h = float(h_over_dx)
    m = int(math.ceil(2 * h)) + 1
    ax = np.arange(-m, m + 1, dtype=np.float64)
    if dim == 2:
        X, Y = np.meshgrid(ax, ax, indexing="ij")
        r = np.sqrt(X * X + Y * Y)
    else:
        X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
        r = np.sqrt(X * X + Y * Y + Z * Z)
    return float(wendland_w(r, h, dim, legacy3d).sum())


def tait_rho_from_p(p, rho0, c0):
    return rho0 * (1.0 + 7.0 * np.asarray(p, np.float64) / (rho0 * c0 * c0)) ** (1.0 / 7.0)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def cavity(n_side: int = 40, seed: int = 1, length: float = 1.0e-3, lid_u: float = 1.0e-3,
           jitter: float = 0.01, steps: int = 3000) -> Case:
    """2D shear-driven cavity (reference case CERNsource/test_cases.f:577-761 with
    the configuration's Wendland/Tait physics): n_side^2 fluid particles in a
    square, 4*2*n_side wall particles at dx/2 spacing on its perimeter, moving
    lid on top; Tait c0 = 0.01 m/s, eta = 1e-3 Pa s, dt = 5e-5 s."""
    rng = np.random.default_rng(seed)
    dx = length / n_side
    h = 1.3 * dx
    rho0 = 1000.0
    i, j = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij")
    xf = np.stack([(i.ravel() + 0.5) * dx, (j.ravel() + 0.5) * dx], axis=1)
    xf += rng.uniform(-jitter, jitter, size=xf.shape) * dx
    k = np.arange(2 * n_side) * (dx / 2)
    bottom = np.stack([k, np.zeros_like(k)], 1)
    right = np.stack([np.full_like(k, length), k], 1)
    top = np.stack([length - k, np.full_like(k, length)], 1)
    left = np.stack([np.zeros_like(k), length - k], 1)
    xw = np.concatenate([bottom, right, top, left])
    vw = np.zeros_like(xw)
    vw[2 * (2 * n_side):3 * (2 * n_side), 0] = lid_u
    nf, nw = xf.shape[0], xw.shape[0]
    n = nf + nw
    P = Params.default(dim=2, pa_sph=1, visc=1, rho0=rho0, c0=0.01, eta=1.0e-3,
                       pmin=-math.inf)
    x = np.concatenate([xf, xw])
    v = np.concatenate([np.zeros_like(xf), vw])
    mass = np.concatenate([np.full(nf, rho0 * dx * dx), np.full(nw, 0.75 * rho0 * dx * dx)])
    return Case("cavity2d", P, 2, _f32(x.ravel()), _f32(v.ravel()), _f32(mass),
                _f32(np.full(n, rho0)), _f32(np.zeros(n)), _f32(np.zeros(n)),
                _f32(np.full(n, h)), np.concatenate([np.ones(nf), np.zeros(nw)]).astype(np.int32),
                dt=5.0e-5, steps=steps, meta=dict(dx=dx, seed=seed))


def dam_break(dx: float = 1.0e-3, col_w: float = 1.0, col_h: float = 2.0, tank_w: float = 4.0,
              tank_h: float = 3.0, layers: int = 3, jitter: float = 0.005, seed: int = 2,
              steps: int = 1000, alpha: float = 0.01, c0: float | None = None) -> Case:
    """2D dam break: a col_w x col_h water column at the left of a tank_w x tank_h
    tank, `layers` layers of fixed wall particles on the bottom and both sides.
    Hydrostatic initial density through the Tait EOS, masses scaled by the
    lattice kernel sum so summation density reproduces it; c0 = 10 sqrt(2 g H),
    dt = 0.2 h / c0, art. visc alpha = 0.01, beta = 0, gravity -9.81, pmin = 0.
    Defaults: dx = 1 mm, 1000 x 2000 = 2.0 M fluid + 30,018 wall particles."""
    rng = np.random.default_rng(seed)
    h = 1.3 * dx
    rho0 = 1000.0
    if c0 is None:
        c0 = 10.0 * math.sqrt(2.0 * G * col_h)
    nx, ny = int(round(col_w / dx)), int(round(col_h / dx))
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    xf = np.stack([(i.ravel() + 0.5) * dx, (j.ravel() + 0.5) * dx], axis=1)
    xf += rng.uniform(-jitter, jitter, size=xf.shape) * dx
    ntx, nty = int(round(tank_w / dx)), int(round(tank_h / dx))
    walls = []
    for kk in range(layers):
        bx = (np.arange(-layers, ntx + layers) + 0.5) * dx
        walls.append(np.stack([bx, np.full_like(bx, -(kk + 0.5) * dx)], 1))
    sy = (np.arange(nty) + 0.5) * dx
    for kk in range(layers):
        walls.append(np.stack([np.full_like(sy, -(kk + 0.5) * dx), sy], 1))
        walls.append(np.stack([np.full_like(sy, tank_w + (kk + 0.5) * dx), sy], 1))
    xw = np.concatenate(walls)
    x = np.concatenate([xf, xw])
    nf, nw = xf.shape[0], xw.shape[0]
    hloc = np.where(x[:, 0] <= col_w, col_h, 0.0)
    p = rho0 * G * np.maximum(0.0, hloc - x[:, 1])
    rho = tait_rho_from_p(p, rho0, c0)
    S = lattice_kernel_sum(2, 1.3)
    mass = rho * dx * dx / S
    P = Params.default(dim=2, pa_sph=1, visc=0, visc_artificial=1, rho0=rho0, c0=c0,
                       av_alpha=alpha, av_beta=0.0, av_eta=0.1, pmin=0.0,
                       gravity=(0.0, -G, 0.0))
    n = nf + nw
    return Case("dambreak2d", P, 2, _f32(x.ravel()), _f32(np.zeros(2 * n)), _f32(mass),
                _f32(rho), _f32(p), _f32(np.zeros(n)), _f32(np.full(n, h)),
                np.concatenate([np.ones(nf), np.zeros(nw)]).astype(np.int32),
                dt=0.2 * h / c0, steps=steps,
                meta=dict(dx=dx, seed=seed, nx=nx, ny=ny, c0=c0))


def channel(n_x: int = 504, n_yz: int = 126, length: float = 0.4, width: float = 0.1,
            layers: int = 3, seed: int = 3, steps: int = 500, u_in: float = 1.0,
            jitter: float = 0.0) -> Case:
    """3D heated liquid-metal channel, periodic in x, `layers` wall layers on the
    four y/z sides (no-slip, wall velocity 0). rho0 = 10500, c0 = 20 m/s,
    art. visc alpha = 0.02, art. heat g1 = g2 = 0.1, Gaussian source q0 = 1e8 W/m^3,
    sigma = 0.01 m centred at x = 0.1 m on the axis, cp = 146 J/(kg K), u = cp T,
    T = 600 K + N(0, 1 K). Default 504 x 126 x 126 = 8.0 M fluid particles."""
    rng = np.random.default_rng(seed)
    dx = length / n_x
    dyz = width / n_yz  # 0.4 / 504 vs 0.1 / 126: near-cubic cells
    h = 1.3 * dx
    rho0, c0, cp = 10500.0, 20.0, 146.0
    ix = np.arange(n_x)
    jy = np.arange(-layers, n_yz + layers)
    I, J, K = np.meshgrid(ix, jy, jy, indexing="ij")
    inside = (J >= 0) & (J < n_yz) & (K >= 0) & (K < n_yz)
    pos = np.stack([(I + 0.5) * dx, (J + 0.5) * dyz, (K + 0.5) * dyz], axis=-1)
    xf = pos[inside].reshape(-1, 3)
    xw = pos[~inside].reshape(-1, 3)
    if jitter:
        xf = xf + rng.uniform(-jitter, jitter, size=xf.shape) * dx
    nf, nw = xf.shape[0], xw.shape[0]
    n = nf + nw
    x = np.concatenate([xf, xw])
    v = np.zeros_like(x)
    v[:nf, 0] = u_in
    S = lattice_kernel_sum(3, 1.3)
    mass = np.full(n, rho0 * dx * dyz * dyz / S)
    T = np.concatenate([600.0 + rng.standard_normal(nf), np.full(nw, 600.0)])
    P = Params.default(dim=3, pa_sph=1, visc_artificial=1, heat_artificial=1, heat_external=1,
                       rho0=rho0, c0=c0, av_alpha=0.02, av_beta=0.0, av_eta=0.1,
                       ah_g1=0.1, ah_g2=0.1, ah_eta=0.1, heat_q0=1.0e8, heat_sigma=0.01,
                       heat_center=(0.1, width / 2, width / 2), pmin=-math.inf,
                       periodic=(1, 0, 0), period_lo=(0.0, 0.0, 0.0),
                       period_hi=(length, 0.0, 0.0))
    return Case("channel3d", P, 3, _f32(x.ravel()), _f32(v.ravel()), _f32(mass),
                _f32(np.full(n, rho0)), _f32(np.zeros(n)), _f32(cp * T),
                _f32(np.full(n, h)), np.concatenate([np.ones(nf), np.zeros(nw)]).astype(np.int32),
                dt=0.2 * h / c0, steps=steps, meta=dict(dx=dx, seed=seed, cp=cp))


def with_mirror_ghosts(case: Case, lo, hi) -> Case:
    """Copy of `case` for the mirror-ghost wall model (wall_model 3): every wall
    particle's velocity entry becomes its inward unit normal, as the CERN
    virtual-particle files carry it (CERNsource/input.f:256-314). The fluid
    region is lo[d] < x_d < hi[d] per axis (None: open); a wall particle on or
    beyond a bound takes the inward direction of that axis, on several axes (a
    corner) their normalised sum."""
    c = case.copy()
    dim = c.dim
    x = c.x.reshape(-1, dim).astype(np.float64)
    nrm = np.zeros_like(x)
    for d in range(dim):
        if lo[d] is not None:
            nrm[:, d] += x[:, d] <= lo[d]
        if hi[d] is not None:
            nrm[:, d] -= x[:, d] >= hi[d]
    wall = c.itype <= 0
    length = np.linalg.norm(nrm, axis=1)
    if np.any(wall & (length == 0)):
        raise ValueError("a wall particle lies inside the fluid region")
    v = c.v.reshape(-1, dim).copy()
    v[wall] = nrm[wall] / length[wall, None]
    c.v = _f32(v.ravel())
    c.params.wall_model = 3
    c.name = c.name + "_ghosts"
    return c


def perturbed(case: Case, seed: int, dv: float = 0.0, du: float = 0.0) -> Case:
    """Copy of `case` with seeded random fluid velocities (std dv) and energy (std du),
    used to give single-step parity tests non-trivial art_visc / art_heat terms."""
    c = case.copy()
    rng = np.random.default_rng(seed)
    fl = c.itype > 0
    if dv:
        vv = c.v.reshape(-1, c.dim)
        vv[fl] += rng.standard_normal((int(fl.sum()), c.dim)).astype(np.float32) * dv
        c.v = _f32(vv.ravel())
    if du:
        c.u[fl] += (rng.standard_normal(int(fl.sum())) * du).astype(np.float32)
    return c


def adjoint_dam_break(n_target: int = 250_000, seed: int = 5, v_std: float = 0.01) -> Case:
    """Reverse-mode workload: the 2D dam break above (same geometry and physics)
    with about `n_target` fluid particles (dx = sqrt(2 m^2 / n_target), 2.83 mm
    for 250k) and seeded initial fluid velocities N(0, v_std)."""
    dx = math.sqrt(2.0 / n_target)
    c = perturbed(dam_break(dx=dx, seed=seed), seed + 100, dv=v_std)
    c.name = "dambreak2d_adjoint"
    return c


# Probe of the reverse-mode loss (mean pressure over a 5 cm patch): centred 10 cm
# inside the column's right face, near the floor. On the face itself the
# surface particles sit at the pmin = 0 clamp of the EOS, where the loss has
# no derivative at FP32 resolution.
ADJOINT_PROBE = ((0.9, 0.05, 0.0), 0.05)


FIELDS = ("x", "v", "mass", "rho", "p", "u", "h", "itype", "dvdt", "dudt")


def pack(case_list):
    """Concatenates instances into the packed layout of a batch context.
    Returns (arrays dict, offsets[n_instances + 1])."""
    arrays = {f: np.ascontiguousarray(np.concatenate([getattr(c, f) for c in case_list]))
              for f in FIELDS}
    counts = np.array([c.n for c in case_list], np.int64)
    return arrays, np.concatenate([[0], np.cumsum(counts)])


def unpack(arrays, offsets, case_list):
    """Copies packed arrays back into per-instance Case objects (new copies)."""
    out = []
    for k, c in enumerate(case_list):
        d = c.copy()
        a, b = int(offsets[k]), int(offsets[k + 1])
        for f in FIELDS:
            src = arrays[f]
            w = c.dim if f in ("x", "v", "dvdt") else 1
            setattr(d, f, np.array(src[a * w:b * w]))
        out.append(d)
    return out


def sweep(n_instances: int = 512, seed: int = 4, n_min: float = 2.0e3, n_max: float = 2.0e5,
          steps: int = 500):
    """Batched parameter sweep: alternating 2D dam breaks and lid-driven
    cavities, particle counts log-uniform in [n_min, n_max], art. visc
    alpha ~ U(0.005, 0.05), c0 ~ U(20, 80) m/s, dam column aspect ~ U(0.5, 3);
    one seeded generator drives every draw. Returns a list of Case."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_instances):
        n_k = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        alpha = float(rng.uniform(0.005, 0.05))
        c0 = float(rng.uniform(20.0, 80.0))
        aspect = float(rng.uniform(0.5, 3.0))
        sub = int(rng.integers(1 << 30))
        if k % 2 == 0:
            dx = 1.0e-3
            nx = max(4, int(round(np.sqrt(n_k / aspect))))
            ny = max(4, int(round(aspect * nx)))
            c = dam_break(dx=dx, col_w=nx * dx, col_h=ny * dx, tank_w=4 * nx * dx,
                          tank_h=1.5 * ny * dx, seed=sub, steps=steps, alpha=alpha, c0=c0)
        else:
            side = max(4, int(round(np.sqrt(n_k))))
            c = cavity(n_side=side, seed=sub, length=1.0, lid_u=1.0, steps=steps)
            c.params.c0 = c0
            c.params.visc = 0
            c.params.visc_artificial = 1
            c.params.av_alpha = alpha
            c.params.av_beta = 0.0
            h = float(c.h[0])
            c.dt = 0.2 * h / c0
        c.name = f"{c.name}#{k}"
        c.meta.update(alpha=alpha, c0=c0, aspect=aspect, index=k)
        out.append(c)
    return out


def sweep_subset(case_list, smallest: int = 64, strata: int = 16):
    """Indices of the instances a CPU check of a sweep covers: the `smallest`
    instances by particle count, plus one instance from the middle of each of
    `strata` equal slices of the others in size order. Sorted ascending."""
    order = sorted(range(len(case_list)), key=lambda k: (case_list[k].n, k))
    pick = set(order[:smallest])
    rest = order[smallest:]
    for q in range(min(strata, len(rest))):
        pick.add(rest[int((q + 0.5) * len(rest) / strata)])
    return sorted(pick)


def gpuc_dam_break(scale: int = 1, fluid=(100, 50), tank=(269, 80), dr1: float = 0.02,
                   rho0: float = 1000.0, c0: float = 50.0, scheme: int = 1) -> Case:
    """The GPU-C codes' 2D dam break (the geometry of ArmandoThrust/acpu.c:
    1784-1902, the published Tab.1 cases): dr = dr1 / scale; a lattice of
    (fluid[0] scale + 1) x (fluid[1] scale + 1) water particles at
    ((i + 1/2) dr, (j + 1/2) dr); three rows of wall particles at integer
    lattice points under the tank (x from -3 dr to (tank[0] scale + 2) dr) and
    three columns on each side (left at -3..-1 dr, right from tank[0] scale dr,
    y from 0 to tank[1] scale dr). h = 1.2 dr, m = rho0 dr^2, rho = rho0, p = u
    = 0; water itype 1, walls -1 (both Tait rho0, c0 in the default material
    table); gravity -9.81; dt = 4e-4 s / scale. Scales 1, 2, 4 give the
    published 6,462 / 22,899 / 85,773 particles."""
    dr = dr1 / scale
    nfx, nfy = fluid[0] * scale + 1, fluid[1] * scale + 1
    i, j = np.meshgrid(np.arange(nfx), np.arange(nfy), indexing="ij")
    xf = np.stack([(i.ravel() + 0.5) * dr, (j.ravel() + 0.5) * dr], axis=1)
    ntx, nty = tank[0] * scale, tank[1] * scale
    walls = []
    bi = np.arange(-3, ntx + 3)
    for row in (-3, -2, -1):
        walls.append(np.stack([bi * dr, np.full(bi.shape, row * dr)], 1))
    sj = np.arange(0, nty + 1)
    for col in list(range(-3, 0)) + list(range(ntx, ntx + 3)):
        walls.append(np.stack([np.full(sj.shape, col * dr), sj * dr], 1))
    xw = np.concatenate(walls)
    x = np.concatenate([xf, xw])
    nf, n = len(xf), len(xf) + len(xw)
    h = 1.2 * dr
    P = Params.default(dim=2, rho0=rho0, c0=c0, gravity=(0.0, -G, 0.0))
    P.scheme = scheme
    return Case(f"gpuc_dambreak_x{scale}", P, 2, _f32(x.ravel()), _f32(np.zeros(2 * n)),
                _f32(np.full(n, rho0 * dr * dr)), _f32(np.full(n, rho0)), _f32(np.zeros(n)),
                _f32(np.zeros(n)), _f32(np.full(n, h)),
                np.concatenate([np.ones(nf), -np.ones(n - nf)]).astype(np.int32),
                dt=4.0e-4 / scale, steps=10000 * scale, meta=dict(dx=dr, scale=scale))


# Mercury for the pressure-wave workload: rho0 13,540 kg/m^3, c0 1,490 m/s and
# Grueneisen gamma 1.96 (the reference's mercury material, FORTRANsource/sph.f90:
# 158-163), as the GPU-C polynomial EOS {rho0, a1, a2, a3, b0, b1, t1, t2} with
# a1 = t1 = rho0 c0^2, b0 = gamma.
MERCURY_RHO0, MERCURY_C0, MERCURY_GAMMA = 13540.0, 1490.0, 1.96


def mercury_poly():
    """The polynomial-EOS material of the pressure-wave workload."""
    from ._abi import Material

    a1 = MERCURY_RHO0 * MERCURY_C0 ** 2
    return Material.make(2, [MERCURY_RHO0, a1, 0.0, 0.0, MERCURY_GAMMA, 0.0, a1, 0.0])


def gpuc_pressure_wave(n_side: int = 401, size: float = 0.1, radius: float = 4.0e-3,
                       e0: float = 1400.0, t_end: float = 1.0e-4, steps: int = None,
                       scheme: int = 1) -> Case:
    """Stand-in for the published pressure-wave workload of the GPU-C code
    (ArmandoOnGPU.pdf section 6.2, Tab.3): a square section of a mercury tank,
    `size` wide, free on every side (no walls), on an n_side x n_side lattice
    (401 / 501 / 601 give the published 160,801 / 251,001 / 361,201
    particles), with an instantaneous energy deposit at its centre, Gaussian
    around the axis: u = e0 exp(-(r / radius)^2). Polynomial EOS of mercury
    (`mercury_poly`, itype 1), h = 1.2 dr, m = rho0 dr^2, no gravity; `steps`
    (default 2 n_side, the published 800 / 1,000 / 1,200) cover t_end = 0.1 ms.
    The deposit's amplitude is not published: e0 = 1,400 J/kg is a 10 K rise
    (cp 140 J/(kg K))."""
    dr = size / (n_side - 1)
    i, j = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij")
    x = np.stack([i.ravel() * dr, j.ravel() * dr], 1) - 0.5 * size
    n = len(x)
    r2 = (x * x).sum(1)
    u = e0 * np.exp(-r2 / (radius * radius))
    steps = 2 * (n_side - 1) if steps is None else steps
    P = Params.default(dim=2, rho0=MERCURY_RHO0, c0=MERCURY_C0, gravity=(0.0, 0.0, 0.0))
    P.scheme = scheme
    return Case(f"gpuc_pressure_wave_{n_side}", P, 2, _f32(x.ravel()), _f32(np.zeros(2 * n)),
                _f32(np.full(n, MERCURY_RHO0 * dr * dr)), _f32(np.full(n, MERCURY_RHO0)),
                _f32(np.zeros(n)), _f32(u), _f32(np.full(n, 1.2 * dr)),
                np.ones(n, np.int32), dt=t_end / steps, steps=steps,
                meta=dict(dx=dr, n_side=n_side))


def gpuc_open_channel(length: float = 0.3, height: float = 0.1, dr: float = 0.01,
                      speed: float = 1.0, rho0: float = 1000.0, c0: float = 20.0,
                      capacity: int = 2000, scheme: int = 1):
    """A 2D open channel for the GPU-C open boundaries: water on a lattice
    ((i + 1/2) dr, (j + 1/2) dr) filling [0, length] x [0, height] at `speed`
    in +x, three wall rows under and over it (x from -3 dr to length + 3 dr),
    an inlet segment across the channel at x = -dr/2 (normal +x, radius
    height/2) emitting water at `speed`, an outlet at x = length (normal -x,
    radius height/2) and a box 10 dr around everything. Returns (case padded
    to `capacity`, n, inlets, outlets, box); h = 1.2 dr, dt = 0.2 h / c0."""
    from ._abi import Inlet, Outlet

    nx, ny = int(round(length / dr)), int(round(height / dr))
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    xf = np.stack([(i.ravel() + 0.5) * dr, (j.ravel() + 0.5) * dr], 1)
    wx = np.arange(-3, nx + 4) * dr
    walls = [np.stack([wx, np.full(wx.shape, y)], 1) for y in
             [-0.5 * dr, -1.5 * dr, -2.5 * dr, height + 0.5 * dr, height + 1.5 * dr, height + 2.5 * dr]]
    xw = np.concatenate(walls)
    x = np.concatenate([xf, xw])
    n, nf = len(x), len(xf)
    h = 1.2 * dr
    m = rho0 * dr * dr
    v = np.zeros_like(x)
    v[:nf, 0] = speed
    P = Params.default(dim=2, rho0=rho0, c0=c0)
    P.scheme = scheme

    def pad(a, width=1, dtype=np.float32):
        out = np.zeros(capacity * width, dtype)
        out[:a.size] = np.asarray(a, dtype).ravel()
        return out

    c = Case("gpuc_open_channel", P, 2, pad(x, 2), pad(v, 2), pad(np.full(n, m)),
             pad(np.full(n, rho0)), pad(np.zeros(n)), pad(np.zeros(n)), pad(np.full(n, h)),
             pad(np.concatenate([np.ones(nf), -np.ones(n - nf)]), 1, np.int32),
             dt=0.2 * h / c0, steps=200, meta=dict(dx=dr, n=n))
    inlets = [Inlet.make((-0.5 * dr, 0.5 * height, 0.0), (1.0, 0.0, 0.0), 0.5 * height, 1, m, h,
                         speed, rho0)]
    outlets = [Outlet.make((length, 0.5 * height, 0.0), (-1.0, 0.0, 0.0), 0.5 * height)]
    box = ((-10 * dr, -10 * dr, -1.0), (length + 10 * dr, height + 10 * dr, 1.0))
    return c, n, inlets, outlets, box
