"""ctypes wrapper of the CPU oracle (liboracle.so).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REPO = os.path.dirname(_HERE)
if _REPO not in sys.path:
    sys.path.insert(0, _REPO)

from armando_gb300._abi import FixZone, Inlet, LoadZone, Material, Outlet, Params  # noqa: E402  (shared C-ABI structs)

LIB_PATH = os.path.join(_HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(_HERE, "_ref", "libacpu.so")

_lib = None


class LossSpec(C.Structure):
    """L = w_ke sum m|v|^2/2 + w_p sum w(x) p / w_ref + w_u sum w(x) u / w_ref on the
    final state (p: pressure output of the last iteration), w(x) = (1 - |x - c|^2/R^2)^3
    inside radius R, fluid particles only."""

    _fields_ = [("w_ke", C.c_double), ("w_p", C.c_double), ("w_u", C.c_double),
                ("c", C.c_double * 3), ("radius", C.c_double), ("w_ref", C.c_double)]

    @classmethod
    def make(cls, w_ke=1.0, w_p=0.0, w_u=0.0, c=(0, 0, 0), radius=1.0, w_ref=1.0):
        l = cls()
        l.w_ke, l.w_p, l.w_u, l.radius, l.w_ref = w_ke, w_p, w_u, radius, w_ref
        for d in range(3):
            l.c[d] = c[d] if d < len(c) else 0.0
        return l


def build(force: bool = False) -> str:
    """Compiles liboracle.so with the committed Makefile."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        i64 = C.c_int64
        L.ao_link_list_f64.argtypes = [i64, C.c_int, vp, vp, vp, vp, vp, vp, vp, i64, vp, vp, C.c_int]
        L.ao_link_list_f64.restype = i64
        L.ao_link_list_f32.argtypes = L.ao_link_list_f64.argtypes
        L.ao_link_list_f32.restype = i64
        L.ao_kernel_f64.argtypes = [C.c_int, C.c_int, i64, vp, vp, vp, vp]
        L.ao_kernel_f64.restype = None
        L.ao_tait_f64.argtypes = [i64, vp, C.c_double, C.c_double, C.c_double, C.c_int, vp]
        L.ao_tait_f64.restype = None
        L.ao_forces_f64.argtypes = [C.POINTER(Params), i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.ao_forces_f64.restype = C.c_int
        L.ao_step_f64.argtypes = [C.POINTER(Params), i64, C.c_int, C.c_double, vp, vp, vp, vp, vp,
                                  vp, vp, vp, vp, vp, vp, C.c_int, vp]
        L.ao_step_f64.restype = C.c_int
        L.ao_step_f32.argtypes = [C.POINTER(Params), i64, C.c_int, C.c_double, vp, vp, vp, vp, vp,
                                  vp, vp, vp, vp, vp]
        L.ao_step_f32.restype = C.c_int
        L.ao_integrate_gather_f64.argtypes = [C.POINTER(Params), i64, C.c_int, C.c_int, C.c_double,
                                              vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int]
        L.ao_integrate_gather_f64.restype = C.c_int
        L.ao_loss_f64.argtypes = [C.POINTER(Params), i64, C.c_int, C.c_int, C.c_double] + \
            [vp] * 10 + [C.POINTER(LossSpec)]
        L.ao_loss_f64.restype = C.c_double
        L.ao_tangent_f64.argtypes = [C.POINTER(Params), i64, C.c_int, C.c_int, C.c_double] + \
            [vp] * 10 + [C.POINTER(LossSpec), vp, vp, vp, vp, vp]
        L.ao_tangent_f64.restype = C.c_int
        L.ao_flops_f64.argtypes = [C.POINTER(Params), i64, C.c_int, C.c_double] + [vp] * 11
        L.ao_flops_f64.restype = C.c_int
        zones = [C.c_int32, C.POINTER(LoadZone), C.c_int32, C.POINTER(FixZone)]
        L.ao_gpuc_step_f64.argtypes = [C.POINTER(Params), C.c_int32, C.POINTER(Material)] + zones + \
            [i64, C.c_int, C.c_double] + [vp] * 10 + [C.c_int]
        L.ao_gpuc_step_f64.restype = C.c_int
        L.ao_gpuc_rates_f64.argtypes = [C.POINTER(Params), C.c_int32, C.POINTER(Material), i64] + \
            [vp] * 11 + [C.c_int]
        L.ao_gpuc_rates_f64.restype = C.c_int
        L.ao_con_density_f64.argtypes = [C.POINTER(Params), i64] + [vp] * 7
        L.ao_con_density_f64.restype = C.c_int
        L.ao_gpuc_open_f64.argtypes = [C.POINTER(Params), C.c_int32, C.POINTER(Material)] + zones + \
                                      [C.c_int32, C.POINTER(Inlet), C.c_int32, C.POINTER(Outlet),
                                       vp, vp, i64, C.POINTER(i64), C.c_int, C.c_double] + \
            [vp] * 10 + [C.c_int]
        L.ao_gpuc_open_f64.restype = C.c_int
        L.ao_gpuc_eos_f64.argtypes = [C.POINTER(Material), i64, vp, vp, vp, vp, vp]
        L.ao_gpuc_eos_f64.restype = None
        L.ao_ghosts_f64.argtypes = [C.POINTER(Params), i64, vp, vp, vp, vp, C.c_int, vp, vp, vp, vp]
        L.ao_ghosts_f64.restype = i64
        L.ao_hardware_threads.argtypes = []
        L.ao_hardware_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _per(params: Params | None, dim: int):
    per = np.zeros(3, np.int32)
    lo = np.zeros(3, np.float64)
    hi = np.zeros(3, np.float64)
    if params is not None:
        for d in range(3):
            per[d] = params.periodic[d]
            lo[d] = params.period_lo[d]
            hi[d] = params.period_hi[d]
    return per, lo, hi


def link_list(x, h, dim, fp32=False, params=None, direct=False):
    """Pairs (i < j) by link_list / direct_find. Returns (pi, pj, cell_ids, grid)
    where grid = dict(o, size, n, ncells)."""
    dt = np.float32 if fp32 else np.float64
    x = np.ascontiguousarray(x, dt)
    h = np.ascontiguousarray(h, dt)
    n = h.shape[0]
    per, lo, hi = _per(params, dim)
    cid = np.zeros(n, np.int64)
    grid = np.zeros(10, np.float64)
    f = lib().ao_link_list_f32 if fp32 else lib().ao_link_list_f64
    npairs = f(n, dim, _p(x), _p(h), _p(per), _p(lo), _p(hi), None, None, 0, _p(cid), _p(grid),
               int(direct))
    if npairs < 0:
        raise RuntimeError("oracle link_list failed")
    pi = np.zeros(npairs, np.int32)
    pj = np.zeros(npairs, np.int32)
    f(n, dim, _p(x), _p(h), _p(per), _p(lo), _p(hi), _p(pi), _p(pj), npairs, None, None, int(direct))
    g = dict(o=grid[0:3].copy(), size=grid[3:6].copy(), n=grid[6:9].astype(np.int64),
             ncells=int(grid[9]))
    return pi, pj, cid, g


def kernel(r, h, dim, legacy3d=0):
    r = np.ascontiguousarray(r, np.float64)
    h = np.ascontiguousarray(np.broadcast_to(h, r.shape), np.float64)
    w = np.zeros_like(r)
    dw = np.zeros_like(r)
    lib().ao_kernel_f64(dim, legacy3d, r.size, _p(r), _p(h), _p(w), _p(dw))
    return w, dw


def tait(rho, rho0, c0, pmin=-np.inf, clamp=False):
    rho = np.ascontiguousarray(rho, np.float64)
    p = np.zeros_like(rho)
    lib().ao_tait_f64(rho.size, _p(rho), rho0, c0, pmin, int(clamp), _p(p))
    return p


def forces(params: Params, x, v, m, rho, p, u, h, itype):
    """int_force (+ art_visc) rates for given rho, p (FP64)."""
    d = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
    x, v, m, rho, p, u, h = map(d, (x, v, m, rho, p, u, h))
    itype = np.ascontiguousarray(itype, np.int32)
    n = m.shape[0]
    dim = params.dim
    dv = np.zeros(n * dim, np.float64)
    du = np.zeros(n, np.float64)
    rc = lib().ao_forces_f64(C.byref(params), n, _p(x), _p(v), _p(m), _p(rho), _p(p), _p(u),
                             _p(h), _p(itype), _p(dv), _p(du))
    if rc:
        raise RuntimeError("oracle forces failed")
    return dv, du


class State:
    """FP64 (or FP32) copy of a case's arrays for the oracle."""

    def __init__(self, case, dtype=np.float64):
        self.dim = case.dim
        self.params = case.params
        d = lambda a: np.array(a, dtype=dtype)  # noqa: E731
        self.x, self.v, self.m = d(case.x), d(case.v), d(case.mass)
        self.rho, self.p, self.u, self.h = d(case.rho), d(case.p), d(case.u), d(case.h)
        self.dvdt, self.dudt = d(case.dvdt), d(case.dudt)
        self.drho = np.zeros(self.m.shape[0], np.float64)  # carried drho/dt (continuity)
        self.itype = np.array(case.itype, np.int32)
        self.extra = None

    @property
    def n(self):
        return self.m.shape[0]


def step(state: State, its: int, dt: float, nbr_fp32: bool = False, extra: bool = False):
    """One leapfrog iteration of the pair-loop oracle (in place)."""
    n = state.n
    ex = np.zeros(2 * n, np.float64) if extra else None
    if state.x.dtype == np.float64:
        rc = lib().ao_step_f64(C.byref(state.params), n, its, dt, _p(state.x), _p(state.v),
                               _p(state.m), _p(state.rho), _p(state.p), _p(state.u), _p(state.h),
                               _p(state.itype), _p(state.dvdt), _p(state.dudt), _p(state.drho),
                               int(nbr_fp32), _p(ex) if extra else None)
    else:
        rc = lib().ao_step_f32(C.byref(state.params), n, its, dt, _p(state.x), _p(state.v),
                               _p(state.m), _p(state.rho), _p(state.p), _p(state.u), _p(state.h),
                               _p(state.itype), _p(state.dvdt), _p(state.dudt))
    if rc:
        raise RuntimeError("oracle step failed")
    if extra:
        state.extra = ex.reshape(n, 2)
    return state


def integrate_gather(state: State, its0: int, steps: int, dt: float, nthreads: int = 0):
    """`steps` iterations of the threaded FP64 gather form (in place)."""
    if nthreads <= 0:
        nthreads = lib().ao_hardware_threads()
    rc = lib().ao_integrate_gather_f64(C.byref(state.params), state.n, its0, steps, dt,
                                       _p(state.x), _p(state.v), _p(state.m), _p(state.rho),
                                       _p(state.p), _p(state.u), _p(state.h), _p(state.itype),
                                       _p(state.dvdt), _p(state.dudt), nthreads)
    if rc:
        raise RuntimeError("oracle gather integrate failed")
    return state


def ghosts(params: Params, x, v, h, itype, fp32=True):
    """Mirror ghosts (wall_model 3) of the given positions and velocities:
    (owner, wall, x_ghost [ng, dim], v_ghost [ng, dim])."""
    d = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
    x, v, h = d(x), d(v), d(h)
    itype = np.ascontiguousarray(itype, np.int32)
    n, dim = h.shape[0], params.dim
    owner = np.zeros(n, np.int64)
    wall = np.zeros(n, np.int64)
    xg = np.zeros(n * dim)
    vg = np.zeros(n * dim)
    ng = lib().ao_ghosts_f64(C.byref(params), n, _p(x), _p(v), _p(h), _p(itype), int(fp32),
                             _p(owner), _p(wall), _p(xg), _p(vg))
    if ng < 0:
        raise RuntimeError("oracle ghosts failed")
    return owner[:ng], wall[:ng], xg[:ng * dim].reshape(ng, dim), vg[:ng * dim].reshape(ng, dim)


def _zones(loads, fixes):
    return (len(loads), (LoadZone * max(len(loads), 1))(*loads), len(fixes),
            (FixZone * max(len(fixes), 1))(*fixes))


def gpuc_step(state: State, steps: int, dt: float, materials=None, fp32: bool = True, loads=(),
              fixes=()):
    """`steps` TVD-RK3 steps of the GPU-C scheme state.params.scheme (1 host-path,
    2 device-kernel physics), in place. materials: list of _abi.Material by
    |itype| (None: Tait with rho0, c0); loads, fixes: _abi.LoadZone / FixZone
    lists. Returns the last stage's (dvdt, dudt)."""
    n, dim = state.n, state.dim
    dv = np.zeros(n * dim)
    du = np.zeros(n)
    tab = None
    nmat = 0
    if materials is not None:
        nmat = len(materials)
        tab = (Material * nmat)(*materials)
    rc = lib().ao_gpuc_step_f64(C.byref(state.params), nmat, tab, *_zones(loads, fixes), n, steps, dt,
                                _p(state.x),
                                _p(state.v), _p(state.m), _p(state.rho), _p(state.p), _p(state.u),
                                _p(state.h), _p(state.itype), _p(dv), _p(du), int(fp32))
    if rc:
        raise RuntimeError("oracle gpuc step failed")
    return dv, du


def con_density(params: Params, x, v, m, rho, h, itype):
    """con_density (density.f:161-218): drho/dt of the fluid particles (FP64)."""
    d = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
    x, v, m, rho, h = map(d, (x, v, m, rho, h))
    it = np.ascontiguousarray(itype, np.int32)
    out = np.zeros(m.shape[0])
    rc = lib().ao_con_density_f64(C.byref(params), m.shape[0], _p(x), _p(v), _p(m), _p(rho),
                                  _p(h), _p(it), _p(out))
    if rc:
        raise RuntimeError("oracle con_density failed")
    return out


def gpuc_rates(params: Params, x, v, m, rho, p, u, h, itype, materials=None, fp32: bool = True):
    """Pair rates (drho/dt, dv/dt, de/dt) of the GPU-C scheme params.scheme at one
    state, p as given; the first stage of a step evaluates these."""
    f = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
    x, v, m, rho, p, u, h = (f(a) for a in (x, v, m, rho, p, u, h))
    it = np.ascontiguousarray(itype, np.int32)
    n, dim = m.shape[0], int(params.dim)
    drho, dv, du = np.zeros(n), np.zeros(n * dim), np.zeros(n)
    tab, nmat = None, 0
    if materials is not None:
        nmat = len(materials)
        tab = (Material * nmat)(*materials)
    rc = lib().ao_gpuc_rates_f64(C.byref(params), nmat, tab, n, _p(x), _p(v), _p(m), _p(rho),
                                 _p(p), _p(u), _p(h), _p(it), _p(drho), _p(dv), _p(du), int(fp32))
    if rc:
        raise RuntimeError("oracle gpuc rates failed")
    return drho, dv, du


def gpuc_open(case, steps, dt, capacity, n=None, inlets=(), outlets=(), box=None,
              materials=None, fp32=True, loads=(), fixes=()):
    """GPU-C steps with open boundaries from the first n particles of a case
    (FP32 arrays; n = all of them by default): returns a dict of FP64 arrays
    (x, v, mass, rho, p, u, h, itype, dvdt, dudt) of the particles left,
    survivors in input order then new ones in emission order."""
    dim = case.dim
    n0 = case.n if n is None else int(n)
    a = {}
    for f, w, dt_ in (("x", dim, np.float64), ("v", dim, np.float64), ("mass", 1, np.float64),
                      ("rho", 1, np.float64), ("p", 1, np.float64), ("u", 1, np.float64),
                      ("h", 1, np.float64), ("itype", 1, np.int32), ("dvdt", dim, np.float64),
                      ("dudt", 1, np.float64)):
        arr = np.zeros(capacity * w, dt_)
        src = np.asarray(getattr(case, f))[:n0 * w]
        arr[:src.size] = src
        a[f] = arr
    n = C.c_int64(n0)
    lo = np.full(3, -3.0e38, np.float32)
    hi = np.full(3, 3.0e38, np.float32)
    if box:
        lo[:len(box[0])] = box[0]
        hi[:len(box[1])] = box[1]
    tin = (Inlet * max(len(inlets), 1))(*inlets)
    tout = (Outlet * max(len(outlets), 1))(*outlets)
    tab, nmat = None, 0
    if materials is not None:
        nmat = len(materials)
        tab = (Material * nmat)(*materials)
    rc = lib().ao_gpuc_open_f64(C.byref(case.params), nmat, tab, *_zones(loads, fixes),
                                len(inlets), tin, len(outlets),
                                tout, _p(lo), _p(hi), capacity, C.byref(n), steps, dt,
                                *[_p(a[f]) for f in ("x", "v", "mass", "rho", "p", "u", "h",
                                                     "itype", "dvdt", "dudt")], int(fp32))
    if rc:
        raise RuntimeError(f"oracle open-boundary run failed ({rc})")
    k = n.value
    return {f: (v[:k * dim] if f in ("x", "v", "dvdt") else v[:k]) for f, v in a.items()}


def gpuc_eos(material, rho, u):
    """EOS of one GPU-C material: (rho after its clamp, p, c)."""
    rho = np.ascontiguousarray(rho, np.float64)
    u = np.ascontiguousarray(np.broadcast_to(u, rho.shape), np.float64)
    r, p, c = np.zeros_like(rho), np.zeros_like(rho), np.zeros_like(rho)
    lib().ao_gpuc_eos_f64(C.byref(material), rho.size, _p(rho), _p(u), _p(r), _p(p), _p(c))
    return r, p, c


def hardware_threads() -> int:
    return lib().ao_hardware_threads()


def flops(state: State, its: int, dt: float):
    """Operation count of iteration `its` of the reference algorithm on this
    state (not modified): (whole iteration, its link_list neighbour search)."""
    out = np.zeros(2)
    rc = lib().ao_flops_f64(C.byref(state.params), state.n, its, dt, *_state_args(state), _p(out))
    if rc:
        raise RuntimeError("oracle flop count failed")
    return float(out[0]), float(out[1])


def _state_args(state):
    return [_p(state.x), _p(state.v), _p(state.m), _p(state.rho), _p(state.p), _p(state.u),
            _p(state.h), _p(state.itype), _p(state.dvdt), _p(state.dudt)]


def loss(state: State, its0: int, steps: int, dt: float, spec: LossSpec, params=None) -> float:
    """FP64 loss after `steps` iterations (state is not modified)."""
    prm = params if params is not None else state.params
    return lib().ao_loss_f64(C.byref(prm), state.n, its0, steps, dt, *_state_args(state),
                             C.byref(spec))


def tangent(state: State, its0: int, steps: int, dt: float, spec: LossSpec, dparam=None,
            dx0=None, dv0=None, du0=None, params=None):
    """FP64 tangent-linear (L, dL) along the seed (dparam = d alpha, d beta, d c0, d q0)."""
    prm = params if params is not None else state.params
    out = np.zeros(2)
    dp = None if dparam is None else np.ascontiguousarray(dparam, np.float64)
    keep = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (dx0, dv0, du0)]
    rc = lib().ao_tangent_f64(C.byref(prm), state.n, its0, steps, dt, *_state_args(state),
                              C.byref(spec), None if dp is None else _p(dp),
                              *[None if a is None else _p(a) for a in keep], _p(out))
    if rc:
        raise RuntimeError("oracle tangent failed")
    return float(out[0]), float(out[1])
