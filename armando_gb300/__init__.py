"""armando_gb300: GB300 (sm_103a) weakly-compressible SPH step of Armando.

Python host mirror of the reference's step interface over the C-ABI in
``include/armando.h``. ``Context.step`` is one iteration of the
``do its = 1, steps`` loop of CERNsource/time_integration.f:131-235 (what
``single_step`` plus the leapfrog update do there); ``Context.integrate`` is
``time_integration`` with ``refresh_step = 1`` and no file output.

All compute runs in the compiled CUDA library; importing the package does not
load it, creating a Context does, and fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import (ERR_UNSUPPORTED, EXPORTED, LIB_PATH, MEM_DEVICE, MEM_HOST, OK,  # noqa: F401
                   N_TUNINGS, STATUS_NAMES, ParamGrads, Params, Stats, Tuning, load_library)

__all__ = ["Context", "Batch", "Params", "Stats", "ArmandoError", "load_library", "MEM_HOST",
           "MEM_DEVICE", "LIB_PATH", "EXPORTED", "read_deck", "write_deck", "write_vtk"]


class ArmandoError(RuntimeError):
    """A non-OK armando_status; ``status`` holds the code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    if hasattr(a, "data_ptr"):  # torch tensor (device memory kind)
        return C.c_void_p(a.data_ptr())
    raise TypeError(f"unsupported array type {type(a)}")


def _check_host(a, n, dtype, name):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous numpy {np.dtype(dtype).name} array")
    if a.size != n:
        raise ValueError(f"{name} has {a.size} elements, expected {n}")


def _sized(a, n, dtype, name):
    """a as a C-contiguous host array of dtype with exactly n elements (the C
    side reads n of them)."""
    a = np.ascontiguousarray(a, dtype)
    if a.size != n:
        raise ValueError(f"{name} has {a.size} elements, expected {n}")
    return a


class Context:
    """One particle system on the current CUDA device (``armando_create``)."""

    def __init__(self, params: Params, n_fluid: int, n_wall: int, mem: int = MEM_HOST):
        self._lib = load_library()
        self.params = params.copy()
        self.dim = int(params.dim)
        self.n = int(n_fluid) + int(n_wall)
        self.mem = mem
        h = C.c_void_p()
        st = self._lib.armando_create(C.byref(h), C.byref(self.params), self.dim, int(n_fluid),
                                      int(n_wall), mem)
        if st != OK:
            raise ArmandoError(st, self._lib.armando_last_error(None).decode())
        self._h = h

    @classmethod
    def _from_handle(cls, lib, h, params, dim, n, mem):
        self = cls.__new__(cls)
        self._lib, self._h, self.params, self.dim, self.n, self.mem = lib, h, params, dim, n, mem
        return self

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.armando_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        if st != OK:
            raise ArmandoError(st, self._lib.armando_last_error(self._h).decode())

    # -- the step ------------------------------------------------------------
    def _validate(self, arrs):
        if self.mem != MEM_HOST:
            return
        n, nd = self.n, self.n * self.dim
        for name, size, dt in (("x", nd, np.float32), ("v", nd, np.float32),
                               ("mass", n, np.float32), ("rho", n, np.float32),
                               ("p", n, np.float32), ("u", n, np.float32), ("h", n, np.float32),
                               ("itype", n, np.int32), ("dvdt", nd, np.float32),
                               ("dudt", n, np.float32)):
            _check_host(arrs[name], size, dt, name)

    def set_params(self, params: Params):
        self._check(self._lib.armando_set_params(self._h, C.byref(params)))
        self.params = params.copy()

    def step(self, s, dt: float, its: int, wait: bool = True):
        """One leapfrog iteration `its` on state `s` (a Case or dict of arrays), in
        place. With device memory the C call is asynchronous; ``wait`` then
        blocks for it and raises its device status (``armando_sync``)."""
        a = s.arrays() if hasattr(s, "arrays") else s
        self._validate(a)
        self._check(self._lib.armando_step(self._h, _ptr(a["x"]), _ptr(a["v"]), _ptr(a["mass"]),
                                           _ptr(a["rho"]), _ptr(a["p"]), _ptr(a["u"]),
                                           _ptr(a["h"]), _ptr(a["itype"]), _ptr(a["dvdt"]),
                                           _ptr(a["dudt"]), float(dt), int(its)))
        if wait and self.mem == MEM_DEVICE:
            self.sync()
        return s

    def integrate(self, s, dt: float, its0: int, steps: int, wait: bool = True):
        """`steps` leapfrog iterations its0.. on state `s`, in place (``wait`` as
        for step)."""
        a = s.arrays() if hasattr(s, "arrays") else s
        self._validate(a)
        self._check(self._lib.armando_integrate(self._h, _ptr(a["x"]), _ptr(a["v"]),
                                                _ptr(a["mass"]), _ptr(a["rho"]), _ptr(a["p"]),
                                                _ptr(a["u"]), _ptr(a["h"]), _ptr(a["itype"]),
                                                _ptr(a["dvdt"]), _ptr(a["dudt"]), float(dt),
                                                int(its0), int(steps)))
        if wait and self.mem == MEM_DEVICE:
            self.sync()
        return s

    # -- reverse mode -----------------------------------------------------------
    def forward_checkpointed(self, s, dt: float, its0: int, steps: int, checkpoint_every: int):
        """armando_integrate keeping a checkpoint every `checkpoint_every` iterations."""
        a = s.arrays() if hasattr(s, "arrays") else s
        self._validate(a)
        self._check(self._lib.armando_forward_checkpointed(
            self._h, _ptr(a["x"]), _ptr(a["v"]), _ptr(a["mass"]), _ptr(a["rho"]), _ptr(a["p"]),
            _ptr(a["u"]), _ptr(a["h"]), _ptr(a["itype"]), _ptr(a["dvdt"]), _ptr(a["dudt"]),
            float(dt), int(its0), int(steps), int(checkpoint_every)))
        return s

    def backward(self, x_bar=None, v_bar=None, u_bar=None, p_bar=None, dvdt_bar=None,
                 dudt_bar=None):
        """Cotangents of the initial state and of the parameters for cotangents of the
        final state of the last forward_checkpointed (host memory kind: numpy)."""
        n, nd = self.n, self.n * self.dim
        ins = [None if a is None else _sized(a, size, np.float32, name)
               for a, size, name in ((x_bar, nd, "x_bar"), (v_bar, nd, "v_bar"), (u_bar, n, "u_bar"),
                                     (p_bar, n, "p_bar"), (dvdt_bar, nd, "dvdt_bar"),
                                     (dudt_bar, n, "dudt_bar"))]
        outs = {"x": np.zeros(nd, np.float32), "v": np.zeros(nd, np.float32),
                "u": np.zeros(n, np.float32), "dvdt": np.zeros(nd, np.float32),
                "dudt": np.zeros(n, np.float32)}
        g = ParamGrads()
        self._check(self._lib.armando_backward(
            self._h, *[_ptr(a) for a in ins], _ptr(outs["x"]), _ptr(outs["v"]), _ptr(outs["u"]),
            _ptr(outs["dvdt"]), _ptr(outs["dudt"]), C.byref(g)))
        outs["params"] = {"av_alpha": g.av_alpha, "av_beta": g.av_beta, "c0": g.c0,
                          "heat_q0": g.heat_q0}
        return outs

    # -- diagnostics ---------------------------------------------------------
    def cell_ids(self, x, h):
        """Cell id per particle (caller order) under the link_list grid of x."""
        out = np.zeros(self.n, np.int32) if self.mem == MEM_HOST else None
        if self.mem == MEM_HOST:
            x = _sized(x, self.n * self.dim, np.float32, "x")
            h = _sized(h, self.n, np.float32, "h")
        else:
            import torch
            out = torch.zeros(self.n, dtype=torch.int32, device="cuda")
        self._check(self._lib.armando_cell_ids(self._h, _ptr(x), _ptr(h), _ptr(out)))
        return out

    def neighbours(self, x, h):
        """CSR (offs[n+1], nbr) of neighbour sets j != i, ascending (host arrays)."""
        x = _sized(x, self.n * self.dim, np.float32, "x")
        h = _sized(h, self.n, np.float32, "h")
        offs = np.zeros(self.n + 1, np.int64)
        total = C.c_int64(0)
        st = self._lib.armando_neighbours(self._h, _ptr(x), _ptr(h), _ptr(offs), None, 0,
                                          C.byref(total))
        if st != OK and total.value == 0 and self.n > 0:
            self._check(st)
        nbr = np.zeros(max(total.value, 1), np.int32)
        self._check(self._lib.armando_neighbours(self._h, _ptr(x), _ptr(h), _ptr(offs), _ptr(nbr),
                                                 nbr.size, C.byref(total)))
        return offs, nbr[:total.value]

    def stats(self) -> Stats:
        st = Stats()
        self._check(self._lib.armando_get_stats(self._h, C.byref(st)))
        return st

    def stream_handle(self) -> int:
        """cudaStream_t of the context (for CUDA events around calls)."""
        sp = C.c_void_p()
        self._check(self._lib.armando_get_stream(self._h, C.byref(sp)))
        return sp.value or 0

    def profile_phases(self, steps: int) -> dict:
        """Mean ms per step of each phase over `steps` further steps (see header)."""
        from ._abi import N_PHASES, PHASE_NAMES
        out = (C.c_float * N_PHASES)()
        self._check(self._lib.armando_profile_phases(self._h, int(steps), out))
        return {PHASE_NAMES[k]: float(out[k]) for k in range(N_PHASES)}

    # -- tuning ----------------------------------------------------------------
    def tuning(self) -> Tuning:
        t = Tuning()
        self._check(self._lib.armando_get_tuning(self._h, C.byref(t)))
        return t

    def set_tuning(self, reach: int = 1, threads_per_particle: int = 1, block: int = 128,
                   skin: int = 0):
        t = Tuning.make(reach, threads_per_particle, block, skin)
        self._check(self._lib.armando_set_tuning(self._h, C.byref(t)))

    @staticmethod
    def tuning_candidates() -> list:
        lib = load_library()
        out = []
        for k in range(N_TUNINGS):
            t = Tuning()
            if lib.armando_tuning_candidate(k, C.byref(t)) != OK:
                raise ArmandoError(1, "armando_tuning_candidate failed")
            out.append(t.as_tuple())
        return out

    def autotune(self, s, dt: float, its0: int, steps_per_trial: int = 5):
        """Times every candidate tuning on state `s` (not modified), keeps the
        fastest; returns (best (reach, tpp, block, skin), {tuning: ms per step}).
        The skin candidates are keyed by the tuning they were timed with."""
        a = s.arrays() if hasattr(s, "arrays") else s
        self._validate(a)
        best = Tuning()
        ms = (C.c_float * N_TUNINGS)()
        self._check(self._lib.armando_autotune(
            self._h, _ptr(a["x"]), _ptr(a["v"]), _ptr(a["mass"]), _ptr(a["rho"]), _ptr(a["p"]),
            _ptr(a["u"]), _ptr(a["h"]), _ptr(a["itype"]), _ptr(a["dvdt"]), _ptr(a["dudt"]),
            float(dt), int(its0), int(steps_per_trial), C.byref(best), ms))
        cands = self.tuning_candidates()
        table = {}
        for k in range(N_TUNINGS):
            key = cands[k]
            if k >= 18:  # the skin on its reach's fastest skin-0 tuning
                same = [j for j in range(18) if cands[j][0] == key[0] and ms[j] > 0]
                if not same:
                    continue
                j = min(same, key=lambda j: ms[j])
                key = cands[j][:3] + (key[3],)
            table[key] = float(ms[k])
        return best.as_tuple(), table

    def set_open_boundaries(self, inlets=(), outlets=(), box=None):
        """Inlets and outlets of the GPU-C schemes (lists of _abi.Inlet and
        _abi.Outlet) and the box [lo, hi] outside which particles leave."""
        from ._abi import Inlet, Outlet

        tin = (Inlet * max(len(inlets), 1))(*inlets)
        tout = (Outlet * max(len(outlets), 1))(*outlets)
        lo = np.full(3, -3.0e38, np.float32)  # axes the box leaves out: unbounded
        hi = np.full(3, 3.0e38, np.float32)
        if box:
            lo[:len(box[0])] = box[0]
            hi[:len(box[1])] = box[1]
        self._check(self._lib.armando_set_open_boundaries(self._h, len(inlets), tin, len(outlets),
                                                          tout, _ptr(lo), _ptr(hi)))

    def integrate_open(self, arrays, dt: float, its0: int, steps: int, n: int) -> int:
        """`steps` GPU-C steps with the open boundaries on the first n particles of
        capacity-sized arrays (dict or Case); returns the particle count after."""
        a = arrays.arrays() if hasattr(arrays, "arrays") else arrays
        self._validate(a)
        cnt = C.c_int64(int(n))
        self._check(self._lib.armando_integrate_open(
            self._h, _ptr(a["x"]), _ptr(a["v"]), _ptr(a["mass"]), _ptr(a["rho"]), _ptr(a["p"]),
            _ptr(a["u"]), _ptr(a["h"]), _ptr(a["itype"]), _ptr(a["dvdt"]), _ptr(a["dudt"]),
            float(dt), int(its0), int(steps), C.byref(cnt)))
        return cnt.value

    def get_hsml(self, out=None):
        """Smoothing lengths after the last call, in caller order (evolved when
        params.sle != 0)."""
        if out is None:
            if self.mem == MEM_DEVICE:
                raise ValueError("pass a device array for a device-memory context")
            out = np.zeros(self.n, np.float32)
        self._check(self._lib.armando_get_hsml(self._h, _ptr(out)))
        return out

    def set_materials(self, materials):
        """Material table of the GPU-C schemes: a list of _abi.Material (or
        (eos, props) pairs), entry k for the particles with |itype| = k."""
        from ._abi import Material

        ms = [m if isinstance(m, Material) else Material.make(*m) for m in materials]
        tab = (Material * len(ms))(*ms)
        self._check(self._lib.armando_set_materials(self._h, len(ms), tab))

    def set_zones(self, loads=(), fixes=()):
        """Load and fix zones of the GPU-C schemes: lists of _abi.LoadZone and
        _abi.FixZone (``armando_set_zones``)."""
        from ._abi import FixZone, LoadZone

        lt = (LoadZone * max(len(loads), 1))(*loads)
        ft = (FixZone * max(len(fixes), 1))(*fixes)
        self._check(self._lib.armando_set_zones(self._h, len(loads), lt, len(fixes), ft))

    def sync(self):
        """Blocks for the context's stream; raises the device status of the
        asynchronous calls since the last report (``armando_sync``)."""
        self._check(self._lib.armando_sync(self._h))

    def set_stream(self, stream_handle: int):
        """Launch on the caller's cudaStream_t (0: the context's own stream)."""
        self._check(self._lib.armando_set_stream(self._h, C.c_void_p(int(stream_handle) or None)))


class Batch(Context):
    """Independent particle systems (a parameter sweep) in one context
    (``armando_batch_create``): packed arrays, one time step per instance."""

    def __init__(self, params_list, n_fluid, n_wall, mem: int = MEM_HOST):
        lib = load_library()
        k = len(params_list)
        arr = (Params * k)(*[p.copy() for p in params_list])
        nf = _sized(n_fluid, k, np.int64, "n_fluid")
        nw = _sized(n_wall, k, np.int64, "n_wall")
        dim = int(params_list[0].dim)
        h = C.c_void_p()
        st = lib.armando_batch_create(C.byref(h), k, arr, dim, nf.ctypes.data_as(C.c_void_p),
                                      nw.ctypes.data_as(C.c_void_p), mem)
        if st != OK:
            raise ArmandoError(st, lib.armando_last_error(None).decode())
        self._lib, self._h, self.params, self.dim = lib, h, params_list[0].copy(), dim
        self.n = int(nf.sum() + nw.sum())
        self.mem = mem
        self.n_instances = k
        self.counts = nf + nw
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)])

    def integrate_batch(self, s, dts, its0: int, steps: int, wait: bool = True):
        """`steps` iterations of every instance, dts[k] the time step of instance k
        (``wait`` as for Context.step)."""
        a = s.arrays() if hasattr(s, "arrays") else s
        self._validate(a)
        d = np.ascontiguousarray(dts, np.float32)
        if d.size != self.n_instances:
            raise ValueError("one dt per instance")
        self._check(self._lib.armando_batch_integrate(
            self._h, _ptr(a["x"]), _ptr(a["v"]), _ptr(a["mass"]), _ptr(a["rho"]), _ptr(a["p"]),
            _ptr(a["u"]), _ptr(a["h"]), _ptr(a["itype"]), _ptr(a["dvdt"]), _ptr(a["dudt"]),
            d.ctypes.data_as(C.c_void_p), int(its0), int(steps)))
        if wait and self.mem == MEM_DEVICE:
            self.sync()
        return s

    def autotune_batch(self, s, dts, its0: int, steps_per_trial: int = 5):
        """Times the candidate tunings that apply to a batch (one thread per
        particle, skin 0: the reach) on the packed state `s` (not modified),
        keeps the fastest; returns (best (reach, tpp, block, skin),
        {tuning: ms per step})."""
        a = s.arrays() if hasattr(s, "arrays") else s
        self._validate(a)
        d = np.ascontiguousarray(dts, np.float32)
        if d.size != self.n_instances:
            raise ValueError("one dt per instance")
        best = Tuning()
        ms = (C.c_float * N_TUNINGS)()
        self._check(self._lib.armando_batch_autotune(
            self._h, _ptr(a["x"]), _ptr(a["v"]), _ptr(a["mass"]), _ptr(a["rho"]), _ptr(a["p"]),
            _ptr(a["u"]), _ptr(a["h"]), _ptr(a["itype"]), _ptr(a["dvdt"]), _ptr(a["dudt"]),
            d.ctypes.data_as(C.c_void_p), int(its0), int(steps_per_trial), C.byref(best), ms))
        cands = self.tuning_candidates()
        return best.as_tuple(), {cands[k]: float(ms[k]) for k in range(N_TUNINGS) if ms[k] > 0}


# ---- particle decks and snapshots (host only) ------------------------------------

DECK_FIELDS = ("x", "v", "mass", "rho", "p", "u", "h", "itype")


def _io_check(lib, st):
    if st != OK:
        raise ArmandoError(st, lib.armando_last_error(None).decode())


def read_deck(directory: str, dim: int) -> dict:
    """CERN-F77 particle deck (f_*.dat, and v_*.dat when present) as step
    arrays: x, v, mass, rho, p, u, h (float32), itype (int32), the real
    particles first, plus the counts n_real and n_virtual."""
    lib = load_library()
    nr, nv = C.c_int64(), C.c_int64()
    d = str(directory).encode()
    _io_check(lib, lib.armando_deck_count(d, C.byref(nr), C.byref(nv)))
    n = nr.value + nv.value
    a = {f: np.zeros(n * dim if f in ("x", "v") else n, np.int32 if f == "itype" else np.float32)
         for f in DECK_FIELDS}
    _io_check(lib, lib.armando_deck_read(d, dim, nr.value, nv.value,
                                         *[_ptr(a[f]) for f in DECK_FIELDS]))
    a["n_real"], a["n_virtual"] = nr.value, nv.value
    return a


def write_deck(directory: str, dim: int, n_real: int, arrays) -> None:
    """Writes the arrays (real particles first, n_real of them) as a CERN-F77
    deck: f_*.dat for the real particles, v_*.dat for the rest."""
    lib = load_library()
    a = arrays.arrays() if hasattr(arrays, "arrays") else arrays
    n = int(np.asarray(a["mass"]).size)
    if not 0 <= n_real <= n:
        raise ValueError("n_real out of range")
    arrs = [_sized(a[f], n * (dim if f in ("x", "v") else 1), np.int32 if f == "itype" else np.float32, f)
            for f in DECK_FIELDS]
    _io_check(lib, lib.armando_deck_write(str(directory).encode(), dim, n_real, n - n_real,
                                          *[_ptr(q) for q in arrs]))


def write_vtk(path: str, dim: int, arrays) -> None:
    """Legacy ASCII VTK snapshot (the GPU-C code's outputVTK format)."""
    lib = load_library()
    a = arrays.arrays() if hasattr(arrays, "arrays") else arrays
    n = int(np.asarray(a["mass"]).size)
    arrs = [_sized(a[f], n * (dim if f in ("x", "v") else 1), np.int32 if f == "itype" else np.float32, f)
            for f in ("x", "v", "rho", "p", "u", "itype")]
    _io_check(lib, lib.armando_write_vtk(str(path).encode(), dim, n, *[_ptr(q) for q in arrs]))
