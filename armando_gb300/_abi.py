"""ctypes mirror of ``include/armando.h`` and the loader of the native library.

The structs here are byte-for-byte the C structs of the header; the loader
fails loudly when the compiled CUDA library is missing (there is no CPU path).
"""
from __future__ import annotations

import ctypes as C
import math
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libarmando_gb300.so")

# armando_status
OK = 0
ERR_INVALID_ARG = 1
ERR_OOM = 2
ERR_GRID_OVERFLOW = 3
ERR_NONFINITE = 4
ERR_OUT_OF_GRID = 5
ERR_TIMEOUT = 6
ERR_CUDA = 7
ERR_NO_DEVICE = 8
ERR_UNSUPPORTED = 9
ERR_IO = 10

STATUS_NAMES = {
    OK: "OK", ERR_INVALID_ARG: "INVALID_ARG", ERR_OOM: "OOM",
    ERR_GRID_OVERFLOW: "GRID_OVERFLOW", ERR_NONFINITE: "NONFINITE",
    ERR_OUT_OF_GRID: "OUT_OF_GRID", ERR_TIMEOUT: "TIMEOUT", ERR_CUDA: "CUDA",
    ERR_NO_DEVICE: "NO_DEVICE", ERR_UNSUPPORTED: "UNSUPPORTED", ERR_IO: "IO",
}

MEM_HOST = 0
MEM_DEVICE = 1

F3 = C.c_float * 3
I3 = C.c_int32 * 3


class Params(C.Structure):
    """``armando_params``: physics constants of the step."""

    _fields_ = [
        ("dim", C.c_int32),
        ("pa_sph", C.c_int32),
        ("visc", C.c_int32),
        ("visc_artificial", C.c_int32),
        ("heat_artificial", C.c_int32),
        ("heat_external", C.c_int32),
        ("kernel_3d_legacy", C.c_int32),
        ("periodic", I3),
        ("rho0", C.c_float),
        ("c0", C.c_float),
        ("pmin", C.c_float),
        ("eta", C.c_float),
        ("av_alpha", C.c_float),
        ("av_beta", C.c_float),
        ("av_eta", C.c_float),
        ("ah_g1", C.c_float),
        ("ah_g2", C.c_float),
        ("ah_eta", C.c_float),
        ("gravity", F3),
        ("heat_q0", C.c_float),
        ("heat_sigma", C.c_float),
        ("heat_center", F3),
        ("heat_t_end", C.c_float),
        ("period_lo", F3),
        ("period_hi", F3),
        ("wall_model", C.c_int32),
        ("scheme", C.c_int32),
        ("density_form", C.c_int32),
        ("average_velocity", C.c_int32),
        ("sle", C.c_int32),
    ]

    @classmethod
    def default(cls, **kw) -> "Params":
        """Reference defaults (art_visc.f:38-44, art_heat.f:38-40), overridable."""
        p = cls()
        p.dim = 2
        p.pa_sph = 1
        p.rho0 = 1000.0
        p.c0 = 1.0
        p.pmin = -math.inf
        p.av_alpha, p.av_beta, p.av_eta = 1.0, 1.0, 0.1
        p.ah_g1, p.ah_g2, p.ah_eta = 0.1, 1.0, 0.1
        p.heat_sigma = 1.0
        p.heat_t_end = math.inf
        for k, v in kw.items():
            p.set(k, v)
        return p

    def set(self, key, value):
        if key in ("periodic", "gravity", "heat_center", "period_lo", "period_hi"):
            arr = getattr(self, key)
            for i in range(3):
                arr[i] = value[i] if i < len(value) else 0
        else:
            setattr(self, key, value)
        return self

    def copy(self) -> "Params":
        q = Params()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(Params))
        return q

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class Material(C.Structure):
    """``armando_material``: EOS type and properties of one material of the
    GPU-C schemes (0 boundary, 1 ideal gas, 2 polynomial, 3 shock, 4 Tait, 5 ESS)."""

    _fields_ = [("eos", C.c_int32), ("prop", C.c_float * 10)]

    @classmethod
    def make(cls, eos, prop=()):
        m = cls()
        m.eos = eos
        for k, v in enumerate(prop):
            m.prop[k] = v
        return m


EOS_BOUNDARY, EOS_GAS, EOS_POLY, EOS_SHOCK, EOS_TAIT, EOS_ESS = range(6)


class Inlet(C.Structure):
    """``armando_inlet``: an inflow disk (3D) or segment (2D) of the GPU-C schemes."""

    _fields_ = [("origin", F3), ("normal", F3), ("radius", C.c_float), ("itype", C.c_int32),
                ("mass", C.c_float), ("hsml", C.c_float), ("speed", C.c_float),
                ("rho", C.c_float), ("u", C.c_float)]

    @classmethod
    def make(cls, origin, normal, radius, itype, mass, hsml, speed, rho, u=0.0):
        i = cls()
        for d in range(3):
            i.origin[d] = origin[d] if d < len(origin) else 0.0
            i.normal[d] = normal[d] if d < len(normal) else 0.0
        i.radius, i.itype, i.mass, i.hsml, i.speed, i.rho, i.u = radius, itype, mass, hsml, speed, rho, u
        return i


class Outlet(C.Structure):
    """``armando_outlet``: particles behind its plane within its radius leave."""

    _fields_ = [("origin", F3), ("normal", F3), ("radius", C.c_float)]

    @classmethod
    def make(cls, origin, normal, radius):
        o = cls()
        for d in range(3):
            o.origin[d] = origin[d] if d < len(origin) else 0.0
            o.normal[d] = normal[d] if d < len(normal) else 0.0
        o.radius = radius
        return o


MAX_OPEN = 10


def _box(z, lo, hi):
    for d in range(3):
        z.lo[d] = lo[d] if d < len(lo) else -float("inf")
        z.hi[d] = hi[d] if d < len(hi) else float("inf")


class LoadZone(C.Structure):
    """``armando_load_zone``: inside the open box lo < x < hi a particle with
    itype > 0 gains accel on dv/dt and w on de/dt."""

    _fields_ = [("lo", F3), ("hi", F3), ("accel", F3), ("w", C.c_float)]

    @classmethod
    def make(cls, lo, hi, accel=(0.0, 0.0, 0.0), w=0.0):
        z = cls()
        _box(z, lo, hi)
        for d in range(3):
            z.accel[d] = accel[d] if d < len(accel) else 0.0
        z.w = w
        return z


class FixZone(C.Structure):
    """``armando_fix_zone``: inside the open box a particle takes velocity vel
    after each stage's update (tau = 0), or relaxes towards it, dv/dt +=
    (vel - v) / tau, in every rate evaluation (tau > 0: a pump zone)."""

    _fields_ = [("lo", F3), ("hi", F3), ("vel", F3), ("tau", C.c_float)]

    @classmethod
    def make(cls, lo, hi, vel, tau=0.0):
        z = cls()
        _box(z, lo, hi)
        for d in range(3):
            z.vel[d] = vel[d] if d < len(vel) else 0.0
        z.tau = tau
        return z


MAX_ZONES = 10
MAX_MATERIALS = 64


class ParamGrads(C.Structure):
    """``armando_param_grads``."""

    _fields_ = [("av_alpha", C.c_double), ("av_beta", C.c_double), ("c0", C.c_double),
                ("heat_q0", C.c_double)]


class Tuning(C.Structure):
    """``armando_tuning``: neighbour-grid reach (cells per support radius),
    threads per particle, threads per CTA of the pair passes and the sort skin
    (percent of max h)."""

    _fields_ = [("reach", C.c_int32), ("threads_per_particle", C.c_int32), ("block", C.c_int32),
                ("skin", C.c_int32)]

    @classmethod
    def make(cls, reach=1, threads_per_particle=1, block=128, skin=0):
        return cls(reach, threads_per_particle, block, skin)

    def as_tuple(self):
        return (self.reach, self.threads_per_particle, self.block, self.skin)


class Stats(C.Structure):
    """``armando_stats``."""

    _fields_ = [
        ("steps_done", C.c_int64),
        ("n_particles", C.c_int64),
        ("n_cells", C.c_int64),
        ("cell_capacity", C.c_int64),
        ("gpu_launches", C.c_int64),
        ("grid_dims", I3),
        ("grid_origin", F3),
        ("grid_cell_size", F3),
        ("device_flags", C.c_uint32),
        ("sorts_done", C.c_int64),
        ("ghosts", C.c_int64),
    ]


# Every symbol include/armando.h declares (checked by the CPU test suite).
EXPORTED = [
    "armando_params_default", "armando_create", "armando_set_params",
    "armando_step", "armando_integrate", "armando_cell_ids",
    "armando_neighbours", "armando_sync", "armando_get_stats",
    "armando_last_error", "armando_destroy", "armando_abi_version", "armando_binary_version",
    "armando_set_stream",
    "armando_get_stream", "armando_profile_phases", "armando_cell_ids_noalloc",
    "armando_batch_create", "armando_batch_integrate",
    "armando_forward_checkpointed", "armando_backward",
    "armando_get_tuning", "armando_set_tuning", "armando_tuning_candidate", "armando_autotune",
    "armando_batch_autotune",
    "armando_deck_count", "armando_deck_read", "armando_deck_write", "armando_write_vtk",
    "armando_set_materials", "armando_get_hsml", "armando_set_open_boundaries",
    "armando_integrate_open", "armando_set_zones",
]
N_TUNINGS = 27
N_PHASES = 6
PHASE_NAMES = ["grid_hash", "radix_sort", "cells_reorder", "density", "shear", "force"]

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads the compiled sm_103a library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"armando_gb300 native library not found at {path}; "
            "run `python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = C.CDLL(path)
    fp = C.POINTER(C.c_float)
    ip = C.POINTER(C.c_int32)
    vp = C.c_void_p
    lib.armando_params_default.argtypes = [C.POINTER(Params)]
    lib.armando_params_default.restype = None
    lib.armando_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Params), C.c_int32,
                                   C.c_int64, C.c_int64, C.c_int32]
    lib.armando_create.restype = C.c_int
    lib.armando_set_params.argtypes = [vp, C.POINTER(Params)]
    lib.armando_set_params.restype = C.c_int
    step_args = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_float, C.c_int32]
    lib.armando_step.argtypes = step_args
    lib.armando_step.restype = C.c_int
    lib.armando_integrate.argtypes = step_args + [C.c_int32]
    lib.armando_integrate.restype = C.c_int
    lib.armando_cell_ids.argtypes = [vp, vp, vp, vp]
    lib.armando_cell_ids.restype = C.c_int
    lib.armando_neighbours.argtypes = [vp, vp, vp, vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    lib.armando_neighbours.restype = C.c_int
    lib.armando_sync.argtypes = [vp]
    lib.armando_sync.restype = C.c_int
    lib.armando_get_stats.argtypes = [vp, C.POINTER(Stats)]
    lib.armando_get_stats.restype = C.c_int
    lib.armando_last_error.argtypes = [vp]
    lib.armando_last_error.restype = C.c_char_p
    lib.armando_destroy.argtypes = [vp]
    lib.armando_destroy.restype = C.c_int
    lib.armando_abi_version.argtypes = []
    lib.armando_abi_version.restype = C.c_int32
    lib.armando_binary_version.argtypes = [ip]
    lib.armando_binary_version.restype = C.c_int
    lib.armando_set_stream.argtypes = [vp, vp]
    lib.armando_set_stream.restype = C.c_int
    lib.armando_get_stream.argtypes = [vp, C.POINTER(C.c_void_p)]
    lib.armando_get_stream.restype = C.c_int
    lib.armando_profile_phases.argtypes = [vp, C.c_int32, C.POINTER(C.c_float)]
    lib.armando_profile_phases.restype = C.c_int
    lib.armando_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(Params),
                                         C.c_int32, vp, vp, C.c_int32]
    lib.armando_batch_create.restype = C.c_int
    lib.armando_batch_integrate.argtypes = [vp] * 11 + [vp, C.c_int32, C.c_int32]
    lib.armando_batch_integrate.restype = C.c_int
    lib.armando_forward_checkpointed.argtypes = step_args + [C.c_int32, C.c_int32]
    lib.armando_forward_checkpointed.restype = C.c_int
    lib.armando_backward.argtypes = [vp] * 12 + [C.POINTER(ParamGrads)]
    lib.armando_backward.restype = C.c_int
    lib.armando_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    lib.armando_get_tuning.restype = C.c_int
    lib.armando_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    lib.armando_set_tuning.restype = C.c_int
    lib.armando_tuning_candidate.argtypes = [C.c_int32, C.POINTER(Tuning)]
    lib.armando_tuning_candidate.restype = C.c_int
    lib.armando_autotune.argtypes = [vp] * 11 + [C.c_float, C.c_int32, C.c_int32,
                                                 C.POINTER(Tuning), C.POINTER(C.c_float)]
    lib.armando_autotune.restype = C.c_int
    lib.armando_batch_autotune.argtypes = [vp] * 12 + [C.c_int32, C.c_int32,
                                                       C.POINTER(Tuning), C.POINTER(C.c_float)]
    lib.armando_batch_autotune.restype = C.c_int
    lib.armando_cell_ids_noalloc.argtypes = [C.POINTER(Params), vp, vp, C.c_int64, vp, vp]
    lib.armando_cell_ids_noalloc.restype = C.c_int
    cp = C.c_char_p
    lib.armando_deck_count.argtypes = [cp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.armando_deck_count.restype = C.c_int
    lib.armando_deck_read.argtypes = [cp, C.c_int32, C.c_int64, C.c_int64] + [vp] * 8
    lib.armando_deck_read.restype = C.c_int
    lib.armando_deck_write.argtypes = [cp, C.c_int32, C.c_int64, C.c_int64] + [vp] * 8
    lib.armando_deck_write.restype = C.c_int
    lib.armando_write_vtk.argtypes = [cp, C.c_int32, C.c_int64] + [vp] * 6
    lib.armando_write_vtk.restype = C.c_int
    lib.armando_set_materials.argtypes = [vp, C.c_int32, C.POINTER(Material)]
    lib.armando_set_materials.restype = C.c_int
    lib.armando_get_hsml.argtypes = [vp, vp]
    lib.armando_get_hsml.restype = C.c_int
    lib.armando_set_open_boundaries.argtypes = [vp, C.c_int32, C.POINTER(Inlet), C.c_int32,
                                                C.POINTER(Outlet), vp, vp]
    lib.armando_set_open_boundaries.restype = C.c_int
    lib.armando_integrate_open.argtypes = [vp] * 11 + [C.c_float, C.c_int32, C.c_int32,
                                                      C.POINTER(C.c_int64)]
    lib.armando_integrate_open.restype = C.c_int
    lib.armando_set_zones.argtypes = [vp, C.c_int32, C.POINTER(LoadZone), C.c_int32, C.POINTER(FixZone)]
    lib.armando_set_zones.restype = C.c_int
    del fp, ip
    _lib = lib
    return lib
