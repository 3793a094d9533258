"""armando_cell_ids_noalloc: the allocation-free cell-id entry point.

It exists for callers that must not allocate device memory (a host code whose
memory pool owns the GPU, a time loop that cannot take cudaMalloc's device
synchronisation). Its scratch lives in a static device array, so this test
checks, through the C-ABI, that two and more calls in a row (the array keeps
the previous call's contents) give exactly the cell ids of the allocating
entry point armando_cell_ids, and that sizes beyond its limit are refused.
Kept in a file pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import _abi, cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from armando_gb300 import build

    build.build_library()
    return ag.load_library()


def _noalloc(lib, case):
    import torch

    x = torch.from_numpy(case.x).cuda()
    h = torch.from_numpy(case.h).cuda()
    out = torch.full((case.n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.armando_cell_ids_noalloc(C.byref(case.params), C.c_void_p(x.data_ptr()),
                                      C.c_void_p(h.data_ptr()), case.n,
                                      C.c_void_p(out.data_ptr()), None)
    assert st == _abi.OK, lib.armando_last_error(None)
    return out.cpu().numpy()


def _reference(case):
    with ag.Context(case.params, case.n_fluid, case.n_wall) as ctx:
        return ctx.cell_ids(case.x, case.h)


def test_noalloc_cell_ids_equal_allocating_entry_point(lib):
    runs = [cases.dam_break(dx=0.02),
            cases.channel(n_x=40, n_yz=12, length=40 * 7.9e-4, width=12 * 7.9e-4, layers=3,
                          jitter=0.01),
            cases.cavity(),
            cases.dam_break(dx=0.02)]
    for c in runs:  # consecutive calls share (and overwrite) the static scratch
        got = _noalloc(lib, c)
        assert np.array_equal(got, _reference(c)), c.name


def test_noalloc_rejects_sizes_beyond_its_limit(lib):
    c = cases.cavity()
    st = lib.armando_cell_ids_noalloc(C.byref(c.params), None, None, (1 << 30) + 1, None, None)
    assert st == _abi.ERR_INVALID_ARG
    assert b"2^30" in lib.armando_last_error(None)
    st = lib.armando_cell_ids_noalloc(C.byref(c.params), None, None, -1, None, None)
    assert st == _abi.ERR_INVALID_ARG


def test_cell_ids_keep_link_list_grid_under_any_tuning(lib, O):
    """A tuning with a sort skin (or a wider reach) changes the step's cells but
    not the cell ids either entry point returns: both stay link_list's grid."""
    c = cases.dam_break(dx=0.02)
    _, _, ref, _ = O.link_list(c.x, c.h, c.dim, fp32=True, params=c.params)
    for tuning in ((1, 1, 128, 10), (3, 1, 256, 40), (2, 2, 128, 20)):
        with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
            ctx.set_tuning(*tuning)
            got = ctx.cell_ids(c.x, c.h)
        assert np.array_equal(got.astype(np.int64), ref), tuning
        assert np.array_equal(_noalloc(lib, c), got), tuning
