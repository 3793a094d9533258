"""The C-ABI library: built for sm_103a, loads, exports exactly what
include/armando.h declares, and its ctypes mirror matches the C layout.
No compute calls (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

import armando_gb300 as ag
from armando_gb300 import _abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(REPO, "include", f) for f in sorted(os.listdir(os.path.join(REPO, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(armando_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from armando_gb300 import build

    build.build_library()
    return ag.load_library()


def test_header_declares_the_python_list():
    assert declared_functions() == sorted(_abi.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", ag.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s+(armando_\w+)", out))
    for name in declared_functions():
        assert name in exported, name
        assert hasattr(lib, name)


def test_library_built_for_sm103a_only():
    from armando_gb300 import build

    flags = " ".join(build.NVCC_FLAGS)
    assert "-gencode arch=compute_103a,code=sm_103a" in flags
    assert flags.count("-gencode") == 1


@pytest.mark.gpu
def test_device_code_is_sm103(lib):
    """cudaFuncGetAttributes of a library kernel: binaryVersion 103."""
    v = C.c_int32(0)
    assert lib.armando_binary_version(C.byref(v)) == _abi.OK, lib.armando_last_error(None)
    assert v.value == 103


def test_struct_layout_matches_c():
    code = r'''
#include <stdio.h>
#include <stddef.h>
#include "armando.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(armando_params), offsetof(armando_params, rho0),
         offsetof(armando_params, gravity), offsetof(armando_params, period_hi),
         sizeof(armando_stats), offsetof(armando_stats, device_flags),
         offsetof(armando_params, wall_model));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(src, "w").write(code)
        subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), src, "-o", exe], check=True)
        got = list(map(int, subprocess.run([exe], capture_output=True, text=True).stdout.split()))
    P, S = _abi.Params, _abi.Stats
    assert got == [C.sizeof(P), P.rho0.offset, P.gravity.offset, P.period_hi.offset,
                   C.sizeof(S), S.device_flags.offset, P.wall_model.offset]


def test_params_default_matches_python(lib):
    p = _abi.Params()
    lib.armando_params_default(C.byref(p))
    q = _abi.Params.default()
    assert p.as_dict() == q.as_dict()


def test_abi_version(lib):
    assert lib.armando_abi_version() == 2


def test_create_without_gpu_reports_status(lib):
    # On a machine without a GPU the call must fail with a status, not crash.
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present: covered by the gpu tests")
    h = C.c_void_p()
    p = _abi.Params.default()
    st = lib.armando_create(C.byref(h), C.byref(p), 2, 10, 0, 0)
    assert st == _abi.ERR_NO_DEVICE
    assert b"device" in lib.armando_last_error(None)


def test_tuning_candidates_enumerate_every_tuning(lib):
    got = []
    for k in range(_abi.N_TUNINGS):
        t = _abi.Tuning()
        assert lib.armando_tuning_candidate(k, C.byref(t)) == _abi.OK
        got.append(t.as_tuple())
    assert sorted(got[:18]) == sorted((r, tp, b, 0) for r in (1, 2, 3) for tp in (1, 2, 4)
                                      for b in (128, 256))
    assert got[0] == (1, 1, 128, 0)  # link_list's grid, one thread per particle, no skin
    assert got[18:] == [(r, 0, 0, sk) for r in (1, 2, 3) for sk in (10, 20, 40)]
    t = _abi.Tuning()
    assert lib.armando_tuning_candidate(_abi.N_TUNINGS, C.byref(t)) == _abi.ERR_INVALID_ARG
    assert lib.armando_tuning_candidate(-1, C.byref(t)) == _abi.ERR_INVALID_ARG


def test_tuning_struct_and_count_match_c():
    code = r'''
#include <stdio.h>
#include <stddef.h>
#include "armando.h"
int main(void) {
  printf("%zu %zu %d\n", sizeof(armando_tuning), offsetof(armando_tuning, block),
         ARMANDO_N_TUNINGS);
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(src, "w").write(code)
        subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), src, "-o", exe], check=True)
        got = list(map(int, subprocess.run([exe], capture_output=True, text=True).stdout.split()))
    assert got == [C.sizeof(_abi.Tuning), _abi.Tuning.block.offset, _abi.N_TUNINGS]
