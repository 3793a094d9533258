"""A compiled C++ caller of the C-ABI (tests/capi_driver.cpp).

The program is built with g++ against include/armando.h and linked to
libarmando_gb300.so, as a C++ host code replacing the Fortran driver would be
(CERNsource/time_integration.f:175-183 calling single_step). On the GPU it
runs the C1 cavity through armando_create / armando_integrate /
armando_destroy from a state file this test writes, and its output must equal
the Python mirror's bit for bit.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORDER = ("x", "v", "mass", "rho", "p", "u", "h", "itype", "dvdt", "dudt")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from armando_gb300 import build

    lib = build.build_library()
    exe = str(tmp_path_factory.mktemp("capi") / "capi_driver")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "capi_driver.cpp"),
                    "-L", libdir, "-larmando_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True)
    return exe


def test_driver_builds_against_the_header(driver):
    assert os.access(driver, os.X_OK)


def _write_state(path, c):
    with open(path, "wb") as f:
        f.write(struct.pack("<iqqf", c.dim, c.n_fluid, c.n_wall, c.dt))
        f.write(bytes(c.params))
        for k in ORDER:
            f.write(np.ascontiguousarray(getattr(c, k)).tobytes())


def _read_state(path, c):
    out = c.copy()
    raw = open(path, "rb").read()
    off = 0
    for k in ORDER:
        a = getattr(c, k)
        nb = a.nbytes
        setattr(out, k, np.frombuffer(raw[off:off + nb], dtype=a.dtype).copy())
        off += nb
    assert off == len(raw)
    return out


@pytest.mark.gpu
def test_cpp_driver_equals_python_mirror(driver, tmp_path):
    c = cases.cavity()  # 1,600 fluid + 320 wall particles
    src, dst = str(tmp_path / "state.bin"), str(tmp_path / "out.bin")
    _write_state(src, c)
    r = subprocess.run([driver, src, dst, "30", "10"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "steps_done 30" in r.stdout
    got = _read_state(dst, c)
    ref = c.copy()
    with ag.Context(c.params, c.n_fluid, c.n_wall) as ctx:
        for its0 in (1, 11, 21):
            ctx.integrate(ref, c.dt, its0, 10)
    for k in ORDER:
        assert np.array_equal(getattr(got, k), getattr(ref, k)), k
