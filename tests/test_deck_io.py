"""Particle decks (armando_deck_*) and VTK snapshots (armando_write_vtk).

Host-only entry points of the library. The fixture holds the first 40
records of the reference's own FORTRANsource deck files (written by its
`output` subroutine, CERNsource/output.f:31-73), cut by
tests/golden/make_deck_fixture.py. The writer's formats are checked against
an independent Python formatter of Fortran e14.8 / I6 / I4, which in turn
reproduces the fixture's lines from their values.
"""
import decimal
import os
import re
import shutil

import numpy as np
import pytest

import armando_gb300 as ag
from armando_gb300 import cases

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "deck")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from armando_gb300 import build

    build.build_library()
    ag.load_library()


def e14_8(v: float) -> str:
    """Fortran e14.8 of a double, by decimal arithmetic."""
    if v == 0.0:
        s = "0.00000000E+00"
    else:
        d = decimal.Decimal(abs(v))
        e = d.adjusted() + 1  # 0.d1... x 10^e
        q = (d.scaleb(-e)).quantize(decimal.Decimal("1e-8"), rounding=decimal.ROUND_HALF_EVEN)
        if q >= 1:
            e += 1
            q = (d.scaleb(-e)).quantize(decimal.Decimal("1e-8"), rounding=decimal.ROUND_HALF_EVEN)
        digits = f"{q:.8f}"[2:]
        exp = f"E{'-' if e < 0 else '+'}{abs(e):02d}" if abs(e) <= 99 else f"{'-' if e < 0 else '+'}{abs(e):03d}"
        s = ("-." if v < 0 else "0.") + digits + exp
    return s.rjust(14)


def reference_lines(name):
    with open(os.path.join(GOLD, name)) as f:
        return f.read().splitlines()


def test_python_formatter_reproduces_the_reference_text():
    """The reference wrote FP64 values with format (1x,I6,k(2x,e14.8)); the
    formatter gives back every fixture line from its parsed values."""
    for name in ("v_xv.dat", "v_state.dat", "f_state.dat"):
        for line in reference_lines(name)[(1 if name.endswith("xv.dat") else 0):]:
            tok = line.split()
            rebuilt = " " + tok[0].rjust(6) + "".join("  " + e14_8(float(t)) for t in tok[1:])
            assert rebuilt == line, (name, line, rebuilt)
    for line in reference_lines("f_other.dat") + reference_lines("v_other.dat"):
        i, mat, h = line.split()
        assert " " + i.rjust(6) + "  " + mat.rjust(4) + "  " + e14_8(float(h)) == line


def test_reader_parses_the_reference_deck(tmp_path):
    """v_ files of the reference (40 records) read back as the FP32 rounding of
    their decimal text; the virtual particles' velocity columns are unit
    normals, the convention wall_model 3 relies on."""
    deck = tmp_path / "deck"
    deck.mkdir()
    for name in ("v_xv.dat", "v_state.dat", "v_other.dat"):
        shutil.copy(os.path.join(GOLD, name), deck / name)
    lines = reference_lines("v_xv.dat")
    (deck / "v_xv.dat").write_text("40\n" + "\n".join(lines[1:]) + "\n")
    # a deck needs real particles: two of them, written by the library
    two = {f: np.zeros(6 if f in ("x", "v") else 2, np.int32 if f == "itype" else np.float32)
           for f in ag.DECK_FIELDS}
    two["itype"][:] = 21
    ag.write_deck(deck, 3, 2, two)
    for name in ("v_xv.dat", "v_state.dat", "v_other.dat"):  # write_deck replaced them
        shutil.copy(os.path.join(GOLD, name), deck / name)
    (deck / "v_xv.dat").write_text("40\n" + "\n".join(lines[1:]) + "\n")
    with pytest.raises(ag.ArmandoError) as e:  # no deck in that directory
        ag.read_deck(tmp_path / "nowhere", 3)
    assert e.value.status == ag._abi.ERR_IO
    a = ag.read_deck(deck, 3)
    assert a["n_real"] == 2 and a["n_virtual"] == 40
    xv = np.array([[float(t) for t in ln.split()[1:]] for ln in lines[1:]], np.float64)
    np.testing.assert_array_equal(a["x"].reshape(-1, 3)[2:], xv[:, :3].astype(np.float32))
    np.testing.assert_array_equal(a["v"].reshape(-1, 3)[2:], xv[:, 3:].astype(np.float32))
    st = np.array([[float(t) for t in ln.split()[1:]] for ln in reference_lines("v_state.dat")])
    np.testing.assert_array_equal(a["mass"][2:], st[:, 0].astype(np.float32))
    np.testing.assert_array_equal(a["rho"][2:], st[:, 1].astype(np.float32))
    ot = [ln.split() for ln in reference_lines("v_other.dat")]
    assert a["itype"][2:].tolist() == [int(t[1]) for t in ot]
    np.testing.assert_array_equal(a["h"][2:], np.array([float(t[2]) for t in ot], np.float32))
    normals = np.linalg.norm(a["v"].reshape(-1, 3)[2:].astype(np.float64), axis=1)
    np.testing.assert_allclose(normals, 1.0, atol=2e-7)


def test_writer_formats_match_fortran(tmp_path):
    """Every written line equals the Python formatter's on the FP32 values:
    signs, zeros, tiny and large magnitudes, rounding at the 8th digit."""
    rng = np.random.default_rng(3)
    n, dim = 64, 3
    vals = np.concatenate([[0.0, -0.0, 1.0, -1.0, 0.999999999, 9.99999999e-5, 1.5e-38, -3.0e38],
                           rng.standard_normal(n * 6 - 8) * 10.0 ** rng.integers(-30, 30, n * 6 - 8)])
    vals = vals.astype(np.float32)
    a = {"x": vals[:n * dim], "v": vals[n * dim:2 * n * dim],
         "mass": np.abs(vals[:n]), "rho": vals[n:2 * n], "p": vals[2 * n:3 * n],
         "u": vals[3 * n:4 * n], "h": np.abs(vals[4 * n:5 * n]),
         "itype": rng.integers(-30, 31, n).astype(np.int32)}
    ag.write_deck(tmp_path, dim, 40, a)
    xv = (tmp_path / "f_xv.dat").read_text().splitlines()
    assert xv[0] == "%12d" % 40
    for i in range(40):
        exp = " " + str(i + 1).rjust(6) + "".join(
            "  " + e14_8(float(q)) for q in list(a["x"][i * 3:i * 3 + 3]) + list(a["v"][i * 3:i * 3 + 3]))
        assert xv[1 + i] == exp
    vo = (tmp_path / "v_other.dat").read_text().splitlines()
    for k, line in enumerate(vo):
        i = 40 + k
        assert line == " " + str(i + 1).rjust(6) + "  " + str(a["itype"][i]).rjust(4) + "  " + \
            e14_8(float(a["h"][i]))
    pat = re.compile(r"^ [ \d]{6}(  (0\.|-\.)\d{8}(E[+-]\d{2}|[+-]\d{3})){4}$")
    for line in (tmp_path / "f_state.dat").read_text().splitlines():
        assert pat.match(line) or "*" in line, line


@pytest.mark.parametrize("dim", [2, 3])
def test_round_trip_of_a_case(tmp_path, dim):
    """Case -> deck -> arrays: within the 8 significant digits of e14.8 (one
    FP32 ulp at most), itype exact, the wall particles in the v_ files."""
    c = cases.dam_break(dx=0.05) if dim == 2 else cases.channel(
        n_x=8, n_yz=4, length=8 * 7.9e-4, width=4 * 7.9e-4, layers=2)
    order = np.argsort(c.itype <= 0, kind="stable")  # real particles first
    a = {f: (getattr(c, f).reshape(c.n, -1)[order].ravel() if f in ("x", "v")
             else getattr(c, f)[order]) for f in ag.DECK_FIELDS}
    nr = int((c.itype > 0).sum())
    ag.write_deck(tmp_path, dim, nr, a)
    b = ag.read_deck(tmp_path, dim)
    assert b["n_real"] == nr and b["n_virtual"] == c.n - nr
    assert np.array_equal(b["itype"], a["itype"])
    for f in ("x", "v", "mass", "rho", "p", "u", "h"):
        x0, x1 = a[f].astype(np.float32), b[f]
        ulp = np.spacing(np.abs(x0))
        assert np.all(np.abs(x1 - x0) <= ulp), f


def test_vtk_snapshot(tmp_path):
    c = cases.dam_break(dx=0.1)
    path = tmp_path / "out00000.vtk"
    ag.write_vtk(path, 2, c)
    lines = path.read_text().splitlines()
    assert lines[:4] == ["# vtk DataFile Version 2.0", "Unstructured Grid Example", "ASCII",
                         "DATASET UNSTRUCTURED_GRID"]
    n = c.n
    assert lines[4] == f"POINTS {n} float"
    pts = np.array([[float(t) for t in ln.split()] for ln in lines[5:5 + n]])
    np.testing.assert_allclose(pts[:, :2], c.x.reshape(-1, 2), rtol=1e-6)
    assert np.all(pts[:, 2] == 0.0)
    k = 5 + n
    assert lines[k] == f"CELLS {n} {2 * n} "
    assert lines[k + 1 + n] == f"CELL_TYPES {n} "
    assert lines[k + 2 + 2 * n] == f"POINT_DATA {n} "
    names = [ln.split()[1] for ln in lines if ln.startswith(("SCALARS", "VECTORS"))]
    assert names == ["material", "density", "pressure", "energy", "velocity"]
    mat = [int(t) for t in lines[k + 5 + 2 * n:k + 5 + 3 * n]]
    assert mat == c.itype.tolist()
    with pytest.raises(ag.ArmandoError) as e:
        ag.write_vtk(tmp_path / "no" / "such" / "dir.vtk", 2, c)
    assert e.value.status == ag._abi.ERR_IO


def test_short_arrays_are_refused_before_the_library_reads_them(tmp_path):
    """The writers read n*dim positions and velocities and n of the rest:
    shorter arrays raise ValueError in Python instead of reaching C."""
    c = cases.dam_break(dx=0.1)
    a = {k: v.copy() for k, v in c.arrays().items()}
    a["x"] = a["x"][:-1]
    with pytest.raises(ValueError):
        ag.write_deck(str(tmp_path), c.dim, c.n_fluid, a)
    with pytest.raises(ValueError):
        ag.write_vtk(str(tmp_path / "s.vtk"), c.dim, a)
