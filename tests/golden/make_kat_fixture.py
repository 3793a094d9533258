"""Golden vector of the reference's own known-answer test.

ArmandoList/armando2Dlist.cu:2451-2548 (check()) runs the reference's GPU pair
kernel (kerInteraction, armando2Dlist.cu:611-686) once on the 100 x 100 lattice
of initFree (armando2Dlist.cu:1834-1880: dr = 0.01, h = 1.2 dr, rho0 = 1000,
c0 = 50) with the manufactured fields p = 1000 (sin(10 pi x) + y^2),
v = (sin(10 pi x), y^2), and writes the rates (drho/dt, dvx/dt, dvy/dt) of
every particle, in the kernel's cell order, to ArmandoList/old.txt; rows of
particles within one cell (0.024) of the square's edges are replaced by the
analytic rates first (armando2Dlist.cu:2492-2502). This script stores those
rows as FP32 (the printed 9 significant digits identify an FP32 value):

  python tests/golden/make_kat_fixture.py      -> tests/golden/kat_old.npz

The reference tree: $ARMANDO_REF_DIR, else its mount point.
"""
import os

import numpy as np

ROOT = os.environ.get("ARMANDO_REF_DIR", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat_old.npz")


def main():
    rows = np.loadtxt(os.path.join(ROOT, "ArmandoList", "old.txt"), dtype=np.float64)
    assert rows.shape == (10000, 3)
    f32 = rows.astype(np.float32)
    # every printed value is an FP32 value to its 9 significant digits
    assert np.array_equal(np.char.mod("%+14.8e", f32.astype(np.float64)),
                          np.char.mod("%+14.8e", rows))
    np.savez_compressed(OUT, rates=f32)
    print(OUT, f32.shape)


if __name__ == "__main__":
    main()
