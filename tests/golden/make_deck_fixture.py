#!/usr/bin/env python
"""Cuts the deck fixture: the first 40 records of the reference's own
FORTRANsource particle files (written by its `output` subroutine,
CERNsource/output.f:31-73), verbatim, count lines included.

  python tests/golden/make_deck_fixture.py [REFERENCE_ROOT]

Writes tests/golden/deck/<name> for v_xv.dat, v_state.dat, v_other.dat,
f_state.dat and f_other.dat (the deck has no f_xv.dat).
"""
import os
import sys

RECORDS = 40
ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ARMANDO_REF_DIR", "/root/reference")
SRC = os.path.join(ROOT, "FORTRANsource")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "deck")

os.makedirs(OUT, exist_ok=True)
for name in ("v_xv.dat", "v_state.dat", "v_other.dat", "f_state.dat", "f_other.dat"):
    with open(os.path.join(SRC, name)) as f:
        lines = f.readlines()
    head = 1 if name.endswith("_xv.dat") else 0  # the count line
    with open(os.path.join(OUT, name), "w") as f:
        f.writelines(lines[:head + RECORDS])
