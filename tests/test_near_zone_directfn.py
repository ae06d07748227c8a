"""The near-zone cubature against the reference's own singular quadrature.

oracle/Makefile compiles the reference's DIRECTFN C++ (the singular
surface-surface integrals behind assembly_N.m:56-81) from the reference
checkout into oracle/_ref; oracle/directfn_ref.py evaluates with it the
surface-surface near zone of the PWC moment (self offset xx, face neighbour
xx and yy).  The oracle's near_zone_relative (and hence the library's
MARIE_GREEN_NEAR_EXACT cubature, equal to it to 1e-14 in
test_green_host.py) must agree.  Skipped where the reference checkout or
g++ is absent.
"""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O

ROOT = Path(__file__).resolve().parent.parent
REF = Path(os.environ.get("MARIE_REFERENCE_ROOT", "/root/reference"))


@pytest.fixture(scope="module")
def directfn():
    if not (REF / "src").is_dir() or not shutil.which("g++") or not shutil.which("make"):
        pytest.skip("reference checkout or toolchain not present")
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), f"REF={REF}"], check=True)
    from oracle import directfn_ref
    return directfn_ref


@pytest.mark.parametrize("freq,res", [(297.2e6, 2e-3), (128e6, 5e-3)])
def test_pwc_near_zone_matches_directfn(directfn, freq, res):
    k0 = O.em_constants(freq)["k0"]
    ref = directfn.pwc_near_entries(k0, res)
    nz = O.near_zone_relative(k0, res, 1, "N", [(0, 0, 0), (1, 0, 0)])
    for key, got in (("self_xx", nz[(0, 0, 0)][0, 0]), ("face_xx", nz[(1, 0, 0)][0, 0]),
                     ("face_yy", nz[(1, 0, 0)][0, 3])):
        assert abs(got - ref[key]) <= 1e-12 * abs(ref[key]), (key, got, ref[key])
    # the stand-in misses the point term (self) and is 13% low on the face neighbour
    st = O.near_zone_standin(k0, res, 1, "N", [(0, 0, 0), (1, 0, 0)])
    assert abs(st[(0, 0, 0)][0, 0]) < 1e-3 * abs(ref["self_xx"])
    assert abs(st[(1, 0, 0)][0, 0] / ref["face_xx"] - 1) > 0.05
