"""MARIE's RHBM body files (the input format of geo_body_domain.m) read by
phantoms.load_rhbm: a synthetic file written here, and the reference's own
body fixtures where the reference checkout is present (the 73 x 73 x 84
inhomogeneous cylinder has an edge the FFT passes take only by embedding)."""
import os
from pathlib import Path

import numpy as np
import pytest

from oracle import marie_oracle as O
from marie_gb300 import phantoms

# the reference checkout's body and input files, linked into oracle/_ref by
# the oracle recipe (or MARIE_REFERENCE_ROOT); the tests that need them skip
# without
ROOT = Path(__file__).resolve().parent.parent
_env = os.environ.get("MARIE_REFERENCE_ROOT")
DATA = {k: (Path(_env) / "data" / k if _env else ROOT / "oracle" / "_ref" / k) for k in ("bodies", "inputs")}
BODIES = DATA["bodies"] / "Scatterers" / "2mm"


def _smooth31(v):
    """All prime factors <= 31 (the FFT lengths the passes take directly)."""
    for p in range(2, 32):
        while v % p == 0:
            v //= p
    return v == 1


def _write_rhbm(path, n, res, er, se, idx1):
    sio = pytest.importorskip("scipy.io")
    origin = np.array([-0.01, 0.02, -0.03])
    ax = [origin[d] + res * np.arange(n[d]) for d in range(3)]
    r = np.stack(np.meshgrid(*ax, indexing="ij"), axis=-1)
    rec = np.empty((1, 1), dtype=[("name", "O"), ("epsilon_r", "O"), ("sigma_e", "O"), ("rho", "O"), ("r", "O"),
                                  ("idxS", "O")])
    rec[0, 0] = ("synthetic", er, se, (er > 1).astype(np.uint8), r, idx1.reshape(-1, 1).astype(np.int32))
    sio.savemat(str(path), {"RHBM": rec})
    return origin


def test_load_synthetic_rhbm(tmp_path):
    n, res = (7, 5, 6), 2e-3
    rng = np.random.default_rng(0)
    mask = rng.uniform(size=n) < 0.5
    er = np.where(mask, rng.integers(5, 80, size=n), 1).astype(np.uint8)
    se = np.where(mask, rng.uniform(0.1, 2.0, size=n), 0.0)
    idx1 = np.nonzero(mask.reshape(-1, order="F"))[0] + 1          # MATLAB find(): 1-based, column-major
    origin = _write_rhbm(tmp_path / "b.mat", n, res, er, se, idx1)
    b = phantoms.load_rhbm(tmp_path / "b.mat")
    assert b.n == n and abs(b.res - res) < 1e-15
    assert np.allclose(b.origin, origin)
    assert np.array_equal(b.idxS, idx1 - 1)
    assert np.array_equal(b.er, er.astype(float)) and np.array_equal(b.se, se)
    # idx_solution as geo_body_domain.m:22-34 builds it (0-based here)
    assert np.array_equal(b.idx_solution(False), O.geo_dims(*n, b.idxS, False, res)["idx_solution"])


def test_rejects_non_rhbm(tmp_path):
    sio = pytest.importorskip("scipy.io")
    sio.savemat(str(tmp_path / "x.mat"), {"other": np.zeros(3)})
    with pytest.raises(ValueError, match="RHBM"):
        phantoms.load_rhbm(tmp_path / "x.mat")


@pytest.mark.skipif(not BODIES.is_dir(), reason="reference body fixtures not present")
@pytest.mark.parametrize("name,n,ns", [("Multilayer_Sphere", (121, 121, 121), 904089),
                                       ("inhomogeneous_cylinder", (73, 73, 84), 316470)])
def test_reference_bodies(name, n, ns):
    b = phantoms.load_rhbm(BODIES / f"{name}.mat")
    assert b.n == n and abs(b.res - 2e-3) < 1e-9 and b.idxS.size == ns
    assert np.all(np.diff(b.idxS) > 0) and b.idxS[-1] < np.prod(n)
    body_er = b.er.reshape(-1, order="F")[b.idxS]
    body_se = b.se.reshape(-1, order="F")[b.idxS]
    assert np.all(np.isfinite(body_er)) and np.all(body_er >= 1) and np.all(body_se >= 0)
    Mr = b.Mr(128e6).reshape(-1, order="F")[b.idxS]
    assert np.all(Mr != 0)
    smooth = [_smooth31(v) for v in n]
    # 73 is prime: the cylinder's grid runs embedded (80 x 80 x 96); 121 = 11^2 runs as given
    assert smooth == ([True] * 3 if name == "Multilayer_Sphere" else [False, False, True])


def test_load_inputs_synthetic(tmp_path):
    import json
    (tmp_path / "inputs").mkdir()
    f = tmp_path / "inputs" / "inp.json"
    f.write_text(json.dumps({"B0": 7.0, "Nucleus": "1H", "Basis_Functions_VIE": 0, "BodyFile": "x/b.mat",
                             "CoilFile": "", "WireFile": "w.msh", "ShieldFile": "", "TMD": 1, "BasisFile": ""}))
    inp = phantoms.load_inputs(f)
    assert abs(inp["freq"] - 42.577478518e6 * 7.0) < 1e-3 and inp["pwl"] is False
    assert inp["body_file"].resolve() == (tmp_path / "bodies" / "x" / "b.mat").resolve()
    assert phantoms.larmor_frequency(3.0, "31p") == 17.235e6 * 3.0


@pytest.mark.skipif(not DATA["inputs"].is_dir(), reason="reference input files not present")
def test_reference_input_file():
    """The reference's own input file: 1H at 3.0063 T is 128 MHz (the first
    configuration's frequency), PWL basis, and its body file loads."""
    inp = phantoms.load_inputs(DATA["inputs"] / "inp_MSphere_HeadCoil1z.json")
    assert abs(inp["freq"] - 128.0e6) < 0.1e6 and inp["pwl"] is True
    b = phantoms.load_rhbm(inp["body_file"])
    assert b.n == (121, 121, 121)
