"""CPU checks of the C ABI: the library builds, loads, exports every symbol the
header declares, and rejects invalid descriptors before touching the GPU."""
import ctypes as ct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from marie_gb300 import _lib, _build

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def test_exports_every_header_symbol(lib):
    syms = _lib.header_symbols()
    assert len(syms) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.lib_path())], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        assert hasattr(lib, s)


def test_version_and_counter(lib):
    assert b"sm_103a" in lib.marie_version()
    assert lib.marie_launch_count() >= 0


def _desc(**kw):
    d = _lib.VieDesc()
    d.n1 = d.n2 = d.n3 = 4
    d.basis = _lib.PWC
    d.res, d.freq = 5e-3, 128e6
    d.precisions, d.max_rhs = 3, 1
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def _create(lib, d):
    h = ct.c_void_p()
    st = lib.marie_vie_create(ct.byref(h), ct.byref(d))
    return st, h


def test_rejects_bad_descriptors(lib):
    idx = np.arange(3 * 5, dtype=np.int64)   # not component-major for a 4^3 grid
    mr = np.ones(2 * 64)
    dense = np.zeros(2 * 64 * 6)
    base = dict(n_b=15, idx_solution=idx.ctypes.data_as(ct.POINTER(ct.c_int64)),
                Mr=mr.ctypes.data_as(_lib.c_double_p), dense_N=dense.ctypes.data_as(_lib.c_double_p))
    cases = [
        dict(base, n1=0),
        dict(base, basis=5),
        dict(base, res=-1.0),
        dict(base, freq=0.0),
        dict(base, precisions=0),
        dict(base, precisions=8),
        dict(base, precisions=16),
        dict(base, precisions=2 | 8),            # per-application Tucker expansion without Tucker blocks
        dict(base, precisions=1 | 8),            # ... or without the complex64 state
        dict(base, precisions=5),                # native and float-float complex128 together
        dict(base, max_rhs=0),
        dict(base, n_b=16),                      # not a multiple of 3
        dict(base),                              # idx_solution not component-major
        dict(base, dense_N=None),                # no operator
    ]
    for kw in cases:
        st, h = _create(lib, _desc(**kw))
        assert st == 1, (kw.keys(), st, _lib.last_error())
        assert not h.value
        assert _lib.last_error()


def test_float_float_needs_four_step_grid(lib):
    """precisions bit 4 (complex128 in float-float arithmetic) is offered on
    grids whose edges are 16*NB with NB <= 8 only."""
    idx = np.arange(3 * 5, dtype=np.int64)
    mr = np.ones(2 * 64)
    dense = np.zeros(2 * 64 * 6)
    d = _desc(n_b=15, idx_solution=idx.ctypes.data_as(ct.POINTER(ct.c_int64)), precisions=6,
              Mr=mr.ctypes.data_as(_lib.c_double_p), dense_N=dense.ctypes.data_as(_lib.c_double_p))
    st, h = _create(lib, d)
    assert st == 7 and not h.value and "16*NB" in _lib.last_error()


def test_rejects_out_of_grid_index(lib):
    Ns = 5
    idxS = np.array([0, 1, 2, 3, 64], dtype=np.int64)      # 64 is outside a 4^3 grid
    idx = np.concatenate([idxS + c * 64 for c in range(3)])
    mr = np.ones(2 * 64)
    dense = np.zeros(2 * 64 * 6)
    d = _desc(n_b=3 * Ns, idx_solution=idx.ctypes.data_as(ct.POINTER(ct.c_int64)),
              Mr=mr.ctypes.data_as(_lib.c_double_p), dense_N=dense.ctypes.data_as(_lib.c_double_p))
    st, h = _create(lib, d)
    assert st == 1 and "outside" in _lib.last_error()


def test_null_handle_calls(lib):
    assert lib.marie_vie_apply(None, 0, None, None, 1, None) == 1
    assert lib.marie_gmres_vie(None, None, None, 1, None, None, None) == 1
    assert lib.marie_vie_destroy(None) == 0


def test_mex_gateway_compiles_against_stub():
    """The MEX gateway (MATLAB caller of the C ABI) compiles against a
    declaration-only mex.h; MATLAB itself is not available to run it."""
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        "-I", str(ROOT / "tests" / "mex_stub"), "-I", str(ROOT / "include"),
                        str(ROOT / "marie-tools_gb300" / "mex" / "marie_mex.c")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "marie_gb300.h"\nint main(void){marie_vie_desc d; (void)d; return 0;}\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-c", str(src),
                        "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_embedded_grid_descriptors_are_validated_on_the_callers_grid(lib):
    """A grid with a prime edge above 31 goes through the embedding branch of
    marie_vie_create; its descriptor is checked on the caller's grid first."""
    n1 = 37
    nD = n1 * 4 * 4
    mr = np.ones(2 * nD)
    dense = np.zeros(2 * nD * 6)
    idxS = np.array([0, 1, nD], dtype=np.int64)               # nD is outside the 37x4x4 grid
    idx = np.concatenate([idxS + c * nD for c in range(3)])
    d = _desc(n1=n1, n_b=9, idx_solution=idx.ctypes.data_as(ct.POINTER(ct.c_int64)),
              Mr=mr.ctypes.data_as(_lib.c_double_p), dense_N=dense.ctypes.data_as(_lib.c_double_p))
    st, h = _create(lib, d)
    assert st == 1 and "outside" in _lib.last_error() and not h.value
    idxS = np.array([0, 1, 2], dtype=np.int64)
    idx = np.concatenate([idxS + c * nD for c in range(3)])
    d = _desc(n1=n1, n_b=9, idx_solution=idx.ctypes.data_as(ct.POINTER(ct.c_int64)), precisions=5,
              Mr=mr.ctypes.data_as(_lib.c_double_p), dense_N=dense.ctypes.data_as(_lib.c_double_p))
    st, h = _create(lib, d)
    assert st == 1 and "exclusive" in _lib.last_error()


def test_assemble_green_ex_rejects_unknown_flags(lib):
    out = np.zeros(2 * 8 * 6)
    st = lib.marie_assemble_green_ex(2, 2, 2, 2e-3, 297.2e6, 0, 0, 4, out.ctypes.data_as(_lib.c_double_p))
    assert st == 1 and "flags" in _lib.last_error()
    st = lib.marie_assemble_green_ex(0, 2, 2, 2e-3, 297.2e6, 0, 0, 2, out.ctypes.data_as(_lib.c_double_p))
    assert st == 1


def test_embedded_descriptor_reaches_the_device_step(lib):
    """A valid descriptor on a grid with a prime edge (37) runs the host-side
    embedding (padding of Mr, idx_solution and the operator; the Tucker
    factors re-derived for the 48 x 16 x 16 grid) and the embedded grid's
    own validation, and stops only where a GPU is needed."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("needs a machine without a GPU")
    from helpers import Problem
    from marie_gb300 import VieOperator
    P = Problem((37, 10, 9), False, seed=3)
    for dense in (False, True):
        N = P.IV_N if dense else P.TN
        K = P.IV_K if dense else P.TK
        with pytest.raises(_lib.MarieError) as e:
            VieOperator(P.n, P.res, P.freq, P.dims["idx_solution"], P.Mr, N, K, pwl=False, precisions=2 | 4,
                        max_rhs=1)
        assert e.value.status == 6 and "CUDA device" in str(e.value)


def test_ctypes_structs_match_header(tmp_path):
    """The Python mirror's ctypes structures have the header's layout
    (sizes and field offsets, compiled with the host C compiler)."""
    import shutil
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    structs = {"marie_gmres_opts": _lib.GmresOpts, "marie_gmres_report": _lib.GmresReport,
               "marie_vie_desc": _lib.VieDesc, "marie_tucker_block": _lib.TuckerBlock, "marie_csr": _lib.Csr,
               "marie_svie_pfft_desc": _lib.SviePfftDesc}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "marie_gb300.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, val = line.split()
        got[(name, field)] = int(val)
    for cname, cls in structs.items():
        assert got[(cname, "size")] == ct.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
