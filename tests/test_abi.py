"""The C ABI library loads and exports every symbol its header declares.

No compute call is made here (CPU-only test); argument validation that
happens on the host before any CUDA call is exercised.
"""
import ctypes
import os
import re

import pytest

from hydro_rs_gb300 import build as B
from hydro_rs_gb300 import gpu as G
from hydro_rs_gb300 import ics

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "mvmm_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mvmm_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    B.build_gpu()
    return G.load_library()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) >= set(G.EXPORTED)


def test_invalid_params_rejected_on_host(lib):
    p = ics.sod_1d(16)
    prm = G._Params(0.9, 0, 0.0, 0.3, 0, 1, 1, 1, 0.2, 1000, 0, 0)  # gamma <= 1
    mv = p.mesh.cview()
    h = ctypes.c_void_p(0)
    rc = lib.mvmm_ctx_create(ctypes.byref(prm), ctypes.byref(mv), ctypes.byref(h))
    assert rc == -1 and h.value is None
    assert b"gamma" in lib.mvmm_last_error()
    prm = G._Params(5 / 3, 0, 0.0, 0.3, 0, 1, 1, 1, 0.2, 1000, 0, 1)  # moving mesh without a box size
    rc = lib.mvmm_ctx_create(ctypes.byref(prm), ctypes.byref(mv), ctypes.byref(h))
    assert rc == -1 and b"box_size" in lib.mvmm_last_error()


def test_bad_mesh_rejected_on_host(lib):
    p = ics.sod_1d(16)
    m = p.mesh
    m.right[3] = 99  # out of range
    prm = G._Params(5 / 3, 0, 0.0, 0.3, 0, 1, 1, 1, 0.2, 1000, 0, 0)
    mv = m.cview()
    h = ctypes.c_void_p(0)
    rc = lib.mvmm_ctx_create(ctypes.byref(prm), ctypes.byref(mv), ctypes.byref(h))
    assert rc == -1 and b"out of range" in lib.mvmm_last_error()
    # boundary faces with periodic boundary conditions (flux.rs:255-257 is unreachable there)
    p = ics.sod_1d(16)
    prm = G._Params(5 / 3, 0, 0.0, 0.3, 0, 0, 1, 1, 0.2, 1000, 0, 0)
    mv = p.mesh.cview()
    rc = lib.mvmm_ctx_create(ctypes.byref(prm), ctypes.byref(mv), ctypes.byref(h))
    assert rc == -1


@pytest.mark.parametrize("defect,message", [
    ("left", b"face left index out of range"),
    ("right", b"face right index out of range"),
    ("csr_off", b"csr_off not monotone"),
    ("csr_face", b"csr face index out of range"),
    ("csr_count", b"csr does not match faces"),
    ("csr_touch", b"csr lists a face not touching the cell"),
])
def test_each_mesh_defect_rejected_on_host(lib, defect, message):
    """Every index a kernel reads through is checked before the context exists
    (check_mesh, run over the host's cores): each defect gets its own error."""
    p = ics.kelvin_helmholtz_2d(12, riemann=ics.HLLC)
    m = p.mesh
    m.left, m.right = m.left.copy(), m.right.copy()
    m.csr_off, m.csr_face = m.csr_off.copy(), m.csr_face.copy()
    if defect == "left":
        m.left[7] = m.n_cells
    elif defect == "right":
        m.right[11] = -2
    elif defect == "csr_off":
        m.csr_off[5], m.csr_off[6] = m.csr_off[6], m.csr_off[5]
    elif defect == "csr_face":
        m.csr_face[3] = m.n_faces
    elif defect == "csr_count":
        f = int(m.csr_face[m.csr_off[4]])  # cell 4 gives a face to cell 5's list
        m.csr_off[5] -= 1
        assert f >= 0
    elif defect == "csr_touch":
        k = int(m.csr_off[20])
        cells = {int(m.left[int(m.csr_face[k])]), int(m.right[int(m.csr_face[k])])}
        other = next(f for f in range(m.n_faces) if 20 not in (int(m.left[f]), int(m.right[f])))
        m.csr_face[k] = other
        assert 20 in cells
    prm = G.make_params(p.params, 0, m.box)
    mv = m.cview()
    h = ctypes.c_void_p(0)
    rc = lib.mvmm_ctx_create(ctypes.byref(prm), ctypes.byref(mv), ctypes.byref(h))
    assert rc == -1 and h.value is None
    assert message in lib.mvmm_last_error(), lib.mvmm_last_error()


def test_product_does_not_import_the_oracle():
    pkg = os.path.join(ROOT, "hydro_rs_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                txt = open(os.path.join(dirpath, fn)).read()
                assert "oracle" not in txt.replace("the oracle", "").replace("The oracle", "") or fn.endswith(".md"), fn
