"""Mesh construction (host side; not part of the hot path).

The reference builds its Voronoi mesh on the host with meshless_voronoi
(``src/space.rs:571-594``), and the mesh stays on the host here too: the hot
path only consumes the face list and the CSR.  1D meshes are analytic here; 2D and
3D meshes come from this library's own C++ builder (``csrc/voronoi.cpp``,
compiled to ``_build/libmvmm_mesh.so`` by :mod:`hydro_rs_gb300.build`).

1D conventions follow the reference's 1D test (``src/space.rs:1453-1491``):
faces are ordered left wall, interior faces left to right, right wall; a cell
owns the faces ``[i, i+1]``; face centroids are ``(x_face, Ly/2, Lz/2)`` and
cell centroids ``(x_c, Ly/2, Lz/2)`` with unit extent along the unused axes.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .layout import Mesh

_HERE = os.path.dirname(os.path.abspath(__file__))
_MESH_LIB = None


def _mesh_lib():
    global _MESH_LIB
    if _MESH_LIB is None:
        path = os.path.join(_HERE, "_build", "libmvmm_mesh.so")
        if not os.path.exists(path):
            raise RuntimeError(f"mesh builder library missing: {path} (run __graft_entry__.build())")
        lib = ctypes.CDLL(path)
        lib.mvmm_voronoi_build.restype = ctypes.c_int
        lib.mvmm_voronoi_build.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                           ctypes.POINTER(ctypes.c_void_p)]
        lib.mvmm_voronoi_fetch.restype = ctypes.c_int
        lib.mvmm_voronoi_fetch.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 10
        lib.mvmm_voronoi_free.restype = None
        lib.mvmm_voronoi_free.argtypes = [ctypes.c_void_p]
        _MESH_LIB = lib
    return _MESH_LIB


def mesh_1d(x: np.ndarray, box=(1.0, 1.0, 1.0), periodic: bool = False) -> Mesh:
    """Analytic 1D Voronoi mesh of sorted generators ``x`` on ``[0, box[0]]``."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    assert n >= 2 and np.all(np.diff(x) > 0), "1D generators must be sorted and distinct"
    L, Ly, Lz = box
    mids = 0.5 * (x[:-1] + x[1:])
    if not periodic:
        fx = np.concatenate([[0.0], mids, [L]])
        f = n + 1
        left = np.concatenate([[0], np.arange(n - 1), [n - 1]]).astype(np.int32)
        right = np.concatenate([[-1], np.arange(1, n), [-1]]).astype(np.int32)
        nx = np.ones(f)
        nx[0] = -1.0
        shift = np.zeros((3, f))
        lo = fx[:-1]
        hi = fx[1:]
        csr_face = np.stack([np.arange(n), np.arange(1, n + 1)], axis=1).reshape(-1).astype(np.int32)
    else:
        # face 0 joins cell 0 and the image of cell n-1 shifted by -L
        wrap = 0.5 * (x[0] + x[-1] - L)
        fx = np.concatenate([[wrap], mids])
        f = n
        left = np.concatenate([[0], np.arange(n - 1)]).astype(np.int32)
        right = np.concatenate([[n - 1], np.arange(1, n)]).astype(np.int32)
        nx = np.ones(f)
        nx[0] = -1.0
        shift = np.zeros((3, f))
        shift[0, 0] = -L
        lo = np.concatenate([[wrap], mids])
        hi = np.concatenate([mids, [wrap + L]])
        # cell i touches faces i (lower) and i+1 (upper); cell n-1's upper face is face 0
        up = np.concatenate([np.arange(1, n), [0]])
        pairs = np.stack([np.arange(n), up], axis=1)
        pairs.sort(axis=1)
        csr_face = pairs.reshape(-1).astype(np.int32)
    normal = np.zeros((3, f))
    normal[0] = nx
    centroid = np.zeros((3, f))
    centroid[0] = fx
    centroid[1] = 0.5 * Ly
    centroid[2] = 0.5 * Lz
    area = np.full(f, Ly * Lz)
    csr_off = (2 * np.arange(n + 1)).astype(np.int32)
    volume = (hi - lo) * Ly * Lz
    cc = np.zeros((3, n))
    cc[0] = 0.5 * (lo + hi)
    cc[1] = 0.5 * Ly
    cc[2] = 0.5 * Lz
    m = Mesh(n_cells=n, left=left, right=right, area=area, normal=normal, centroid=centroid,
             shift=np.ascontiguousarray(shift), csr_off=csr_off, csr_face=csr_face, volume=volume,
             cell_centroid=cc, dimensionality=1, box=tuple(box), periodic=periodic)
    return m


def mesh_voronoi(gen: np.ndarray, dim: int, box, periodic: bool, n_threads: int = 0, arrays=None) -> Mesh:
    """2D/3D Voronoi mesh of generators ``gen`` ([3][n]) with the C++ builder.

    arrays: optional ``arrays(specs) -> list of ndarrays`` that provides the
    output arrays for a list of (shape, dtype), e.g. page-locked host memory
    (``gpu.PinnedArrays``) from which the mesh uploads at the link's speed."""
    lib = _mesh_lib()
    gen = np.ascontiguousarray(gen, dtype=np.float64)
    n = gen.shape[1]
    boxa = np.ascontiguousarray(np.asarray(box, dtype=np.float64))
    nf = ctypes.c_int64(0)
    h = ctypes.c_void_p(0)
    rc = lib.mvmm_voronoi_build(dim, n, gen.ctypes.data, boxa.ctypes.data, int(periodic), n_threads,
                                ctypes.byref(nf), ctypes.byref(h))
    if rc != 0:
        raise RuntimeError(f"Voronoi construction failed (code {rc})")
    f = nf.value
    try:
        # csr_face holds 2F - (#walls) entries: room for 2F, trimmed below
        specs = [(f, np.int32), (f, np.int32), (f, np.float64), ((3, f), np.float64), ((3, f), np.float64),
                 ((3, f), np.float64), (n + 1, np.int32), (n, np.float64), ((3, n), np.float64), (2 * f, np.int32)]
        if arrays is None:
            out = [np.empty(shape, dt) for shape, dt in specs]
        else:
            out = arrays(specs)
        left, right, area, normal, centroid, shift, csr_off, volume, cc, csr_face = out
        lib.mvmm_voronoi_fetch(h, left.ctypes.data, right.ctypes.data, area.ctypes.data, normal.ctypes.data,
                               centroid.ctypes.data, shift.ctypes.data, csr_off.ctypes.data, csr_face.ctypes.data,
                               volume.ctypes.data, cc.ctypes.data)
        csr_face = np.ascontiguousarray(csr_face[: csr_off[-1]])
    finally:
        lib.mvmm_voronoi_free(h)
    return Mesh(n_cells=n, left=left, right=right, area=area, normal=normal, centroid=centroid, shift=shift,
                csr_off=csr_off, csr_face=csr_face, volume=volume, cell_centroid=cc, dimensionality=dim,
                box=tuple(float(b) for b in box), periodic=periodic)
