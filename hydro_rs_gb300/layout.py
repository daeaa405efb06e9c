"""SoA host layout of the cell state and the face mesh, and their C views.

The reference keeps one ``Particle`` struct per Voronoi cell
(``src/part.rs:10-39``) and a ``Vec<VoronoiFace>`` plus the cell->face CSR
``voronoi_cell_face_connections`` (``src/space.rs:70-81``).  This library
keeps the same quantities as structure-of-arrays (one contiguous float64 block
per field, ``[components][n]``), which is the layout the GPU kernels read and
the layout of the C-ABI structs ``mvmm_cells`` / ``mvmm_mesh``
(``include/mvmm_gpu.h``).

Field meaning (reference name -> SoA field):

=================================  =====================  ==============
Particle field                     SoA field              shape
=================================  =====================  ==============
conserved  (m, p, E)               ``cons``               [5][n]
primitives (rho, v, P)             ``prim``               [5][n]
gradients  (5 x DVec3)             ``grad``               [15][n], row 3q+k
gradients_centroid                 ``gc``                 [3][n]
extrapolations                     ``extrap``             [5][n]
fluxes (pending accumulator)       ``facc``               [5][n]
volume                             ``volume``             [n]
loc / centroid / v / v_rel         ``loc`` ...            [3][n]
max_a_over_r, max_signal_velocity  same names             [n]
dt, timebin                        ``dt``, ``timebin``    [n] f64, [n] i8
=================================  =====================  ==============

Faces: ``left``/``right`` int32 (``right = -1`` is ``face.right() == None``),
``area`` [F], ``normal``/``centroid``/``shift`` [3][F] (``shift`` is zero when
``face.shift()`` is ``None``), ``csr_off`` int32 [N+1], ``csr_face`` int32.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

F64 = np.float64

CELL_FIELDS = (
    ("cons", 5), ("prim", 5), ("grad", 15), ("gc", 3), ("extrap", 5), ("facc", 5),
    ("volume", 1), ("loc", 3), ("centroid", 3), ("v", 3), ("v_rel", 3),
    ("max_a_over_r", 1), ("max_signal_velocity", 1), ("dt", 1),
)


CELL_ROWS = sum(k for _, k in CELL_FIELDS)


class CCells(ctypes.Structure):
    """C view of ``mvmm_cells`` / the oracle's ``orc_cells`` (same layout)."""

    _fields_ = [("n", ctypes.c_int64)] + [
        (name, ctypes.c_void_p) for name, _ in CELL_FIELDS
    ] + [("timebin", ctypes.c_void_p)]


class CMesh(ctypes.Structure):
    """C view of ``mvmm_mesh`` / the oracle's ``orc_mesh`` (same layout)."""

    _fields_ = [
        ("n_cells", ctypes.c_int64), ("n_faces", ctypes.c_int64),
        ("left", ctypes.c_void_p), ("right", ctypes.c_void_p),
        ("area", ctypes.c_void_p), ("normal", ctypes.c_void_p),
        ("centroid", ctypes.c_void_p), ("shift", ctypes.c_void_p),
        ("csr_off", ctypes.c_void_p), ("csr_face", ctypes.c_void_p),
    ]


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data


@dataclass
class Cells:
    """Cell state of one simulation, SoA float64 (timebin int8)."""

    n: int
    arrays: dict = field(default_factory=dict)

    @classmethod
    def zeros(cls, n: int) -> "Cells":
        c = cls(n=n)
        for name, k in CELL_FIELDS:
            c.arrays[name] = np.zeros((k, n) if k > 1 else (n,), dtype=F64)
        c.arrays["timebin"] = np.zeros(n, dtype=np.int8)
        return c

    @classmethod
    def packed(cls, n: int, block: np.ndarray, timebin: np.ndarray) -> "Cells":
        """Fields as views of one float64 block of ``CELL_ROWS * n`` values in
        ``CELL_FIELDS`` order, the device's own field order, so that
        ``mvmm_upload_cells`` / ``mvmm_download_cells`` move it in one copy."""
        assert block.dtype == F64 and block.size == CELL_ROWS * n and timebin.size == n
        c = cls(n=n)
        off = 0
        for name, k in CELL_FIELDS:
            v = block[off * n:(off + k) * n]
            c.arrays[name] = v.reshape(k, n) if k > 1 else v
            off += k
        c.arrays["timebin"] = timebin
        return c

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays")
        if arrays is not None and name in arrays:
            return arrays[name]
        raise AttributeError(name)

    def copy(self) -> "Cells":
        return Cells(n=self.n, arrays={k: v.copy() for k, v in self.arrays.items()})

    def cview(self) -> CCells:
        """The C struct of pointers to the arrays.  Kept while the same array
        objects (and the same n) are in place, as building it costs more than
        a call into the library; the cache holds the arrays, so an array that
        was replaced cannot hand its address to a new one."""
        arrs = tuple(self.arrays[name] for name, _ in CELL_FIELDS) + (self.arrays["timebin"],)
        cached = self.__dict__.get("_cview")
        if cached is not None and cached[0] == self.n and len(cached[1]) == len(arrs) and \
                all(a is b for a, b in zip(cached[1], arrs)):
            return cached[2]
        cv = CCells()
        cv.n = self.n
        for (name, _), a in zip(CELL_FIELDS, arrs):
            setattr(cv, name, _ptr(a))
        cv.timebin = _ptr(arrs[-1])
        self.__dict__["_cview"] = (self.n, arrs, cv)
        return cv

    def nbytes(self) -> int:
        return int(sum(a.nbytes for a in self.arrays.values()))


@dataclass
class Mesh:
    """Face list + cell->face CSR; what the host Voronoi step hands the hot path."""

    n_cells: int
    left: np.ndarray
    right: np.ndarray
    area: np.ndarray
    normal: np.ndarray
    centroid: np.ndarray
    shift: np.ndarray
    csr_off: np.ndarray
    csr_face: np.ndarray
    volume: np.ndarray          # per cell
    cell_centroid: np.ndarray   # [3][n]
    dimensionality: int = 1
    box: tuple = (1.0, 1.0, 1.0)
    periodic: bool = False

    @property
    def n_faces(self) -> int:
        return int(self.left.shape[0])

    def cview(self) -> CMesh:
        m = CMesh()
        m.n_cells = self.n_cells
        m.n_faces = self.n_faces
        for name in ("left", "right", "area", "normal", "centroid", "shift", "csr_off", "csr_face"):
            setattr(m, name, _ptr(getattr(self, name)))
        return m

    def check(self) -> None:
        """Structural invariants the kernels rely on (host-side bounds checks)."""
        n, f = self.n_cells, self.n_faces
        assert self.left.dtype == np.int32 and self.right.dtype == np.int32
        assert self.csr_off.dtype == np.int32 and self.csr_face.dtype == np.int32
        assert self.csr_off.shape == (n + 1,) and self.csr_off[0] == 0
        assert np.all(np.diff(self.csr_off) >= 0)
        assert self.csr_face.shape == (int(self.csr_off[-1]),)
        if f:
            assert self.left.min() >= 0 and self.left.max() < n
            assert self.right.max() < n and self.right.min() >= -1
            assert self.csr_face.min() >= 0 and self.csr_face.max() < f
        for a, shp in ((self.area, (f,)), (self.normal, (3, f)), (self.centroid, (3, f)), (self.shift, (3, f))):
            assert a.shape == shp and a.dtype == F64 and a.flags["C_CONTIGUOUS"]
        # every face appears in the CSR of its left cell and (if any) its right cell
        deg = np.bincount(self.left, minlength=n) + np.bincount(self.right[self.right >= 0], minlength=n)
        assert np.array_equal(deg, np.diff(self.csr_off)), "CSR does not match the face list"
