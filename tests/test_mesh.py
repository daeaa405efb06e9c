"""Mesh builder checks (host side; the reference's space.rs tests)."""
import math

import numpy as np
import pytest

from hydro_rs_gb300 import ics
from hydro_rs_gb300.mesh import mesh_1d, mesh_voronoi


def test_1d_mesh_matches_reference_test():
    """space.rs:1453-1491: 4 generators in [0,1], volumes and face centroids."""
    m = mesh_1d(np.array([0.25, 0.65, 0.75, 0.85]))
    m.check()
    assert np.allclose(m.volume, [0.45, 0.25, 0.1, 0.2], atol=1e-10)
    assert m.n_faces == 5
    assert np.allclose(m.area, 1.0)
    assert np.allclose(m.centroid[0], [0.0, 0.45, 0.7, 0.8, 1.0])
    assert list(m.right) == [-1, 1, 2, 3, -1]


def _closure(m):
    acc = np.zeros((3, m.n_cells))
    for k in range(3):
        np.add.at(acc[k], m.left, m.area * m.normal[k])
        rr = m.right >= 0
        np.add.at(acc[k], m.right[rr], -m.area[rr] * m.normal[k][rr])
    return np.abs(acc).max()


@pytest.mark.parametrize("periodic", [False, True])
def test_2d_invariants(periodic):
    """space.rs:1493-1529: total volume = box, perimeter above the isoperimetric bound."""
    rng = np.random.default_rng(1)
    x, box, _, _ = ics.lattice((2.0, 2.0, 1.0), 256, 2, 0.1, rng)
    m = mesh_voronoi(x, 2, box, periodic)
    m.check()
    assert abs(m.volume.sum() - 4.0) <= 1e-12 * 4
    per = np.bincount(m.left, weights=m.area, minlength=m.n_cells)
    rr = m.right >= 0
    per += np.bincount(m.right[rr], weights=m.area[rr], minlength=m.n_cells)
    radius = np.sqrt(m.volume / math.pi)
    assert np.all(per > 2 * math.pi * radius)
    assert _closure(m) < 1e-13
    if periodic:
        assert np.all(m.right >= 0)
    else:
        assert np.sum(m.right < 0) > 0


@pytest.mark.parametrize("periodic", [False, True])
def test_3d_invariants(periodic):
    """space.rs:1531-1567: total volume, isoperimetric bound; closed cells."""
    rng = np.random.default_rng(2)
    x, box, _, _ = ics.lattice((2.0, 2.0, 2.0), 512, 3, 0.1, rng)
    m = mesh_voronoi(x, 3, box, periodic)
    m.check()
    assert abs(m.volume.sum() - 8.0) <= 1e-11 * 8
    area = np.bincount(m.left, weights=m.area, minlength=m.n_cells)
    rr = m.right >= 0
    area += np.bincount(m.right[rr], weights=m.area[rr], minlength=m.n_cells)
    radius = (3.0 / 4.0 / math.pi * m.volume) ** (1.0 / 3.0)
    assert np.all(area > 4 * math.pi * radius * radius)
    assert _closure(m) < 1e-12


def test_periodic_shift_convention():
    """A periodic face stores the image offset of its right cell (flux.rs:34-38)."""
    p = ics.kelvin_helmholtz_2d(8)
    m = p.mesh
    loc = p.cells.loc
    d = loc[:, m.right] + m.shift - loc[:, m.left]
    # every face joins generators that are close in the periodic sense
    assert np.abs(d).max() < 3.0 / 8
    # normal points from left to the (shifted) right generator
    dots = (d * m.normal).sum(axis=0)
    assert np.all(dots > 0)


@pytest.mark.parametrize("dim,periodic", [(2, True), (2, False), (3, True), (3, False)])
def test_builder_is_deterministic_across_thread_counts(dim, periodic):
    """The cells are clipped in parallel and the face list and CSR assembled in
    parallel: the mesh is the same bits whatever the number of threads."""
    rng = np.random.default_rng(17)
    n1d = 24 if dim == 2 else 7
    x, box, _, _ = ics.lattice((1.0, 1.0, 1.0), n1d ** dim, dim, 0.3, rng)
    meshes = [mesh_voronoi(x, dim, box, periodic, n_threads=t) for t in (1, 3, 8)]
    for m in meshes[1:]:
        for name in ("left", "right", "area", "normal", "centroid", "shift", "csr_off", "csr_face", "volume",
                     "cell_centroid"):
            a, b = getattr(meshes[0], name), getattr(m, name)
            assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), name
    m = meshes[0]
    for i in range(m.n_cells):  # each cell's faces in increasing index, each touching it
        fs = m.csr_face[m.csr_off[i]:m.csr_off[i + 1]]
        assert np.all(np.diff(fs) > 0)
        assert np.all((m.left[fs] == i) | (m.right[fs] == i))
