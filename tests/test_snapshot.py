"""HDF5 snapshots and initial conditions (hydro_rs_gb300/snapshot.py) on the CPU.

No HDF5 library is installed, so the files are checked two ways: their
structures against the HDF5 file-format specification's fixed layouts
(signatures, the superblock's end-of-file address, node sizes, sorted names),
and by a round trip through the module's reader, bit for bit.  The group and
dataset names, element types and shapes are the reference's
(space.rs:1283-1417, initial_conditions.rs:336-416).
"""
import os
import struct

import numpy as np

from hydro_rs_gb300 import ics
from hydro_rs_gb300 import snapshot as S
from oracle import oracle as O

PT0 = ["Centroids", "Coordinates", "Densities", "Entropies", "GravitationalAccelerations", "InternalEnergies",
       "Masses", "Momenta", "ParticleVelocities", "Pressures", "Timestep", "TotalEnergies", "Velocities", "Volumes"]


def _state():
    p = ics.kelvin_helmholtz_2d(16, riemann=ics.HLLC)
    o = O.OracleSim(p)
    o.run(max_steps=5)
    return p, o.state()


def test_snapshot_round_trip(tmp_path):
    p, st = _state()
    fn = os.path.join(tmp_path, "snap.hdf5")
    S.write_snapshot(fn, st, p.mesh, p.params, 0.125)
    t = S.read(fn)["children"]
    assert sorted(t) == ["Header", "PartType0", "VoronoiFaces"]
    h = t["Header"]["attrs"]
    assert h["Time"].tolist() == [0.125] and h["BoxSize"].tolist() == [1.0, 1.0, 1.0]
    assert h["Numpart_Total"].dtype == np.uint64 and h["Numpart_Total"].tolist() == [st.n, 0, 0, 0, 0]
    assert h["Dimension"].tolist() == [2]
    d = t["PartType0"]["children"]
    assert sorted(d) == PT0
    pairs = {"Coordinates": st.loc.T, "Masses": st.cons[0], "Densities": st.prim[0], "Momenta": st.cons[1:4].T,
             "Velocities": st.prim[1:4].T, "Pressures": st.prim[4], "TotalEnergies": st.cons[4],
             "Volumes": st.volume, "Centroids": st.centroid.T, "ParticleVelocities": st.v.T, "Timestep": st.dt}
    for k, v in pairs.items():
        assert d[k].dtype == np.float64 and np.array_equal(d[k], v), k
    u = (st.cons[4] - 0.5 * (st.cons[1:4] * st.prim[1:4]).sum(axis=0)) / st.cons[0]
    assert np.array_equal(d["InternalEnergies"], u)  # Particle::internal_energy (part.rs:314-317)
    g = p.params.gamma
    assert np.allclose(d["Entropies"], (g - 1.0) * u * st.prim[0] ** (1.0 - g), rtol=1e-15, atol=0)
    assert np.all(d["GravitationalAccelerations"] == 0.0) and d["GravitationalAccelerations"].shape == (st.n, 3)
    f = t["VoronoiFaces"]["children"]
    assert f["Left"].dtype == np.uint64 and f["Right"].dtype == np.int64
    assert np.array_equal(f["Right"], p.mesh.right) and np.array_equal(f["Area"], p.mesh.area)
    assert np.array_equal(f["Normal"], p.mesh.normal.T)


def test_file_structure(tmp_path):
    """Fixed layouts of the specification: version 0 superblock with the file's
    length as its end-of-file address; the root group's symbol-table entry
    points at an object header whose symbol-table message names a B-tree
    ("TREE", group nodes, level 0) and a local heap ("HEAP"); each B-tree child
    is a symbol-table node ("SNOD", version 1) of 2K 40-byte entries whose
    names are in strictly increasing byte order."""
    p, st = _state()
    fn = os.path.join(tmp_path, "snap.hdf5")
    S.write_snapshot(fn, st, p.mesh, p.params, 0.0)
    b = open(fn, "rb").read()
    assert b[:8] == b"\x89HDF\r\n\x1a\n" and b[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])
    leaf_k, internal_k = struct.unpack_from("<HH", b, 16)
    assert struct.unpack_from("<Q", b, 40)[0] == len(b)
    root = struct.unpack_from("<Q", b, 64)[0]
    assert struct.unpack_from("<I", b, 72)[0] == 1  # cache type 1: B-tree and heap in the scratch pad

    def walk(oh):
        assert oh % 8 == 0 and b[oh] == 1  # version 1 object header, 8-byte aligned
        n_msg, _, size = struct.unpack_from("<HII", b, oh + 2)
        o, names_seen = oh + 16, 0
        for _ in range(n_msg):
            mtype, msize = struct.unpack_from("<HH", b, o)
            assert msize % 8 == 0
            if mtype == 0x0011:
                btree, heap = struct.unpack_from("<QQ", b, o + 8)
                assert b[btree:btree + 4] == b"TREE" and b[btree + 4] == 0 and b[btree + 5] == 0
                assert b[heap:heap + 4] == b"HEAP"
                hdata = struct.unpack_from("<Q", b, heap + 24)[0]
                used = struct.unpack_from("<H", b, btree + 6)[0]
                prev = b""
                for i in range(used):
                    snod = struct.unpack_from("<Q", b, btree + 24 + 16 * i + 8)[0]
                    assert b[snod:snod + 4] == b"SNOD" and b[snod + 4] == 1
                    for k in range(struct.unpack_from("<H", b, snod + 6)[0]):
                        noff, child = struct.unpack_from("<QQ", b, snod + 8 + 40 * k)
                        name = b[hdata + noff:b.index(b"\0", hdata + noff)]
                        assert name > prev
                        prev = name
                        names_seen += 1
                        walk(child)
            o += 8 + msize
        assert o == oh + 16 + size
        return names_seen

    assert walk(root) == 3
    assert leaf_k == S.LEAF_K and internal_k == S.INTERNAL_K


def test_ics_round_trip_and_problem(tmp_path):
    """InitialConditions::save then from_hdf5; a problem built from the file
    steps like the one built from the same arrays."""
    p = ics.sod_1d(64)
    c = p.cells
    u = c.cons[4] / c.cons[0]  # at rest: all energy internal
    fn = os.path.join(tmp_path, "ic.hdf5")
    S.write_ics(fn, c.loc, c.cons[0], c.prim[1:4], u, p.mesh.box, 1, volumes=c.volume)
    raw = S.read(fn)["children"]
    d = raw["PartType0"]["children"]
    assert d["Coordinates"].shape == (3 * c.n,) and d["ParticleIDs"].tolist() == list(range(1, c.n + 1))
    assert np.allclose(d["SmoothingLength"], 1.5 * 0.5 * c.volume, rtol=0, atol=0)
    assert raw["Header"]["attrs"]["NumPart_Total"].tolist() == [c.n, 0, 0, 0, 0]
    r = S.read_ics(fn)
    assert r["num_part"] == c.n and r["dimension"] == 1 and not r["periodic"]
    assert np.array_equal(r["coordinates"], c.loc) and np.array_equal(r["masses"], c.cons[0])
    q = S.problem_from_ics(fn, ics.Params(gamma=p.params.gamma, cfl=p.params.cfl, riemann=p.params.riemann,
                                          boundary=p.params.boundary, sync_all=True, t_end=p.params.t_end))
    for k in ("cons", "prim", "volume", "loc"):
        assert np.allclose(getattr(q.cells, k), getattr(c, k), rtol=1e-15, atol=1e-15), k
    a, b = O.OracleSim(p), O.OracleSim(q)
    a.run(max_steps=20)
    b.run(max_steps=20)
    assert a.ti_current == b.ti_current
    assert np.allclose(a.state().cons, b.state().cons, rtol=1e-13, atol=1e-15)
