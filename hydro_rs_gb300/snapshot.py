"""HDF5 snapshots and initial conditions in the reference's on-disk layout.

``write_snapshot`` writes what ``Space::dump`` writes (``src/space.rs:1283-1417``):
a ``Header`` group with the attributes ``Time``, ``BoxSize``, ``Numpart_Total``
and ``Dimension``; a ``PartType0`` group with one dataset per particle field
(``Coordinates``, ``Masses``, ``Densities``, ``Momenta``, ``Velocities``,
``Pressures``, ``TotalEnergies``, ``InternalEnergies``, ``Entropies``,
``Volumes``, ``Centroids``, ``ParticleVelocities``,
``GravitationalAccelerations``, ``Timestep``), vectors as one element of a
3-double array type per particle as the reference's ``[f64; 3]`` rows are; and
optionally ``VoronoiFaces`` (``Area``, ``Centroid``, ``Normal``, ``Left``,
``Right``).  ``write_ics`` / ``read_ics`` follow ``InitialConditions::save`` and
``InitialConditions::from_hdf5`` (``src/initial_conditions.rs:47-117, 336-416``).

No HDF5 library is available in this environment, so the files are written
directly from the HDF5 file-format specification (version 0 superblock,
version 1 object headers, symbol-table groups: a version 1 B-tree of group
nodes over symbol-table nodes, names in a local heap; contiguous datasets;
IEEE little-endian doubles, 64-bit integers and array types).  ``read`` is a
reader of exactly that subset, for the round trip.

``snapshot_of(sim)`` takes the state from the device (``mvmm_download_cells``)
at the simulation's current time.
"""
from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 16      # group leaf node K: a symbol-table node holds up to 2K entries
INTERNAL_K = 16  # group internal node K: a B-tree node holds up to 2K children
ENTRY_SIZE = 40  # symbol-table entry with 8-byte offsets


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


# ---- datatype messages -----------------------------------------------------
def _dt_float64() -> bytes:
    # class 1 (floating point), version 1; little-endian, implied MSB
    # normalisation (0x20), sign at bit 63; offset 0, precision 64, exponent at
    # 52 of 11 bits, mantissa at 0 of 52 bits, bias 1023
    return bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)


def _dt_int64(signed: bool) -> bytes:
    # class 0 (fixed point), version 1; little-endian, bit 3 = signed
    return bytes([0x10, 0x08 if signed else 0x00, 0, 0]) + struct.pack("<I", 8) + struct.pack("<HH", 0, 64)


def _dt_int32(signed: bool) -> bytes:
    return bytes([0x10, 0x08 if signed else 0x00, 0, 0]) + struct.pack("<I", 4) + struct.pack("<HH", 0, 32)


def _dt_array(base: bytes, base_size: int, dims) -> bytes:
    # class 10 (array), version 3: dimensionality, dimension sizes, base type
    size = base_size * int(np.prod(dims))
    body = bytes([len(dims)]) + b"".join(struct.pack("<I", d) for d in dims) + base
    return bytes([0x3A, 0, 0, 0]) + struct.pack("<I", size) + body


def _datatype(arr: np.ndarray, vector3: bool):
    """(datatype message, element dims) for an array of float64 / int64 / uint64 / int32."""
    kind = arr.dtype
    if kind == np.float64:
        base, bsize = _dt_float64(), 8
    elif kind == np.int64:
        base, bsize = _dt_int64(True), 8
    elif kind == np.uint64:
        base, bsize = _dt_int64(False), 8
    elif kind == np.int32:
        base, bsize = _dt_int32(True), 4
    else:
        raise TypeError(f"unsupported dtype {kind}")
    if vector3:
        return _dt_array(base, bsize, [3]), arr.shape[:-1]
    return base, arr.shape


# ---- header messages --------------------------------------------------------
def _msg(mtype: int, data: bytes, flags: int = 0) -> bytes:
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _dataspace(shape) -> bytes:
    # version 1: rank, no maximum dimensions
    return struct.pack("<BBBB4x", 1, len(shape), 0, 0) + b"".join(struct.pack("<Q", int(d)) for d in shape)


def _object_header(messages) -> bytes:
    body = b"".join(messages)
    # version 1 prefix (12 bytes) padded to 16 so that messages are 8-byte aligned
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


class _File:
    def __init__(self):
        self.buf = bytearray(96)  # the superblock is filled in last

    def alloc(self, data: bytes) -> int:
        pad = -len(self.buf) % 8
        self.buf += b"\0" * pad
        addr = len(self.buf)
        self.buf += data
        return addr

    def dataset(self, arr: np.ndarray, vector3: bool = False) -> int:
        arr = np.ascontiguousarray(arr)
        if arr.dtype.byteorder == ">":
            arr = arr.astype(arr.dtype.newbyteorder("<"))
        dt, shape = _datatype(arr, vector3)
        raw = arr.tobytes()
        addr = self.alloc(raw) if raw else UNDEF
        msgs = [
            _msg(0x0001, _dataspace(shape)),
            _msg(0x0003, dt, flags=1),  # constant
            # fill value, version 2: allocation late, write if set, no value defined
            _msg(0x0005, struct.pack("<BBBB", 2, 2, 2, 0), flags=1),
            # data layout, version 3: contiguous at addr, len(raw) bytes
            _msg(0x0008, struct.pack("<BBQQ", 3, 1, addr, len(raw))),
        ]
        return self.alloc(_object_header(msgs))

    def attribute(self, name: str, arr: np.ndarray) -> bytes:
        arr = np.ascontiguousarray(arr)
        dt, shape = _datatype(arr, False)
        nm = name.encode() + b"\0"
        ds = _dataspace(shape)
        data = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds)) + _pad8(nm) + _pad8(dt) + _pad8(ds) + arr.tobytes()
        return _msg(0x000C, data)

    def group(self, children, attrs=None) -> int:
        """children: {name: object header address}; attrs: {name: array}."""
        names = sorted(children, key=lambda s: s.encode())
        # local heap: the empty string at offset 0, then each name (8-byte padded)
        heap = bytearray(8)
        offs = {}
        for nm in names:
            offs[nm] = len(heap)
            heap += _pad8(nm.encode() + b"\0")
        heap_data = self.alloc(bytes(heap))
        heap_addr = self.alloc(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), UNDEF, heap_data))
        # symbol-table nodes of up to 2 LEAF_K entries, in name order
        per = 2 * LEAF_K
        chunks = [names[i:i + per] for i in range(0, len(names), per)] or [[]]
        if len(chunks) > 2 * INTERNAL_K:
            raise ValueError("too many objects in one group")
        snods = []
        for ch in chunks:
            ents = b"".join(struct.pack("<QQII16x", offs[nm], children[nm], 0, 0) for nm in ch)
            ents += b"\0" * (ENTRY_SIZE * (per - len(ch)))  # the node is read at its full size
            snods.append(self.alloc(b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)) + ents))
        # one B-tree leaf (level 0) over them; key i is the heap offset of the
        # last name below child i-1 (key 0: the empty string)
        keys = [0] + [offs[ch[-1]] if ch else 0 for ch in chunks]
        node = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(chunks) if names else 0, UNDEF, UNDEF)
        slots = 2 * INTERNAL_K
        kc = b""
        for i in range(slots):
            kc += struct.pack("<Q", keys[i] if i < len(keys) else 0)
            kc += struct.pack("<Q", snods[i] if (i < len(snods) and names) else 0)
        kc += struct.pack("<Q", keys[slots] if slots < len(keys) else 0)
        btree = self.alloc(node + kc)
        msgs = [_msg(0x0011, struct.pack("<QQ", btree, heap_addr))]
        for nm, a in (attrs or {}).items():
            msgs.append(self.attribute(nm, np.asarray(a)))
        return self.alloc(_object_header(msgs)), btree, heap_addr

    def finish(self, root_oh: int, root_btree: int, root_heap: int) -> bytes:
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, len(self.buf), UNDEF)
        sb += struct.pack("<QQII", 0, root_oh, 1, 0) + struct.pack("<QQ", root_btree, root_heap)
        assert len(sb) == 96
        self.buf[:96] = sb
        return bytes(self.buf)


def write(path: str, tree: dict) -> None:
    """Writes a tree {group: {"attrs": {...}, "datasets": {name: (array, vector3)}}}
    (groups directly under the root)."""
    f = _File()
    groups = {}
    for gname, g in tree.items():
        kids = {nm: f.dataset(np.asarray(a), v3) for nm, (a, v3) in g.get("datasets", {}).items()}
        groups[gname] = f.group(kids, g.get("attrs"))[0]
    root = f.group(groups)
    with open(path, "wb") as fh:
        fh.write(f.finish(*root))


# ---- reader of the subset written above -------------------------------------
def _parse_dt(b: bytes, o: int):
    cv = b[o]
    cls, ver = cv & 0x0F, cv >> 4
    size = struct.unpack_from("<I", b, o + 4)[0]
    if cls == 1:
        assert size == 8 and b[o + 1] & 1 == 0
        return np.dtype("<f8"), (), o + 8 + 12
    if cls == 0:
        signed = bool(b[o + 1] & 0x08)
        return np.dtype(("<i" if signed else "<u") + str(size)), (), o + 8 + 4
    if cls == 10:
        assert ver == 3
        nd = b[o + 8]
        dims = struct.unpack_from("<" + "I" * nd, b, o + 9)
        base, _, end = _parse_dt(b, o + 9 + 4 * nd)
        return base, tuple(dims), end
    raise ValueError(f"datatype class {cls} not supported")


def _messages(b: bytes, addr: int):
    ver, _, nmsg, _, size = struct.unpack_from("<BBHII", b, addr)
    assert ver == 1
    o, end, out = addr + 16, addr + 16 + size, []
    while o < end and len(out) < nmsg:
        mtype, msize, flags = struct.unpack_from("<HHB", b, o)
        out.append((mtype, o + 8, msize))
        o += 8 + msize
    return out


def _dataspace_shape(b, o):
    ver, rank = b[o], b[o + 1]
    assert ver == 1
    return struct.unpack_from("<" + "Q" * rank, b, o + 8)


def _read_object(b: bytes, addr: int):
    msgs = _messages(b, addr)
    types = {m[0]: m for m in msgs}
    if 0x0011 in types:  # a group
        btree, heap = struct.unpack_from("<QQ", b, types[0x0011][1])
        attrs = {}
        for mtype, o, _ in msgs:
            if mtype == 0x000C:
                _, _, nlen, dlen, slen = struct.unpack_from("<BBHHH", b, o)
                p = o + 8
                name = b[p:p + nlen - 1].decode()
                p += nlen + (-nlen % 8)
                dt, sub, _ = _parse_dt(b, p)
                p += dlen + (-dlen % 8)
                shape = _dataspace_shape(b, p)
                p += slen + (-slen % 8)
                n = int(np.prod(shape)) * int(np.prod(sub) if sub else 1)
                attrs[name] = np.frombuffer(b, dtype=dt, count=n, offset=p).copy()
        return {"attrs": attrs, "children": _read_group(b, btree, heap)}
    shape = _dataspace_shape(b, types[0x0001][1])
    dt, sub, _ = _parse_dt(b, types[0x0003][1])
    lo = types[0x0008][1]
    ver, cls, daddr, dsize = struct.unpack_from("<BBQQ", b, lo)
    assert ver == 3 and cls == 1
    full = tuple(shape) + tuple(sub)
    n = int(np.prod(full)) if full else 1
    if dsize == 0:
        return np.zeros(full, dtype=dt)
    return np.frombuffer(b, dtype=dt, count=n, offset=daddr).reshape(full).copy()


def _read_group(b: bytes, btree: int, heap: int):
    assert b[heap:heap + 4] == b"HEAP"
    _, hsize, _, hdata = struct.unpack_from("<B3xQQQ", b, heap + 4)
    assert b[btree:btree + 4] == b"TREE"
    ntype, level, used = struct.unpack_from("<BBH", b, btree + 4)
    assert ntype == 0 and level == 0
    out = {}
    p = btree + 24
    for i in range(used):
        child = struct.unpack_from("<Q", b, p + 16 * i + 8)[0]
        assert b[child:child + 4] == b"SNOD"
        nsym = struct.unpack_from("<H", b, child + 6)[0]
        for k in range(nsym):
            noff, oh = struct.unpack_from("<QQ", b, child + 8 + ENTRY_SIZE * k)
            end = b.index(b"\0", hdata + noff)
            out[b[hdata + noff:end].decode()] = _read_object(b, oh)
    return out


def read(path: str) -> dict:
    with open(path, "rb") as fh:
        b = fh.read()
    assert b[:8] == SIGNATURE and b[8] == 0
    eof = struct.unpack_from("<Q", b, 40)[0]
    assert eof == len(b)
    root_oh = struct.unpack_from("<Q", b, 64)[0]
    return _read_object(b, root_oh)


# ---- the reference's layouts -------------------------------------------------
def _entropy(gamma, u, rho, eos=0, iso_u=0.0):
    """GasLaw::gas_entropy_from_internal_energy (gas_law.rs:108-122)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        uu = u if eos == 0 else np.full_like(u, iso_u)
        return (gamma - 1.0) * uu * np.power(rho, 1.0 - gamma)


def snapshot_tree(cells, mesh, params, time: float, a_grav=None, save_faces: bool = True) -> dict:
    """Space::dump's groups for a cell state (space.rs:1283-1417)."""
    n = cells.n
    with np.errstate(divide="ignore", invalid="ignore"):
        # Particle::internal_energy (part.rs:314-317)
        u = (cells.cons[4] - 0.5 * (cells.cons[1:4] * cells.prim[1:4]).sum(axis=0)) / cells.cons[0]
    box = np.asarray(mesh.box, dtype=np.float64)
    pt0 = {
        "Coordinates": (cells.loc.T, True),
        "Masses": (cells.cons[0], False),
        "Densities": (cells.prim[0], False),
        "Momenta": (cells.cons[1:4].T, True),
        "Velocities": (cells.prim[1:4].T, True),
        "Pressures": (cells.prim[4], False),
        "TotalEnergies": (cells.cons[4], False),
        "InternalEnergies": (u, False),
        "Entropies": (_entropy(params.gamma, u, cells.prim[0], params.eos, params.isothermal_internal_energy), False),
        "Volumes": (cells.volume, False),
        "Centroids": (cells.centroid.T, True),
        "ParticleVelocities": (cells.v.T, True),
        "GravitationalAccelerations": ((np.zeros((n, 3)) if a_grav is None else np.asarray(a_grav).T), True),
        "Timestep": (cells.dt, False),
    }
    tree = {
        "Header": {"attrs": {"Time": np.array([time]), "BoxSize": box,
                             "Numpart_Total": np.array([n, 0, 0, 0, 0], dtype=np.uint64),
                             "Dimension": np.array([params.dimensionality], dtype=np.uint64)}},
        "PartType0": {"datasets": pt0},
    }
    if save_faces:
        tree["VoronoiFaces"] = {"datasets": {
            "Area": (mesh.area, False),
            "Centroid": (mesh.centroid.T, True),
            "Normal": (mesh.normal.T, True),
            "Left": (mesh.left.astype(np.uint64), False),
            "Right": (mesh.right.astype(np.int64), False),
        }}
    return tree


def write_snapshot(path: str, cells, mesh, params, time: float, a_grav=None, save_faces: bool = True) -> None:
    write(path, snapshot_tree(cells, mesh, params, time, a_grav, save_faces))


def snapshot_of(sim, path: str, save_faces: bool = True) -> None:
    """Space::dump of a GPU simulation: the state comes from the device."""
    p = sim.problem.params
    time = sim.ti_current * (p.t_end / float(1 << 57))  # TimestepInfo::dt_from_dti(ti_current)
    write_snapshot(path, sim.state(), sim.mesh, p, time, save_faces=save_faces)


def write_ics(path: str, loc, masses, velocities, internal_energy, box, dimensionality: int,
              volumes=None, smoothing_lengths=None, ids=None) -> None:
    """InitialConditions::save (initial_conditions.rs:336-416): coordinates and
    velocities as flat 3N arrays, smoothing lengths 1.5 x the cell radius."""
    loc = np.asarray(loc, dtype=np.float64)
    n = loc.shape[1]
    if smoothing_lengths is None:
        vol = np.asarray(volumes, dtype=np.float64)
        if dimensionality == 1:
            r = 0.5 * vol
        elif dimensionality == 2:
            r = np.sqrt(vol / np.pi)
        else:
            r = np.power(0.25 * 3.0 / np.pi * vol, 1.0 / 3.0)
        smoothing_lengths = 1.5 * r
    ids = np.arange(1, n + 1, dtype=np.uint64) if ids is None else np.asarray(ids, dtype=np.uint64)
    pt0 = {
        "Coordinates": (loc.T.reshape(-1), False),
        "Masses": (np.asarray(masses, dtype=np.float64), False),
        "Velocities": (np.asarray(velocities, dtype=np.float64).T.reshape(-1), False),
        "InternalEnergy": (np.asarray(internal_energy, dtype=np.float64), False),
        "SmoothingLength": (np.asarray(smoothing_lengths, dtype=np.float64), False),
        "ParticleIDs": (ids, False),
    }
    if volumes is not None:
        pt0["Volumes"] = (np.asarray(volumes, dtype=np.float64), False)
    tree = {
        "Header": {"attrs": {"BoxSize": np.asarray(box, dtype=np.float64),
                             "NumPart_Total": np.array([n, 0, 0, 0, 0], dtype=np.uint64),
                             "Dimension": np.array([dimensionality], dtype=np.uint64),
                             "Flag_Entropy_ICs": np.array([0], dtype=np.int32),
                             "NumPart_Total_HighWord": np.array([0, 0, 0, 0, 0], dtype=np.int32)}},
        "PartType0": {"datasets": pt0},
    }
    write(path, tree)


def read_ics(path: str) -> dict:
    """InitialConditions::from_hdf5 (initial_conditions.rs:47-117): header,
    coordinates and velocities [3][n], masses and internal energies [n]."""
    t = read(path)["children"]
    h = t["Header"]["attrs"]
    n = int(h["NumPart_Total"][0])
    dim = int(h["Dimension"][0])
    periodic = bool(h["Periodic"][0]) if "Periodic" in h else False
    box = list(np.asarray(h["BoxSize"], dtype=np.float64))
    for i in range(dim, 3):
        if len(box) < i + 1:
            box.append(1.0)
        else:
            box[i] = 1.0
    d = t["PartType0"]["children"]
    coords = np.asarray(d["Coordinates"]).reshape(-1)
    vel = np.asarray(d["Velocities"]).reshape(-1)
    assert coords.size == 3 * n and vel.size == 3 * n, "Incorrect length of coordinates / velocities"
    assert d["Masses"].size == n and d["InternalEnergy"].size == n
    return {"num_part": n, "dimension": dim, "periodic": periodic, "box_size": tuple(box[:3]),
            "coordinates": coords.reshape(n, 3).T.copy(), "velocities": vel.reshape(n, 3).T.copy(),
            "masses": np.asarray(d["Masses"]), "internal_energy": np.asarray(d["InternalEnergy"])}


def problem_from_ics(path: str, params):
    """A Problem from an initial-conditions file: the generators' Voronoi mesh
    built on the host (as Space::initialize builds it, space.rs:88-211) and the
    cells from the stored masses, velocities and internal energies
    (Particle::from_ic + first_init, part.rs:200-217).  params: an ics.Params
    (its dimensionality and box are taken from the file)."""
    from . import ics
    from .mesh import mesh_1d, mesh_voronoi

    d = read_ics(path)
    params.dimensionality = d["dimension"]
    x = d["coordinates"]
    box = d["box_size"]
    if d["dimension"] == 1:
        mesh = mesh_1d(x[0], box=box, periodic=d["periodic"])
    else:
        mesh = mesh_voronoi(x, d["dimension"], box, d["periodic"])
    cells = ics.cells_from_ic(mesh, x, d["masses"], d["velocities"], d["internal_energy"], params.gamma)
    return ics.Problem("from_ics", params, mesh, cells)
