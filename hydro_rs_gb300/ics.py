"""Initial conditions: seeded synthetic inputs with the reference's shapes.

Follows ``InitialConditions::from_fn`` (``src/initial_conditions.rs:121-186``),
``Particle::from_ic`` (``src/part.rs:207-217``) and ``Space::first_init_parts``
/ ``Particle::first_init`` (``src/space.rs:571-594``, ``src/part.rs:200-205``).
Differences, chosen so that the oracle and the GPU see identical inputs: the
lattice jitter is symmetric, ``U[-j, j)`` times the spacing, and drawn from a
seeded numpy generator (the reference's is one-sided and unseeded,
``initial_conditions.rs:143,167-169``).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from .layout import Cells, Mesh
from .mesh import mesh_1d, mesh_voronoi

HLLC, EXACT, PVRS, AIRS, TSRS, TRRS, LINEAR_ADVECTION = 0, 1, 2, 3, 4, 5, 6
# gravity.kind (bin/main.rs:643-662): none, self_gravity, external potential Constant / Keplerian
GRAVITY_NONE, GRAVITY_SELF, GRAVITY_CONSTANT, GRAVITY_KEPLERIAN = 0, 1, 2, 3
PERIODIC, REFLECTIVE, OPEN, VACUUM = 0, 1, 2, 3
OPTIMAL_ORDER, GODUNOV = 0, 1
# engine.particle_motion (engine.rs:7-13)
FIXED, STEER, STEER_PAKMOR, FLUID = 0, 1, 2, 3
MOTION_NAMES = {"fixed": FIXED, "steer": STEER, "steer_pakmor": STEER_PAKMOR, "fluid": FLUID}
# riemann_solver.kind and engine.runner strings (bin/main.rs:625-673)
SOLVER_NAMES = {"HLLC": HLLC, "Exact": EXACT, "PVRS": PVRS, "AIRS": AIRS, "TSRS": TSRS, "TRRS": TRRS,
                "LinearAdvection": LINEAR_ADVECTION}
RUNNER_NAMES = {"OptimalOrder": OPTIMAL_ORDER, "Godunov": GODUNOV}


@dataclass
class Params:
    """Run parameters (the reference's hydrodynamics/time_integration/space config)."""

    gamma: float = 5.0 / 3.0
    cfl: float = 0.3
    riemann: int = HLLC
    boundary: int = REFLECTIVE
    dimensionality: int = 1
    sync_all: bool = True
    t_end: float = 0.2
    precision: int = 0  # 0 = plain FP64, 1 = FP32 faces / FP64 accumulate
    max_newton_iter: int = 1000
    runner: int = OPTIMAL_ORDER
    particle_motion: int = FIXED
    airs_threshold: float | None = None       # riemann_solver.threshold (required by AIRS)
    advection_velocity: tuple | None = None   # riemann_solver.velocity (required by LinearAdvection)
    eos: int = 0                              # 0 = EquationOfState::Ideal, 1 = Isothermal (gas_law.rs:59-63)
    isothermal_internal_energy: float = 0.0   # the Isothermal payload
    # gravity solver (bin/main.rs:643-662): GRAVITY_* kind, softening_length,
    # Potential::Constant acceleration, KeplerianPotential position, and whether
    # the accelerations (external potential or self-gravity) are computed at the
    # runner's "TODO: gravity" point (the reference never computes them)
    gravity: int = 0
    gravity_softening: float = 0.0
    gravity_acceleration: tuple = (0.0, 0.0, 0.0)
    gravity_position: tuple = (0.0, 0.0, 0.0)
    gravity_accelerations: bool = False
    # 1: the cell-wise limiter's face offsets in flux_exchange's frame instead of
    # the reference's (runner/hydrodynamics.rs:119, which across a periodic seam
    # are a box length long); not the reference's arithmetic
    limiter_frame: int = 0

    def gravity_fields(self):
        """The members of the C parameter structs after box_size, in order: the
        gravity solver's, then limiter_frame."""
        return (int(self.gravity), float(self.gravity_softening),
                (ctypes.c_double * 3)(*[float(x) for x in self.gravity_acceleration]),
                (ctypes.c_double * 3)(*[float(x) for x in self.gravity_position]), int(self.gravity_accelerations),
                int(self.limiter_frame))

    def solver_extras(self):
        """(threshold, velocity) as passed to the C structs; NaN marks a missing value."""
        thr = math.nan if self.airs_threshold is None else float(self.airs_threshold)
        v = (math.nan,) * 3 if self.advection_velocity is None else tuple(float(x) for x in self.advection_velocity)
        return thr, v


@dataclass
class Problem:
    name: str
    params: Params
    mesh: Mesh
    cells: Cells
    extra: dict = field(default_factory=dict)


def gas_internal_energy_from_pressure(gamma, p, rho_inv):
    """gas_law.rs:81-88 (ideal gas)."""
    return p * rho_inv * (1.0 / (gamma - 1.0))


def lattice(box, num_part: int, dim: int, jitter: float, rng):
    """Generator positions as in from_fn (initial_conditions.rs:133-176)."""
    box = list(box)
    if dim < 2:
        box[1] = 1.0
    if dim < 3:
        box[2] = 1.0
    volume = box[0] * box[1] * box[2]
    nppul = (num_part / volume) ** (1.0 / dim)
    npx = int(round(box[0] * nppul))
    npy = int(round(box[1] * nppul)) if dim > 1 else 1
    npz = int(round(box[2] * nppul)) if dim > 2 else 1
    n = npx * npy * npz
    idx = np.arange(n)
    i = idx // (npy * npz)
    j = (idx - i * npy * npz) // npz
    k = idx - i * npy * npz - j * npz
    pert = np.zeros((3, n))
    if jitter:
        for a in range(dim):
            pert[a] = jitter * (2.0 * rng.random(n) - 1.0)
    x = np.empty((3, n))
    x[0] = (i + 0.5 + pert[0]) / npx * box[0]
    x[1] = (j + 0.5 + pert[1]) / npy * box[1]
    x[2] = (k + 0.5 + pert[2]) / npz * box[2]
    return x, tuple(box), volume / n, (npx, npy, npz)


def cells_from_ic(mesh: Mesh, x, mass, vel, u, gamma, iso_u=None) -> Cells:
    """Particle::from_ic + update_geometry + first_init (part.rs:151-217).

    iso_u: the isothermal internal energy of EquationOfState::Isothermal, whose
    pressure is (gamma - 1) iso_u rho (gas_law.rs:90-97); None for an ideal gas."""
    n = mesh.n_cells
    c = Cells.zeros(n)
    mass = np.asarray(mass, dtype=np.float64)
    vel = np.asarray(vel, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    c.cons[0] = mass
    c.cons[1:4] = mass * vel
    c.cons[4] = mass * u + 0.5 * mass * (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2])
    c.volume[:] = mesh.volume
    c.centroid[:] = mesh.cell_centroid
    c.loc[:] = x
    # State<Primitive>::from_conserved (physical_quantities.rs:213-226)
    with np.errstate(divide="ignore", invalid="ignore"):
        m_inv = 1.0 / mass
        rho = mass / mesh.volume
        v = c.cons[1:4] * m_inv
        lsq = c.cons[1] * c.cons[1] + c.cons[2] * c.cons[2] + c.cons[3] * c.cons[3]
        thermal = c.cons[4] - 0.5 * lsq * m_inv
        ui = thermal * m_inv
        p = (gamma - 1.0) * (ui if iso_u is None else iso_u) * rho
    pos = mass > 0
    c.prim[0] = np.where(pos, rho, 0.0)
    c.prim[1:4] = np.where(pos, v, 0.0)
    c.prim[4] = np.where(pos, p, 0.0)
    return c


def sod_1d(n: int = 1000, riemann: int = HLLC, t_end: float = 0.2, cfl: float = 0.3,
           boundary: int = REFLECTIVE, iso_u: float | None = None) -> Problem:
    """1D Sod shock tube (bin/main.rs:35-40 preset) on [0,1], reflective (or the
    given wall boundary: open or vacuum).  iso_u: an isothermal gas
    (EquationOfState::Isothermal) with that internal energy everywhere, so the
    density jump drives the flow (gas_law.rs:81-106)."""
    params = Params(gamma=5.0 / 3.0, cfl=cfl, riemann=riemann, boundary=boundary, dimensionality=1,
                    sync_all=True, t_end=t_end)
    if iso_u is not None:
        params.eos, params.isothermal_internal_energy = 1, float(iso_u)
    x, box, vpp, _ = lattice((1.0, 1.0, 1.0), n, 1, 0.0, None)
    mesh = mesh_1d(x[0], box=box, periodic=False)
    left = x[0] < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    vel = np.zeros((3, x.shape[1]))
    if iso_u is None:
        u = gas_internal_energy_from_pressure(params.gamma, p, 1.0 / rho)
    else:
        u = np.full(x.shape[1], float(iso_u))  # gas_internal_energy_from_pressure of the isothermal gas
    cells = cells_from_ic(mesh, x, rho * vpp, vel, u, params.gamma, iso_u=iso_u)
    return Problem("sod_1d" if iso_u is None else "sod_1d_isothermal", params, mesh, cells)


def riemann_1d(n: int, left_state, right_state, riemann: int, t_end: float, gamma: float = 5.0 / 3.0,
               cfl: float = 0.3, x0: float = 0.5) -> Problem:
    """One 1D Riemann problem (rho, v, P) | (rho, v, P) at x0, reflective walls."""
    params = Params(gamma=gamma, cfl=cfl, riemann=riemann, boundary=REFLECTIVE, dimensionality=1,
                    sync_all=True, t_end=t_end)
    x, box, vpp, _ = lattice((1.0, 1.0, 1.0), n, 1, 0.0, None)
    mesh = mesh_1d(x[0], box=box, periodic=False)
    lft = x[0] < x0
    rho = np.where(lft, left_state[0], right_state[0])
    vx = np.where(lft, left_state[1], right_state[1])
    p = np.where(lft, left_state[2], right_state[2])
    vel = np.zeros((3, x.shape[1]))
    vel[0] = vx
    u = gas_internal_energy_from_pressure(gamma, p, 1.0 / rho)
    cells = cells_from_ic(mesh, x, rho * vpp, vel, u, gamma)
    return Problem("riemann_1d", params, mesh, cells)


def kelvin_helmholtz_2d(nx: int = 256, seed: int = 2, riemann: int = EXACT, t_end: float = 1.5,
                        jitter: float = 0.1, cfl: float = 0.3) -> Problem:
    """2D shear layer on the periodic unit square (seeded +-jitter lattice)."""
    params = Params(gamma=5.0 / 3.0, cfl=cfl, riemann=riemann, boundary=PERIODIC, dimensionality=2,
                    sync_all=True, t_end=t_end)
    rng = np.random.default_rng(seed)
    x, box, vpp, _ = lattice((1.0, 1.0, 1.0), nx * nx, 2, jitter, rng)
    mesh = mesh_voronoi(x, 2, box, True)
    xn = x[0] / box[0]
    yn = x[1] / box[1]
    inner = np.abs(yn - 0.5) < 0.25
    rho = np.where(inner, 2.0, 1.0)
    vel = np.zeros_like(x)
    vel[0] = np.where(inner, 0.5, -0.5)
    vel[1] = 0.1 * np.sin(4.0 * math.pi * xn)
    p = np.full(x.shape[1], 2.5)
    u = gas_internal_energy_from_pressure(params.gamma, p, 1.0 / rho)
    cells = cells_from_ic(mesh, x, rho * vpp, vel, u, params.gamma)
    return Problem("kelvin_helmholtz_2d", params, mesh, cells)


def wall_flow_2d(nx: int = 32, boundary: int = REFLECTIVE, v=(1.5, 0.4), seed: int = 11, riemann: int = HLLC,
                 t_end: float = 0.5, jitter: float = 0.1, cfl: float = 0.3, dim: int = 2) -> Problem:
    """Flow into the walls of the unit square (cube for dim=3; seeded +-jitter
    lattice of nx per side, no periodic images): density 1 + 0.3 sin(2 pi x)
    sin(2 pi y), pressure 1, velocity v (v[2] = 0.3 v[1] in 3D) plus 0.2 sin(2 pi
    y) along x, generators moving with the fluid.  Generators next to the walls
    the flow heads for leave the box: a reflective box mirrors them back, an
    open or vacuum box loses them."""
    params = Params(gamma=5.0 / 3.0, cfl=cfl, riemann=riemann, boundary=boundary, dimensionality=dim,
                    sync_all=True, t_end=t_end, particle_motion=FLUID)
    rng = np.random.default_rng(seed)
    x, box, vpp, _ = lattice((1.0, 1.0, 1.0), nx ** dim, dim, jitter, rng)
    mesh = mesh_voronoi(x, dim, box, False)
    rho = 1.0 + 0.3 * np.sin(2.0 * math.pi * x[0]) * np.sin(2.0 * math.pi * x[1])
    vel = np.zeros_like(x)
    vel[0] = v[0] + 0.2 * np.sin(2.0 * math.pi * x[1])
    vel[1] = v[1]
    if dim == 3:
        vel[2] = 0.3 * v[1]
    u = gas_internal_energy_from_pressure(params.gamma, np.ones(x.shape[1]), 1.0 / rho)
    cells = cells_from_ic(mesh, x, rho * mesh.volume, vel, u, params.gamma)
    return Problem(f"wall_flow_{dim}d", params, mesh, cells)


def point_blast_3d(n1d: int = 128, seed: int = 3, riemann: int = HLLC, t_end: float = 0.05,
                   jitter: float = 0.1, sync_all: bool = False, cfl: float = 0.3) -> Problem:
    """3D point blast: E=1 of thermal energy split over cells within 2 spacings of the centre."""
    params = Params(gamma=5.0 / 3.0, cfl=cfl, riemann=riemann, boundary=PERIODIC, dimensionality=3,
                    sync_all=sync_all, t_end=t_end)
    rng = np.random.default_rng(seed)
    x, box, vpp, _ = lattice((1.0, 1.0, 1.0), n1d ** 3, 3, jitter, rng)
    mesh = mesh_voronoi(x, 3, box, True)
    n = x.shape[1]
    rho = np.ones(n)
    p = np.full(n, 1e-6)
    vel = np.zeros((3, n))
    u = gas_internal_energy_from_pressure(params.gamma, p, 1.0 / rho)
    mass = rho * vpp
    r = np.sqrt(((x - 0.5) ** 2).sum(axis=0))
    hot = r < 2.0 / n1d
    nh = int(hot.sum())
    u = np.where(hot, (1.0 / nh) / mass, u)
    cells = cells_from_ic(mesh, x, mass, vel, u, params.gamma)
    return Problem("point_blast_3d", params, mesh, cells, extra={"n_hot": nh})


def yee_cells(mesh: Mesh, x, beta: float, v_adv, gamma: float = 1.4, box_len: float = 10.0, T_inf: float = 1.0):
    """Isentropic (Yee) vortex centred in the box plus a uniform advection velocity,
    python/utils.py:242-256 (Hopkins 2016 appendix A), masses from the nominal
    per-cell volume as in from_fn."""
    c = x[:2] - 0.5 * box_len
    r2 = (c * c).sum(axis=0)
    temp = T_inf - (gamma - 1) * beta ** 2 / (8 * gamma * math.pi ** 2) * np.exp(1 - r2)
    rho = np.power(temp, 1 / (gamma - 1))
    v_fac = 0.5 * beta / math.pi * np.exp(0.5 * (1 - r2))
    vel = np.zeros_like(x)
    vel[0] = -c[1] * v_fac + v_adv[0]
    vel[1] = c[0] * v_fac + v_adv[1]
    u = temp / (gamma - 1)
    mass = rho * (box_len * box_len / x.shape[1])
    return cells_from_ic(mesh, x, mass, vel, u, gamma)


def yee_vortex_2d(nx: int, beta: float, v_adv, seed: int = 5, box_len: float = 10.0, t_end: float = 1.0,
                  riemann: int = HLLC, jitter: float = 0.1, cfl: float = 0.3) -> Problem:
    """Isentropic vortex on the periodic [0, box_len]^2 (T_inf = 1, gamma = 1.4), advected by v_adv."""
    gamma = 1.4
    params = Params(gamma=gamma, cfl=cfl, riemann=riemann, boundary=PERIODIC, dimensionality=2,
                    sync_all=True, t_end=t_end)
    rng = np.random.default_rng(seed)
    x, box, vpp, _ = lattice((box_len, box_len, 1.0), nx * nx, 2, jitter, rng)
    mesh = mesh_voronoi(x, 2, box, True)
    cells = yee_cells(mesh, x, beta, v_adv, gamma, box_len)
    return Problem("yee_vortex_2d", params, mesh, cells, extra={"beta": beta, "v_adv": tuple(v_adv)})


def riemann_batch_1d(n_instances: int = 512, seed: int = 4, n_min: int = 200, n_max: int = 20000,
                     riemann: int = EXACT, t_end: float = 0.15, gamma: float = 5.0 / 3.0):
    """Independent 1D Riemann problems: N log-uniform in [n_min, n_max]; rho_L, rho_R
    log-uniform in [0.1, 10]; P log-uniform in [1e-3, 1e3]; v uniform in [-2, 2];
    discontinuity at x = 0.5, reflective walls."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_instances):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        rho = 10 ** rng.uniform(-1, 1, 2)
        p = 10 ** rng.uniform(-3, 3, 2)
        v = rng.uniform(-2, 2, 2)
        out.append(riemann_1d(n, (rho[0], v[0], p[0]), (rho[1], v[1], p[1]), riemann, t_end, gamma=gamma))
    return out


def pack(problems):
    """Packs independent problems (same physics parameters) into one mesh union:
    cells and faces of problem k follow those of problem k-1, with indices
    offset.  Returns (Problem, cell_offsets, t_end array)."""
    from .layout import Cells, Mesh

    assert problems
    p0 = problems[0].params
    for q in problems[1:]:
        a, b = q.params, p0
        assert (a.gamma, a.cfl, a.riemann, a.boundary, a.dimensionality, a.sync_all, a.precision) == \
            (b.gamma, b.cfl, b.riemann, b.boundary, b.dimensionality, b.sync_all, b.precision), "mixed physics"
    n = [q.mesh.n_cells for q in problems]
    f = [q.mesh.n_faces for q in problems]
    cell_off = np.concatenate([[0], np.cumsum(n)]).astype(np.int64)
    face_off = np.concatenate([[0], np.cumsum(f)]).astype(np.int64)
    csr_len = [int(q.mesh.csr_off[-1]) for q in problems]
    csr_base = np.concatenate([[0], np.cumsum(csr_len)]).astype(np.int64)
    N, F = int(cell_off[-1]), int(face_off[-1])
    left = np.concatenate([q.mesh.left + cell_off[k] for k, q in enumerate(problems)]).astype(np.int32)
    right = np.concatenate([np.where(q.mesh.right >= 0, q.mesh.right + cell_off[k], -1)
                            for k, q in enumerate(problems)]).astype(np.int32)
    cat3 = lambda name: np.ascontiguousarray(np.concatenate([getattr(q.mesh, name) for q in problems], axis=1))
    csr_off = np.concatenate([[0]] + [q.mesh.csr_off[1:] + csr_base[k] for k, q in enumerate(problems)]).astype(np.int32)
    csr_face = np.concatenate([q.mesh.csr_face + face_off[k] for k, q in enumerate(problems)]).astype(np.int32)
    mesh = Mesh(n_cells=N, left=left, right=right, area=np.concatenate([q.mesh.area for q in problems]),
                normal=cat3("normal"), centroid=cat3("centroid"), shift=cat3("shift"), csr_off=csr_off,
                csr_face=csr_face, volume=np.concatenate([q.mesh.volume for q in problems]),
                cell_centroid=np.ascontiguousarray(np.concatenate([q.mesh.cell_centroid for q in problems], axis=1)),
                dimensionality=problems[0].mesh.dimensionality, box=problems[0].mesh.box,
                periodic=problems[0].mesh.periodic)
    cells = Cells(n=N)
    for name, arr in problems[0].cells.arrays.items():
        axis = 1 if arr.ndim == 2 else 0
        cells.arrays[name] = np.ascontiguousarray(np.concatenate([q.cells.arrays[name] for q in problems], axis=axis))
    t_end = np.array([q.params.t_end for q in problems], dtype=np.float64)
    return Problem("batch", p0, mesh, cells, extra={"n_instances": len(problems)}), cell_off, t_end


def unpack_cells(cells, cell_off):
    """Splits packed cell state back into one Cells per instance."""
    from .layout import Cells

    out = []
    for k in range(len(cell_off) - 1):
        a, b = int(cell_off[k]), int(cell_off[k + 1])
        c = Cells(n=b - a)
        for name, arr in cells.arrays.items():
            c.arrays[name] = np.ascontiguousarray(arr[..., a:b])
        out.append(c)
    return out
