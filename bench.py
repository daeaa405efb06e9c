"""Benchmark: active-face updates/s of the per-face finite-volume update.

Workload (one "step" = one OptimalOrderRunner step): the 2D shear-layer
(Kelvin-Helmholtz) problem on the periodic unit square, 256x256 generators on a
seeded +-0.1-jittered lattice (65,536 cells, 196,608 Voronoi faces), exact
Riemann solver, gamma = 5/3, all cells active every step.  Inputs are seeded
synthetic data of that shape; the working set (~40-70 MB) is below the L2 size,
so L2 is flushed (256 MB write) before every timed step.

Headline ``value``: the plain FP64 drop-in (the reference's arithmetic, the
same configuration the reference arm runs), device-resident; ``e2e`` the same
through the C ABI with host buffers (copies inside the timed region).  The
line also carries the roofline of the face stage (HBM, and FP64 against a
DGEMM measured here), the FP32-face / FP64-accumulate form under
``fp32_face`` (its throughput, end-to-end number, roofline and L1 density
error against the plain FP64 result), and the CPU oracle timed on the host
cores.

``--impl reference`` times the CPU restatement of the reference (the oracle,
OpenMP over all host cores): the Rust reference cannot be built here (no Rust
toolchain), so the C restatement is the reference arm.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "active-face updates/s"
UNIT = "faces/s"
NX = 256
L2_FLUSH_BYTES = 256 << 20
PRECISION_FP64 = "fp64 (the reference's arithmetic: the plain drop-in form)"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def aggregate_replicas(times_ms, faces, all_reduce_max, all_reduce_sum):
    """Replica scaling (no data-path collective): the job's time is the slowest
    rank's, its work the sum over ranks."""
    return all_reduce_max(times_ms), all_reduce_sum(faces)


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


WORKLOADS = {
    # the headline: 2D shear layer, 256^2 jittered lattice, exact solver, all cells active
    "kh2d": "kelvin_helmholtz_2d {n}x{n} jittered periodic Voronoi, exact Riemann solver, gamma=5/3",
    # the shear layer with the HLLC solver (no root finding: the plain form's face stage streams)
    "kh2d_hllc": "kelvin_helmholtz_2d {n}x{n} jittered periodic Voronoi, HLLC Riemann solver, gamma=5/3",
    # 1D Sod shock tube, reflective walls, HLLC, synchronised steps
    "sod1d": "sod_1d {n} cells, reflective, HLLC, gamma=5/3",
    # 3D point blast, 128^3 jittered lattice, HLLC, hierarchical time bins
    "blast3d": "point_blast_3d {n}^3 jittered periodic Voronoi, HLLC, hierarchical time bins, gamma=5/3",
    # {n} independent 1D Riemann problems packed in one batch, N log-uniform in [200, 20000]
    "batch1d": "{n} independent 1D Riemann problems (N log-uniform 200..20000), exact solver, one batch, t_end=0.15",
    # the same batch with the PVRS solver
    "batch1d_pvrs": "{n} independent 1D Riemann problems (N log-uniform 200..20000), PVRS solver, one batch, "
                    "t_end=0.15",
    # moving mesh: the shear layer with steered generators, host Voronoi rebuild every step
    "kh2d_moving": "kelvin_helmholtz_2d {n}x{n} jittered periodic Voronoi, exact Riemann solver, gamma=5/3, "
                   "steered generators (particle_motion=steer), mesh rebuilt on the host every step",
    # the shear layer with any of the reference's solvers and runners (--riemann, --runner)
    "kh2d_solver": "kelvin_helmholtz_2d {n}x{n} jittered periodic Voronoi, {riemann} Riemann solver, {runner} runner, "
                   "gamma=5/3",
    # self-gravity kicks: the shear layer with the direct O(N^2) sum over j > i every step
    "kh2d_selfgrav": "kelvin_helmholtz_2d {n}x{n} jittered periodic Voronoi, HLLC, gamma=5/3, self-gravity "
                     "(softening 0.01) accelerations computed and kicked every step",
    # served: Poisson stream (50 req/s) of {n} isentropic-vortex runs, 32^2..512^2, HLLC, t_end=1
    "serve2d": "{n} served isentropic-vortex requests (Poisson 50/s, 32^2..512^2 periodic Voronoi, HLLC, t_end=1)",
}
DATA = {
    "kh2d_solver": "synthetic (seeded jittered lattice, shear-layer ICs)",
    "kh2d_selfgrav": "synthetic (seeded jittered lattice, shear-layer ICs)",
    "kh2d": "synthetic (seeded jittered lattice, shear-layer ICs)",
    "kh2d_hllc": "synthetic (seeded jittered lattice, shear-layer ICs)",
    "sod1d": "synthetic (uniform 1D lattice, Sod ICs)",
    "blast3d": "synthetic (seeded jittered cubic lattice, point-blast ICs)",
    "batch1d": "synthetic (seeded random 1D Riemann problems)",
    "batch1d_pvrs": "synthetic (seeded random 1D Riemann problems)",
}
DEFAULT_N = {"kh2d_solver": NX, "kh2d_selfgrav": 128, "kh2d_moving": NX, "kh2d": NX, "kh2d_hllc": 1024, "sod1d": 1000, "blast3d": 128, "batch1d": 512, "batch1d_pvrs": 512, "serve2d": 60}


# AIRiemannSolver's threshold and LinearAdvection's velocity for the kh2d_solver workload
AIRS_THRESHOLD = 2.0
ADVECTION_VELOCITY = (0.7, -0.4, 0.2)


def _workload_name(args) -> str:
    return WORKLOADS[args.workload].format(n=args.nx, riemann=args.riemann, runner=args.runner)


def _problem(nx=NX, workload="kh2d", riemann="TSRS", runner="OptimalOrder"):
    from hydro_rs_gb300 import ics

    t0 = time.perf_counter()
    if workload in ("batch1d", "batch1d_pvrs"):
        kind = ics.PVRS if workload == "batch1d_pvrs" else ics.EXACT
        probs = ics.riemann_batch_1d(nx, seed=4, riemann=kind, t_end=0.15)
        p, off, te = ics.pack(probs)
        p.extra.update(cell_offsets=off, t_end=te, problems=probs)
    elif workload == "sod1d":
        p = ics.sod_1d(nx)
    elif workload == "blast3d":
        p = ics.point_blast_3d(nx, seed=3, riemann=ics.HLLC, t_end=0.05, sync_all=False)
    elif workload == "kh2d_solver":
        p = ics.kelvin_helmholtz_2d(nx, seed=2, riemann=ics.SOLVER_NAMES[riemann], t_end=1.5)
        p.params.runner = ics.RUNNER_NAMES[runner]
        p.params.airs_threshold = AIRS_THRESHOLD
        p.params.advection_velocity = ADVECTION_VELOCITY
    else:
        kind = ics.HLLC if workload in ("kh2d_hllc", "kh2d_selfgrav") else ics.EXACT
        p = ics.kelvin_helmholtz_2d(nx, seed=2, riemann=kind, t_end=1.5)
        if workload == "kh2d_selfgrav":
            p.params.gravity, p.params.gravity_softening = ics.GRAVITY_SELF, 0.01
            p.params.gravity_accelerations = True
    return p, time.perf_counter() - t0


def _cpu_sample(problem, label, budget_s: float = 10.0, max_steps: int = 400):
    """The oracle on all host cores, and beside it on one core (a shorter sample)."""
    out = _cpu_sample_threads(problem, label, os.cpu_count() or 1, budget_s, max_steps)
    one = _cpu_sample_threads(problem, label, 1, budget_s / 3, max_steps)
    out["one_thread"] = {"value": one["value"], "sample": one["sample"]}
    return out


def _cpu_sample_threads(problem, label, threads, budget_s, max_steps):
    """The oracle on `threads` host threads: warm-up step, then steps until the budget."""
    from oracle import oracle as O

    if "problems" in problem.extra:  # a batch: the oracle runs one simulation after another
        faces, dt, n = 0, 0.0, 0
        for q in problem.extra["problems"]:
            sim = O.OracleSim(q, n_threads=threads)
            sim.step()
            f0 = sim.active_faces
            t0 = time.perf_counter()
            sim.run(max_steps=20)
            dt += time.perf_counter() - t0
            faces += sim.active_faces - f0
            n += 1
            if dt >= budget_s:
                break
        return {"value": faces / dt, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"first {n} simulations of the batch ({label}), 20 steps each after the first, one after "
                          f"another ({faces} face updates, {dt:.1f} s); C restatement of the reference, OpenMP"}
    sim = O.OracleSim(problem, n_threads=threads)
    sim.step()  # the dt = 0 first step
    sim.step()
    f0 = sim.active_faces
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        sim.step()
        n += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    faces = sim.active_faces - f0
    return {"value": faces / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} OptimalOrder steps of the same workload ({label}; {faces} face updates, "
                      f"{dt:.1f} s wall) after 2 warm-up steps; C restatement of the reference, OpenMP, "
                      f"{threads} thread(s)"}


class _Clocks:
    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self, dev: int = 0):
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or parts[0] != str(dev):
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _time_steps(sim, steps, stream, flush_buf, torch):
    """Times `steps` device-resident steps with one event pair each and an L2
    flush before each.  Everything is enqueued first and synchronised once, so
    the GPU runs flush, step, flush, step, ... without host gaps; only the
    event-bracketed step times are summed."""
    sim.set_time()
    sim.flush_deferred()  # work deferred by earlier steps is not timed ...
    evs = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush_buf.zero_()  # on the simulation's stream, so it is ordered with the steps
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.enqueue_steps(1)
        e1.record(stream)
        evs.append((e0, e1))
    # ... and the work the timed steps deferred is (hierarchical steps extrapolate
    # inactive cells when a step reads them: what is still pending runs here)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.flush_deferred()
    e1.record(stream)
    evs.append((e0, e1))
    torch.cuda.synchronize()
    total = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    sim.sync_time()
    return total


# Compulsory HBM bytes of the face stage per launch.
#   plain FP64 (k_face_flux): per active face its indices, area, normal, centroid
#   and shift (88 B) and the 7 FP64 result rows (56 B); per cell next to an
#   active face its 44 FP64 face-stage inputs and the active flag (353 B).
#   FP32-face form: the face kernel reads per cell the 37 FP32 copies, dt and
#   the flag (157 B) and per active face the indices, the 26-float static
#   geometry and writes 7 FP32 result rows (140 B).  Steps over all cells write
#   the FP32 copies in the predict kernel (k_predict32); hierarchical steps run
#   k_prep32 in the face stage, which reads 40 FP64 rows and writes 37 FP32 rows
#   per cell next to an active face (468 B).
def face_stage_bytes(prec, nc, nfa, all_cells):
    touched = min(nc, 2 * nfa)
    if prec == 1:
        return (0 if all_cells else touched * 468) + touched * 157 + nfa * 140
    return touched * 353 + nfa * 144


# Compulsory HBM bytes of a whole step, each datum once: 88 B per active face
# (indices, area, normal, centroid, shift) and per active cell 800 B in the
# plain form (the flux-stage state read 328, extrapolation write 40, flux
# accumulator and conserved read+write 160, signal-speed rows 16, c2p 48,
# gradient write 144, timestep writes 64); the FP32-face form's face stage
# reads FP32 copies (164 B instead of 328): 636 B.
STEP_BYTES_FACE = 88
STEP_BYTES_CELL = {0: 800, 1: 636}

# FP64 flop per face of the plain face stage (k_face_flux + k_face_search +
# k_face_finish; 2 DFMA + DMUL + DADD over active threads) from an ncu capture
# at the bench size: profiles/face_stage_fp64_exact_pipes_kh256.txt.
FP64_FLOP_PER_FACE = {("kh2d", 256): 1522}


def face_stage_kernels(prec, all_cells, riemann=None):
    if prec == 0:
        return "k_face_flux + k_face_search + k_face_finish" if riemann == 1 else "k_face_flux"
    return "k_face_flux32" if all_cells else "k_prep32 + k_face_flux32"


def _fp64_peak(torch):
    """FP64 throughput of this GPU measured with cuBLAS DGEMM (TFLOP/s)."""
    try:
        n = 4096
        a = torch.randn(n, n, dtype=torch.float64, device="cuda")
        b = torch.randn(n, n, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        best = None
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    except Exception:
        return None


# DRAM bytes (read + write) per launch of the face stage from ncu captures at
# the bench sizes (cold caches, ncu's default cache control): the committed
# summaries in profiles/ give the commands.  Keyed by (workload, nx, form).
# FP32 form: profiles/face_stage_traffic_kh256.txt (k_face_flux32); plain form:
# profiles/face_stage_fp64_exact_pipes_kh256.txt (k_face_flux + k_face_search +
# k_face_finish: 42.3 + 61.0 + 47.3 MB, the job queue written once and read twice,
# the search pool's register spills).
TRAFFIC = {("kh2d", 256, 1): 26_891_008, ("kh2d", 256, 0): 150_600_000}


def _face_kernel_ms(sim, steps):
    sim.profile(True)
    sim.set_time()
    sim.enqueue_steps(steps)
    prof = sim.profile_read()
    sim.profile(False)
    sim.sync_time()
    return prof


def run_ours(args):
    import torch

    from hydro_rs_gb300 import gpu as G
    from hydro_rs_gb300.layout import CELL_ROWS, Cells

    ws, rank = _dist()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from hydro_rs_gb300 import ics

    problem, mesh_s = _problem(args.nx, args.workload, args.riemann, args.runner)
    problem.params.limiter_frame = args.limiter_frame
    nf, nc = problem.mesh.n_faces, problem.mesh.n_cells
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    sims = {}
    batch = problem.extra.get("cell_offsets") is not None
    hier = not batch and not problem.params.sync_all  # hierarchical steps of one simulation
    tuned = {}
    ctx_s = {}
    for prec in (1, 0):
        t_ctx = time.perf_counter()
        with torch.cuda.stream(stream):
            if batch:
                sims[prec] = G.GpuSim(problem, precision=prec, stream=stream.cuda_stream,
                                      cell_offsets=problem.extra["cell_offsets"], t_end=problem.extra["t_end"])
            else:
                sims[prec] = G.GpuSim(problem, precision=prec, stream=stream.cuda_stream)
        torch.cuda.synchronize()
        # mvmm_ctx_create (device allocation + mesh upload) and the first mvmm_upload_cells
        ctx_s[prec] = time.perf_counter() - t_ctx
        # thread-block sizes picked by the library's autotuner on this workload (untimed; state restored)
        tuned[prec] = sims[prec].autotune(3)
    # advance both forms identically past the dt=0 first step + warm-up
    res = {}
    for prec, sim in sims.items():
        try:
            sim.run(max_steps=2 + args.warmup)
        except G.MvmmError as e:  # a batch reports failed simulations and runs on
            if not batch or e.code != -3:
                raise
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    with _Clocks() as clk:
        for prec, sim in sims.items():
            barrier()
            f0 = sim.sync_time()[1]
            ms = _time_steps(sim, args.steps, stream, flush, torch)
            barrier()
            faces = sim.sync_time()[1] - f0
            res[prec] = (ms, faces)
    clocks = clk.summary(dev)

    # L1 density error of the FP32 form against the plain FP64 form at the same
    # simulated time.  Where one form's global time bin crossed a power of two on
    # the other side, the two integer timelines part; after the timed region the
    # one behind is stepped to the next point both timelines share.
    aligned = 0
    if not batch:
        while sims[1].ti_current != sims[0].ti_current and aligned < 256 and \
                not (sims[0].finished or sims[1].finished):
            (sims[1] if sims[1].ti_current < sims[0].ti_current else sims[0]).step()
            aligned += 1
    a, b = sims[1].state(), sims[0].state()
    l1 = float(np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum())
    same_time = sims[1].ti_current == sims[0].ti_current

    # per-kernel times (events around each kernel) for the roofline
    prof, nfa, nca = {}, {}, {}
    for prec, sim in sims.items():
        k_prof = min(args.steps, 20)
        st0 = sim.stats()
        prof[prec] = _face_kernel_ms(sim, k_prof)
        st1 = sim.stats()
        nfa[prec] = (st1["active_faces"] - st0["active_faces"]) / k_prof  # active faces per profiled step
        nca[prec] = (st1["active_cells"] - st0["active_cells"]) / k_prof  # active cells per profiled step

    # end-to-end through the C ABI with pinned host buffers: one pinned block in
    # the device's field order, stepped in place; both forms
    def e2e_measure(sim, changed=False):
        pinned = (torch.empty(CELL_ROWS * nc, dtype=torch.float64, pin_memory=True),
                  torch.empty(nc, dtype=torch.int8, pin_memory=True))
        cells = Cells.packed(nc, pinned[0].numpy(), pinned[1].numpy())
        sim.state(cells)
        first = [True]

        def e2e_step():
            if changed:
                # the host block stays the state; the first call uploads it whole,
                # the others list no host-side change and store what the step rewrote
                sim.step_cells_changed(cells, None if first[0] else [])
                first[0] = False
            elif batch:
                sim.upload(cells)
                try:
                    sim.step()
                except G.MvmmError as e:
                    if e.code != -3:
                        raise
                sim.state(cells)
            else:
                sim.step_cells(cells)  # upload + step + download in one C call

        # warm-up: the first call creates the copy stream and the snapshot block, and
        # the first few run slower while the host block's pages settle
        for _ in range(3 if batch else 10):
            e2e_step()
        n_steps = 10 if batch else 50  # a fixed sample (a batch moves ~1 GB per call), whatever --steps is
        st0 = sim.stats()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        f0 = sim.active_faces
        for _ in range(n_steps):
            e2e_step()
        secs = time.perf_counter() - t0
        barrier()
        st1 = sim.stats()
        # bytes the library moved between the host block and the device (counted by it)
        return {"seconds": secs, "faces": sim.active_faces - f0, "steps": n_steps,
                "h2d": (st1["host_bytes_in"] - st0["host_bytes_in"]) / n_steps,
                "d2h": (st1["host_bytes_out"] - st0["host_bytes_out"]) / n_steps, "bytes_cells": cells.nbytes()}

    e2e = {prec: e2e_measure(sims[prec]) for prec in (0, 1)}
    # hierarchical steps of one simulation: also through mvmm_step_cells_changed
    e2e_chg = {prec: e2e_measure(sims[prec], changed=True) for prec in (0, 1)} \
        if not batch and not problem.params.sync_all else {}

    st32 = sims[1].stats()
    fallback32 = {"faces": st32["fp64_fallback_faces"], "of_active_faces": st32["active_faces"]}
    ms32, faces32 = res[1]
    ms64, faces64 = res[0]
    batch_info = None
    if batch:
        st = sims[1].batch_state()
        st64 = sims[0].batch_state()
        # instances stopped by a numerical failure (the reference panics there), after
        # each form's own number of steps in this process
        batch_info = {"instances": int(len(st["err"])), "flagged_instances": int((st["err"] != 0).sum()),
                      "flagged_instances_fp64": int((st64["err"] != 0).sum()),
                      "steps": {"fp32_face": int(st["steps"].max()), "fp64": int(st64["steps"].max())},
                      "finished_instances": int(st["finished"].sum()),
                      "autotuned_blocks": {"fp32_face": tuned.get(1), "fp64": tuned.get(0)},
                      "graph": "each batched step is one CUDA graph launch over all unfinished simulations"}
    # max over ranks of the timed region; faces summed
    if ws > 1:
        import torch.distributed as dist

        def red(op):
            def f(vals):
                t = torch.tensor(vals, device="cuda", dtype=torch.float64)
                dist.all_reduce(t, op=op)
                return t.tolist()
            return f

        (ms32, ms64, e2e[0]["seconds"], e2e[1]["seconds"]), (faces32, faces64, e2e[0]["faces"], e2e[1]["faces"]) = \
            aggregate_replicas([ms32, ms64, e2e[0]["seconds"], e2e[1]["seconds"]],
                               [faces32, faces64, e2e[0]["faces"], e2e[1]["faces"]],
                               red(dist.ReduceOp.MAX), red(dist.ReduceOp.SUM))
        for e in e2e_chg.values():
            (e["seconds"],), (e["faces"],) = aggregate_replicas([e["seconds"]], [e["faces"]],
                                                                red(dist.ReduceOp.MAX), red(dist.ReduceOp.SUM))
    if rank != 0:
        return
    peak, peak_kind = _peaks()
    all_cells = batch or problem.params.sync_all

    def kernel_ms(prec):
        # per-launch milliseconds of each step kernel from event nodes placed
        # around it in the step graph, less the interval of an empty event pair
        # (the "end" slot, which holds no kernel: the step's bookkeeping runs in
        # the limiter's last block)
        pr = prof[prec]
        ev_ms = pr["end"][0] / max(pr["end"][1], 1)
        out = {k: max(v[0] / max(v[1], 1) - ev_ms, 0.0) for k, v in pr.items() if k != "end"}
        return out, ev_ms

    def roof(prec):
        kms, ev_ms = kernel_ms(prec)
        ms_launch = kms["face_flux"]
        bytes_launch = face_stage_bytes(prec, nc, nfa[prec], all_cells)
        ach = bytes_launch / (ms_launch * 1e-3) / 1e9
        traffic = TRAFFIC.get((args.workload, args.nx, prec))
        return {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "traffic": traffic,
                "kernel": face_stage_kernels(prec, all_cells, problem.params.riemann),
                "kernel_ms": round(ms_launch, 4), "algorithmic_bytes_per_launch": int(bytes_launch),
                "active_faces_per_launch": nfa[prec],
                "peak_kind": peak_kind, "note": "of measured" if peak_kind == "measured" else "of fallback",
                "kernel_ms_source": "CUDA events recorded as graph nodes around each stage of the step graph on "
                                    "the context stream, minus the interval of an empty event pair "
                                    f"({ev_ms:.4f} ms)",
                "step_kernel_ms": {k: round(v, 4) for k, v in kms.items()}}

    fp64_peak = _fp64_peak(torch)

    def fp64_roof():
        # the plain face stage against the FP64 pipe: flop per face (measured once
        # by ncu at this size) x active faces / the stage's event time, against the
        # FP64 throughput measured here (cuBLAS DGEMM)
        fpf = FP64_FLOP_PER_FACE.get((args.workload, args.nx))
        if fpf is None or fp64_peak is None:
            return None
        ms = kernel_ms(0)[0]["face_flux"]
        ach = fpf * nfa[0] / (ms * 1e-3) / 1e12
        return {"bound": "fp64", "achieved": round(ach, 4), "peak": round(fp64_peak, 3), "unit": "TFLOP/s",
                "frac": round(ach / fp64_peak, 4), "flop_per_face": fpf, "kernel": face_stage_kernels(0, all_cells,
                                                                                                problem.params.riemann),
                "peak_kind": "measured here: torch.matmul float64 4096^3 (cuBLAS DGEMM), best of 5",
                "note": "flop per face from one ncu capture of the face stage (profiles/)"}

    def step_roof(prec, ms_step):
        b = STEP_BYTES_FACE * nfa[prec] + STEP_BYTES_CELL[prec] * nca[prec]
        ach = b / (ms_step * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4),
                "bytes_per_step": int(b), "active_faces_per_step": nfa[prec], "active_cells_per_step": nca[prec],
                "bytes_per_face": STEP_BYTES_FACE, "bytes_per_cell": STEP_BYTES_CELL[prec],
                "note": "whole step (all kernels) over ms_per_step; " +
                        ("of measured" if peak_kind == "measured" else "of fallback")}

    def e2e_line(prec):
        e = e2e[prec]
        return {"value": e["faces"] / e["seconds"], "unit": UNIT, "h2d_bytes_per_step": int(e["h2d"]),
                "d2h_bytes_per_step": int(e["d2h"]), "host_block_bytes": e["bytes_cells"], "steps": e["steps"],
                "how": ("mvmm_upload_cells + mvmm_step + mvmm_download_cells per step" if batch else
                        "mvmm_step_cells per step (upload, step and download in one C call; the step's "
                        "state comes back in place, only the 8 KB chunks it changed)") +
                       ", one pinned host block in the device field order, wall clock, bytes as counted "
                       "by the library",
                **({"changed_cells": e2e_changed_line(prec)} if prec in e2e_chg else {})}

    def e2e_changed_line(prec):
        e = e2e_chg[prec]
        return {"value": e["faces"] / e["seconds"], "unit": UNIT, "h2d_bytes_per_step": int(e["h2d"]),
                "d2h_bytes_per_step": int(e["d2h"]), "steps": e["steps"],
                "how": "mvmm_step_cells_changed per step on the same pinned block: the block stays the state, "
                       "no host-side change is listed, and the cells the step rewrote (32 at a time) are "
                       "written back in place"}

    cpu = _cpu_sample(problem, _workload_name(args)) if (ws == 1 and not args.no_cpu) else None
    value64 = faces64 / (ms64 * 1e-3)
    value32 = faces32 / (ms32 * 1e-3)
    exact = problem.params.riemann == ics.EXACT
    line = {
        "metric": METRIC, "value": value64, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms64 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": DATA.get(args.workload, "synthetic, seeded"),
        "config": {"workload": _workload_name(args),
                   "cells": nc, "faces": nf, "precision": PRECISION_FP64,
                   "l2": "flushed (256 MB write) before each timed step", "parallelism": f"replicas x{ws}",
                   "mesh_build_s": round(mesh_s, 3),
                   **({"limiter_frame": "flux_exchange's (not the reference's)"} if args.limiter_frame else {}),
                   "ctx_create_and_upload_s": {"fp64": round(ctx_s[0], 4), "fp32_face": round(ctx_s[1], 4)},
                   "blocks_face_cell": {"fp64": tuned.get(0), "fp32_face": tuned.get(1)}},
        "active_face_fraction": faces64 / (args.steps * nf * ws),
        "batch": batch_info,
        "roofline": roof(0),
        "fp64_roofline": fp64_roof(),
        "step_roofline": step_roof(0, ms64 / args.steps),
        "e2e": e2e_line(0),
        "fp32_face": {"value": value32, "unit": UNIT, "ms_per_step": ms32 / args.steps,
                      "dtype": "f32-face/f64-accumulate", "speedup_vs_fp64": value32 / value64,
                      "e2e": e2e_line(1),
                      "l1_density_err_vs_fp64": l1, "l1_same_time": same_time, "l1_alignment_steps": aligned,
                      "fp64_fallback_faces": fallback32,
                      "roofline": roof(1), "step_roofline": step_roof(1, ms32 / args.steps)},
        "cpu_baseline": cpu,
        # per step, both forms timed: over all cells k_predict / k_predict32, face, update, gradients,
        # limiter (5 + 5); the plain form's exact solver adds k_face_search and k_face_finish;
        # hierarchical steps add k_compact to both and k_prep32 to the FP32 form, and each form's
        # timed region ends with one k_extrap_flush
        "gpu_launches": args.steps * ((5 + 5) + (2 if exact else 0) + (3 if hier else 0)) + (2 if hier else 0),
        "clocks": clocks,
    }
    print(json.dumps(line))


def run_serve(args):
    """Config 5: continuous batching of a Poisson request stream (rank 0 only)."""
    import torch

    from hydro_rs_gb300 import serve

    ws, rank = _dist()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if rank != 0:
        return
    reqs = serve.poisson_requests(args.nx, rate=50.0, seed=5)
    srv = serve.Server(budget_bytes=32 << 30, chunk=16, precision=1)
    t0 = time.perf_counter()
    for nx in sorted({r.nx for r in reqs}):
        srv.template(nx)  # host meshes, built once per resolution
    mesh_s = time.perf_counter() - t0
    warm = serve.poisson_requests(5, rate=1e6, seed=6, resolutions=sorted({r.nx for r in reqs}))
    srv.run(warm, realtime=False)  # slots created, graphs captured
    with _Clocks() as clk:
        res, wall = srv.run(reqs, realtime=True)
    clocks = clk.summary(0)
    summ = serve.latency_summary(res, wall)
    accuracy = _serve_accuracy(srv, reqs, check_oracle=not args.no_cpu)
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        done, t_cpu, faces = 0, 0.0, 0
        for r in sorted(reqs, key=lambda r: r.nx)[:8]:
            sim = O.OracleSim(srv.problem_for(r), n_threads=threads)
            t1 = time.perf_counter()
            sim.run()
            t_cpu += time.perf_counter() - t1
            faces += sim.active_faces
            done += 1
            if t_cpu > 20.0:
                break
        rate = faces / t_cpu
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "solves_per_s_estimate": summ["requests"] / (summ["active_faces"] / rate),
               "sample": f"the {done} smallest requests of the stream run one after another to t_end on the oracle "
                         f"({t_cpu:.1f} s, {faces} face updates); solves/s estimated as the stream's total face "
                         f"updates at that CPU rate"}
    line = {
        "metric": METRIC, "value": summ["active_faces"] / wall, "unit": UNIT, "n_gpus": 1, "steps": None,
        "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-face/f64-accumulate", "data": "synthetic (seeded Poisson request stream, isentropic vortices)",
        "config": {"workload": WORKLOADS["serve2d"].format(n=args.nx), "hbm_budget_bytes": srv.budget,
                   "chunk_steps": srv.chunk, "mesh_build_s": round(mesh_s, 2)},
        "serving": {k: v for k, v in summ.items()} | {"peak_concurrent": srv.peak_running,
                                                       "slots": len(srv.slots), "slot_bytes": srv.used},
        "accuracy": accuracy, "cpu_baseline": cpu, "clocks": clocks,
    }
    srv.close()
    print(json.dumps(line))


def _serve_accuracy(srv, reqs, check_oracle: bool, n_check: int = 3):
    """L1 density errors of served requests (untimed): the smallest requests solved
    alone with the server's form (served results are bit-identical to those,
    tests/test_gpu_serve.py), against the analytic solution (the initial vortex
    carried by the advection velocity through the periodic box) and against the
    oracle."""
    import numpy as np

    from hydro_rs_gb300 import gpu as G
    from hydro_rs_gb300 import ics

    out = []
    for r in sorted(reqs, key=lambda r: (r.nx, r.rid))[:n_check]:
        q = srv.problem_for(r)
        sim = G.GpuSim(q, precision=srv.precision)
        sim.run()
        st = sim.state()
        sim.close()
        box = 10.0
        x = np.array(st.loc, dtype=np.float64)  # the initial state samples the vortex at the generators
        x[:2] = np.mod(x[:2] - np.asarray(r.v_adv, dtype=np.float64)[:2, None] * r.t_end, box)
        exact = ics.yee_cells(q.mesh, x, r.beta, r.v_adv).prim[0]
        row = {"rid": r.rid, "nx": r.nx, "beta": round(r.beta, 3),
               "l1_vs_analytic": float(np.abs(st.prim[0] - exact).sum() / np.abs(exact).sum())}
        if check_oracle:
            from oracle import oracle as O

            o = O.OracleSim(q, n_threads=os.cpu_count() or 1)
            o.run()
            ref = o.state().prim[0]
            row["l1_vs_oracle"] = float(np.abs(st.prim[0] - ref).sum() / np.abs(ref).sum())
        out.append(row)
    return out


def run_batch_to_end(args):
    """The batched configuration as named: every simulation of the batch run to
    its t_end = 0.15, both forms from the same initial state, the whole run
    timed (mvmm_run: one CUDA graph launch per batched step until every
    simulation has finished or been stopped by a numerical failure).  The
    forms are compared per simulation at t_end, the same simulated time.

    A few simulations of the batch take millions of steps of their own (their
    time bins fall as far as the timeline allows), so each form runs from the
    same state until every simulation has finished or --budget-s of wall time
    has passed (0: no limit); its rate is that window's.  The forms are
    compared on the simulations both have finished (the same simulated time,
    t_end), and the ones still running are listed with their steps and the
    simulated time they reached."""
    import torch

    from hydro_rs_gb300 import gpu as G
    from hydro_rs_gb300 import ics

    ws, rank = _dist()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    problem, mesh_s = _problem(args.nx, args.workload, args.riemann, args.runner)
    problem.params.limiter_frame = args.limiter_frame
    off, te = problem.extra["cell_offsets"], problem.extra["t_end"]
    res = {}
    with _Clocks() as clk:
        for prec in (1, 0):
            sim = G.GpuSim(problem, precision=prec, cell_offsets=off, t_end=te)
            tuned = sim.autotune(3)  # block sizes on the live state, which it restores
            f0 = sim.stats()["active_faces"]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            budget = args.budget_s
            while not sim.finished:  # chunks of steps, with progress on stderr
                if budget > 0 and time.perf_counter() - t0 >= budget:
                    break
                try:
                    sim.run(max_steps=4096)
                except G.MvmmError as e:  # a stopped simulation is reported per instance; the others run on
                    if e.code != -3:
                        raise
                st = sim.batch_state()
                sim.finished = bool(st["finished"].all())
                print(f"[to-end] form {prec}: {int(st['finished'].sum())} of {len(st['finished'])} finished, "
                      f"{int(st['steps'].max())} steps, {time.perf_counter() - t0:.1f} s", file=sys.stderr,
                      flush=True)
            torch.cuda.synchronize()
            secs = time.perf_counter() - t0
            st = sim.batch_state()
            res[prec] = {"seconds": secs, "faces": sim.stats()["active_faces"] - f0, "state": st,
                         "cells": ics.unpack_cells(sim.state(), off), "blocks": tuned}
            sim.close()
    clocks = clk.summary(0)
    if rank != 0:
        return
    ok = (res[0]["state"]["err"] == 0) & (res[1]["state"]["err"] == 0) & (res[0]["state"]["finished"] != 0) & \
        (res[1]["state"]["finished"] != 0)
    l1 = []
    for k in np.nonzero(ok)[0]:
        a, b = res[1]["cells"][k].prim[0], res[0]["cells"][k].prim[0]
        l1.append(float(np.abs(a - b).sum() / np.abs(b).sum()))
    l1 = np.array(l1)

    def form(prec):
        r = res[prec]
        return {"value": r["faces"] / r["seconds"], "unit": UNIT, "seconds": round(r["seconds"], 3),
                "face_updates": int(r["faces"]), "max_steps": int(r["state"]["steps"].max()),
                "finished": int(r["state"]["finished"].sum()), "flagged": int((r["state"]["err"] != 0).sum()),
                "blocks_face_cell": r["blocks"]}

    line = {
        "metric": METRIC, "value": res[0]["faces"] / res[0]["seconds"], "unit": UNIT, "n_gpus": 1,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": DATA.get(args.workload, "synthetic, seeded"),
        "config": {"workload": _workload_name(args) + ", the whole run",
                   "cells": problem.mesh.n_cells, "faces": problem.mesh.n_faces, "precision": PRECISION_FP64,
                   "mesh_build_s": round(mesh_s, 3),
                   "timing": "wall clock around mvmm_run, each form until every simulation finished" +
                             (f" or {args.budget_s:g} s passed" if args.budget_s > 0 else "")},
        "fp64": form(0), "fp32_face": form(1),
        "fp32_face_speedup": (res[1]["faces"] / res[1]["seconds"]) / (res[0]["faces"] / res[0]["seconds"]),
        "l1_density_err_fp32_vs_fp64_at_t_end": {"instances": int(ok.sum()), "median": float(np.median(l1)),
                                                 "max": float(np.max(l1))} if l1.size else None,
        "running_at_end_fp32_face": [
            {"instance": int(k), "cells": int(off[k + 1] - off[k]), "steps": int(res[1]["state"]["steps"][k]),
             "t_reached": float(res[1]["state"]["ti_current"][k]) / float(1 << 57) * float(te[k])}
            for k in np.nonzero(res[1]["state"]["finished"] == 0)[0][:16]],
        "same_flagged_instances": bool(np.array_equal((res[0]["state"]["err"] != 0)[res[0]["state"]["finished"] != 0],
                                                      (res[1]["state"]["err"] != 0)[res[0]["state"]["finished"] != 0])),
        "clocks": clocks,
    }
    print(json.dumps(line))


def run_moving(args):
    """Moving mesh (drift, a host Voronoi build every step, re-upload): each
    step drifts the generators on the device, reads them back, rebuilds the
    Voronoi mesh on the host, uploads it and steps.  `value` is active-face
    updates per second of device step time (CUDA events on the context's
    stream); `e2e` divides by the wall time of the whole cycle, and `stages_s`
    gives each part as its own line."""
    import torch

    from hydro_rs_gb300 import gpu as G
    from hydro_rs_gb300 import ics
    from hydro_rs_gb300.moving import MovingMeshStepper

    ws, rank = _dist()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if rank != 0:
        return
    t0 = time.perf_counter()
    problem = ics.kelvin_helmholtz_2d(args.nx, seed=2, riemann=ics.EXACT, t_end=1.5)
    problem.params.particle_motion = ics.STEER
    mesh_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    stream = torch.cuda.Stream()
    res, stages, sims = {}, {}, {}
    with _Clocks() as clk:
        for prec in (1, 0):
            sim = G.GpuSim(problem, precision=prec, stream=stream.cuda_stream)
            st = MovingMeshStepper(sim, problem.mesh, n_threads=threads)
            for _ in range(args.warmup):
                st.step()
            st.seconds = {k: 0.0 for k in st.seconds}
            f0, dev_ms = sim.active_faces, 0.0
            t_wall = time.perf_counter()
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                # the step's own stream work (drift and mesh upload are their own lines)
                orig_step = sim.step

                def timed_step(sim=sim, orig=orig_step, e0=e0, e1=e1):
                    e0.record(stream)
                    done = orig()
                    e1.record(stream)
                    return done
                sim.step = timed_step
                st.step()
                sim.step = orig_step
                e1.synchronize()
                dev_ms += e0.elapsed_time(e1)
            wall = time.perf_counter() - t_wall
            faces = sim.active_faces - f0
            res[prec] = (faces, dev_ms, wall)
            stages[prec] = {k: round(v / args.steps * 1e3, 3) for k, v in st.seconds.items()}
            sims[prec] = sim
    a, b = sims[1].state(), sims[0].state()
    l1 = float(np.abs(a.prim[0] - b.prim[0]).sum() / np.abs(b.prim[0]).sum())
    same_time = sims[1].ti_current == sims[0].ti_current
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O

        osim = O.OracleSim(problem, n_threads=threads)
        ost = MovingMeshStepper(osim, problem.mesh, n_threads=threads)
        ost.step()
        f0, t1, n = osim.active_faces, time.perf_counter(), 0
        while time.perf_counter() - t1 < 10.0 and n < 100:
            ost.step()
            n += 1
        t_cpu = time.perf_counter() - t1
        cpu = {"value": (osim.active_faces - f0) / t_cpu, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} moving-mesh steps of the same workload on the oracle, each with the host Voronoi "
                         f"rebuild ({t_cpu:.1f} s wall, whole cycle)"}
    faces32, ms32, wall32 = res[1]
    faces64, ms64, wall64 = res[0]
    m = sims[1].mesh  # mvmm_set_mesh uploads the faces, the CSR and the new volumes and centroids
    mesh_bytes = int(m.n_faces * 88 + (m.n_cells + 1) * 4 + m.csr_face.size * 4 + m.n_cells * 32)
    line = {
        "metric": METRIC, "value": faces32 / (ms32 * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-face/f64-accumulate",
        "data": "synthetic (seeded jittered lattice, shear-layer ICs)",
        "config": {"workload": WORKLOADS["kh2d_moving"].format(n=args.nx), "cells": problem.mesh.n_cells,
                   "faces_initial": problem.mesh.n_faces, "precision": "fp32_face",
                   "l2": "not flushed: the mesh upload before each step rewrites the face arrays",
                   "parallelism": "replicas x1", "mesh_build_s": round(mesh_s, 3)},
        "l1_density_err_vs_fp64": l1, "l1_same_time": same_time,
        "stages_ms_per_step": {"fp32_face": stages[1], "fp64": stages[0]},
        "plain_fp64": {"value": faces64 / (ms64 * 1e-3), "unit": UNIT, "ms_per_step": ms64 / args.steps},
        "e2e": {"value": faces32 / wall32, "unit": UNIT,
                "h2d_bytes_per_step": mesh_bytes, "d2h_bytes_per_step": problem.mesh.n_cells * 24,
                "how": "whole moving-mesh cycle per step, wall clock: mvmm_drift, mvmm_get_positions, host Voronoi "
                       "build, mvmm_set_mesh, mvmm_step"},
        "cpu_baseline": cpu, "clocks": clk.summary(0),
    }
    print(json.dumps(line))


# FP64 operations per pair of k_self_gravity's sum: 3 subtractions, 3 products
# and 2 sums for |d|^2, the square root, + softening, r r r (2), m d (3), the 3
# divisions and the 3 accumulations (square root and division counted as one).
SELF_GRAVITY_FLOP_PER_PAIR = 21


def run_self_gravity(args):
    """Self-gravity kicks: SelfGravity::compute_accelerations (gravity.rs:22-43)
    at the runner's "TODO: gravity" point of every step, then kick2 / kick1.
    `value` is active-face updates per second of device step time (plain FP64
    form); `self_gravity` gives the update stage (k_update + k_self_gravity,
    from event nodes in the step graph) as pairs per second and against the
    FP64 throughput measured here."""
    import torch

    from hydro_rs_gb300 import gpu as G
    from hydro_rs_gb300 import ics

    ws, rank = _dist()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if rank != 0:
        return
    problem, _ = _problem(args.nx, "kh2d_selfgrav")
    n = problem.mesh.n_cells
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    sim = G.GpuSim(problem, stream=stream.cuda_stream)
    with _Clocks() as clk:
        for _ in range(args.warmup):
            sim.step()
        f0 = sim.sync_time()[1]
        ms = _time_steps(sim, args.steps, stream, flush, torch)
        faces = sim.sync_time()[1] - f0
        prof = _face_kernel_ms(sim, 3)
    ev_ms = prof["end"][0] / max(prof["end"][1], 1)
    upd_ms = max(prof["update"][0] / max(prof["update"][1], 1) - ev_ms, 0.0)
    pairs = n * (n - 1) // 2
    fp64_peak = _fp64_peak(torch)
    ach = SELF_GRAVITY_FLOP_PER_PAIR * pairs / (upd_ms * 1e-3) / 1e12
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        osim = O.OracleSim(problem, n_threads=threads)
        osim.step()
        f1, t1, k = osim.active_faces, time.perf_counter(), 0
        while time.perf_counter() - t1 < 15.0 and k < 50:
            osim.step()
            k += 1
        t_cpu = time.perf_counter() - t1
        cpu = {"value": (osim.active_faces - f1) / t_cpu, "unit": UNIT, "cores": threads, "kind": "port",
               "pairs_per_s": pairs * k / t_cpu,
               "sample": f"{k} steps of the same workload on the oracle ({t_cpu:.1f} s)"}
    line = {
        "metric": METRIC, "value": faces / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice, shear-layer ICs)",
        "config": {"workload": WORKLOADS["kh2d_selfgrav"].format(n=args.nx), "cells": n,
                   "faces": problem.mesh.n_faces, "precision": PRECISION_FP64,
                   "l2": "flushed before each step", "parallelism": "replicas x1"},
        "self_gravity": {"kernel": "k_update + k_self_gravity", "stage_ms": round(upd_ms, 4),
                         "pairs_per_launch": pairs, "pairs_per_s": pairs / (upd_ms * 1e-3),
                         "roofline": None if fp64_peak is None else {
                             "bound": "fp64", "achieved": round(ach, 4), "peak": round(fp64_peak, 3),
                             "unit": "TFLOP/s", "frac": round(ach / fp64_peak, 4),
                             "flop_per_pair": SELF_GRAVITY_FLOP_PER_PAIR,
                             "peak_kind": "measured here: torch.matmul float64 4096^3 (cuBLAS DGEMM), best of 5"}},
        # predict, face flux, update, self-gravity, gradients, limiter
        "gpu_launches": args.steps * 6,
        "cpu_baseline": cpu, "clocks": clk.summary(0),
    }
    print(json.dumps(line))


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return
    problem, _ = _problem(args.nx, args.workload, args.riemann, args.runner)
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    sim = O.OracleSim(problem, n_threads=threads)
    for _ in range(2 + args.warmup):
        sim.step()
    f0 = sim.active_faces
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.step()
    dt = time.perf_counter() - t0
    faces = sim.active_faces - f0
    v = faces / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice, shear-layer ICs)",
        "config": {"workload": _workload_name(args), "cells": problem.mesh.n_cells,
                   "faces": problem.mesh.n_faces, "precision": PRECISION_FP64},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steps after {2 + args.warmup} warm-up steps; the Rust reference "
                                   "cannot be built here (no cargo/rustc), the C restatement runs instead"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="kh2d", choices=sorted(WORKLOADS),
                    help="kh2d (the headline), sod1d, blast3d (extra measurements)")
    ap.add_argument("--nx", type=int, default=None, help="lattice side / cell count (default per workload)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg (profiling runs)")
    ap.add_argument("--riemann", default="TSRS", choices=["HLLC", "Exact", "PVRS", "AIRS", "TSRS", "TRRS",
                                                           "LinearAdvection"],
                    help="kh2d_solver: the Riemann solver (bin/main.rs names)")
    ap.add_argument("--runner", default="OptimalOrder", choices=["OptimalOrder", "Godunov"],
                    help="kh2d_solver: the runner")
    ap.add_argument("--limiter-frame", type=int, default=0, choices=[0, 1],
                    help="1: the cell-wise limiter's face offsets in flux_exchange's frame (not the reference's)")
    ap.add_argument("--to-end", action="store_true",
                    help="batch workloads: time the whole run, every simulation to its t_end")
    ap.add_argument("--budget-s", type=float, default=300.,
                    help="--to-end: wall seconds the plain form runs for (0: to the end)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.nx is None:
        args.nx = DEFAULT_N[args.workload]
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serve2d":
        run_serve(args)
    elif args.workload == "kh2d_moving":
        run_moving(args)
    elif args.workload == "kh2d_selfgrav":
        run_self_gravity(args)
    elif args.to_end and args.workload in ("batch1d", "batch1d_pvrs"):
        run_batch_to_end(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
