#!/usr/bin/env python
"""Load steps/s of the LPM quasi-static Newton load step on one GB300.

Workload: the 3-D simple-cubic lattice of 101^3 = 1,030,301 particles
(18,240,600 directed bonds, 60,969,107 3x3 tangent blocks), lattice
constant 0.2 mm, E = 200 GPa, nu = 0.3, bottom face clamped, top face pulled
in z by 0.002 mm per load step.  A load step = apply the step's boundary
conditions, assemble the tangent (symmetric variant, BC elimination), and
Newton iterations (tol 1e-5) each with a Jacobi-CG solve to 1e-10.

Reported (one JSON line on rank 0):
  value        load steps/s of the mixed form (FP32 CG in FP64 refinement),
               device-timed with CUDA events on the library's stream
  fp64         the same with the plain FP64 CG
  e2e          steps driven through the C ABI with host buffers: each step
               passes its BC descriptors from pinned host memory and reads
               positions and internal forces back into pinned host memory
  roofline     the CG sparse product (dominant kernel): algorithmic bytes
               per launch / average launch time, against the measured HBM
               copy bandwidth
  cpu_baseline the CPU oracle (a restatement of the reference algorithm) on
               the host cores: one complete FP64 load step, timed whole
  parity       that CPU step against the GPU's first FP64 step and the
               GPU's first mixed step against its FP64 one (displacement and
               reaction errors)
  adjoint      one backward step (gradient of a reaction with respect to
               every bond's constants), in ms and relative to a forward step
  bonds_per_s  the force pass alone and with the tangent assembly
  setup        the GPU bond search (checked identical to the CPU
               generator's bonds) and the creation of the device lattice
  fatigue      compact-tension fatigue cycles at full size (configuration 5)
  fatigue_coarse  the same cycles with the coarse-space preconditioner
  fatigue_sensitivity  those cycles carrying the damage's tangents along the
               HCF A and B, relative to fatigue_coarse
  softening    load steps of the notched plate with the softening bond law
               and damage rounds at full size (configuration 3): by default
               the one step in which the first bonds soften (about 170
               damage rounds); --softening-steps 4 times the crack's burst
               too (minutes)
  softening_coarse  the same steps with the coarse-space preconditioner
               (Jacobi plus rigid-body modes of boxes of particles)
  softening_sensitivity  the coarse-preconditioned steps carrying the
               reaction's tangents along E and the Weibull scale through every
               damage round, relative to softening_coarse
  j2_sensitivity  cost of carrying d/d(yield stress) and d/d(hardening)
               through J2 load steps of a BCC polycrystal (40^3 cells)
  polycrystal  configuration 4 at full size (BCC 60^3 cells, 20 grains):
               bounded loading and unloading steps past yield, without and
               with the two tangent directions
  matrix_free  the mixed load step with the tangent applied from bond data

--impl reference times complete CPU oracle load steps of the same workload.
Multi-GPU runs are independent replicas (the path has no exchange step).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "load steps/s, 1M-particle SC lattice (quasi-static Newton load step)"
UNIT = "load steps/s"


def parse_args(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=101, help="particles per cube edge")
    p.add_argument("--du", type=float, default=0.002, help="top-face displacement per step (mm)")
    p.add_argument("--cg-tol", type=float, default=1e-10)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-matrix-free", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="time the load steps only (no e2e, adjoint, force/assembly, set-up, fatigue, J2 legs): "
                        "for profiling runs")
    p.add_argument("--profile-solve", choices=["sent", "ct", "sent-coarse", "ct-coarse"],
                   help="profiling entry: one mixed solve (300 iterations) on the full-size SENT or CT plate's "
                        "tangent, which runs as one persistent kernel (with the coarse-space preconditioner for "
                        "the -coarse cases); prints its time and exits")
    p.add_argument("--softening-steps", type=int, default=1,
                   help="timed load steps of configuration 3 at full size from the first softened bond on (0: none; "
                        "4 includes the crack's burst, several minutes)")
    return p.parse_args(argv)


# ------------------------------------------------------------------ set-up
def workload(n, a=0.2, E=200e3, nu=0.3):
    import __graft_entry__ as ge
    lat = ge.load_package().lattice
    cell = lat.UnitCell(lat.SIMPLECUBIC3D, a / 2)
    xyz = lat.sc_cuboid(n, n, n, a)
    t0 = time.perf_counter()
    p1, p2, layer = lat.find_bonds(xyz, cell)
    t_bonds = time.perf_counter() - t0
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(E, nu, layout="row"))
    z = xyz[:, 2]
    bottom = np.where(z < z.min() + 1e-9)[0]
    top = np.where(z > z.max() - 1e-9)[0]
    return dict(cell=cell, xyz=xyz, p1=p1, p2=p2, layer=layer, Kn=Kn, Tv=Tv, bottom=bottom, top=top,
                find_bonds_s=t_bonds)


def describe(w):
    return "SC %d^3 lattice (%d particles, %d bonds), a=0.2 mm, E=200 GPa, nu=0.3, clamped base, top +%g mm/step" % (
        round(len(w["xyz"]) ** (1 / 3)), len(w["xyz"]), len(w["p1"]), ARGS.du)


T_START = time.perf_counter()


def run_leg(line, key, fn, *a, **k):
    """One optional bench leg: its result under `key`, or the error it
    raised (an extra leg never takes the headline line down with it)."""
    progress(key)
    try:
        line[key] = fn(*a, **k)
    except Exception as e:  # noqa: BLE001 - reported in the line
        line[key] = {"error": "%s: %s" % (type(e).__name__, e)}


def progress(what):
    """One line on stderr per bench leg, with the elapsed time."""
    sys.stderr.write("[bench %7.1f s] %s\n" % (time.perf_counter() - T_START, what))
    sys.stderr.flush()


# ------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for k, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ distributed
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, world):
    """Max of a float over ranks (identity on one process)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def aggregate(elapsed_s, steps, world):
    """Whole-job throughput: every rank ran `steps`; the job took the slowest rank's time."""
    t = max_over_ranks(elapsed_s, world)
    return world * steps / t, t


# --------------------------------------------------------------- GPU arm
def gpu_run(w, args, precision, world, local, operator=0):
    import torch
    import __graft_entry__ as ge
    capi = ge.load_package().capi
    g = capi.Lattice(3, w["xyz"], w["p1"], w["p2"], w["layer"], w["Kn"], w["Tv"], w["cell"].particle_volume,
                     w["cell"].nneighbors)
    g.set_operator(operator)
    gb, gt = g.add_group(w["bottom"]), g.add_group(w["top"])
    bcs = [("disp", gb, 0, 0.0), ("disp", gb, 1, 0.0), ("disp", gb, 2, 0.0), ("disp", gt, 2, args.du)]
    opts = dict(tangent=capi.TANGENT_SYMMETRIC, precision=precision, max_iter=30, tol=1e-5, cg_tol=args.cg_tol)
    g.update()
    for _ in range(args.warmup):
        r = g.load_step(bcs, **opts)
        if r["status"] != 0:
            raise RuntimeError("warm-up step did not converge: %s" % r)
    stream = torch.cuda.ExternalStream(g.stream(), device="cuda:%d" % local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    g.reset_stats()
    newton, cg = [], []
    barrier(world)
    torch.cuda.synchronize()
    g.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        r = g.load_step(bcs, **opts)
        if r["status"] != 0:
            raise RuntimeError("timed step did not converge: %s" % r)
        newton.append(r["newton_iters"])
        cg.append(r["cg_iters"])
    e1.record(stream)
    e1.synchronize()
    g.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    st = g.stats()
    # kernel-timing pass: one more step with CUDA events around every
    # sparse-product launch.  The mixed solve then launches its kernels one by
    # one from the host instead of as one graph; the product kernel is the same.
    g.set_kernel_timing(True)
    g.reset_stats()
    r = g.load_step(bcs, **opts)
    g.synchronize()
    kt = g.stats()
    g.set_kernel_timing(False)
    if r["status"] != 0:
        raise RuntimeError("kernel-timing step did not converge: %s" % r)
    out = dict(ms=ms, stats=st, ktime=kt, newton=newton, cg=cg, handle=g, bcs=bcs, opts=opts)
    return out


def e2e_run(g, bcs, opts, steps, world):
    """Steps through the C ABI with host buffers: BC descriptors from pinned
    host memory, positions and internal forces read back into pinned memory."""
    import torch
    capi = sys.modules["lpm_mac_gb300"].capi
    n = g.n
    xyz_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    pin_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    L = g._L
    barrier(world)
    g.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        r = g.load_step(bcs, **opts)
        if r["status"] != 0:
            raise RuntimeError("e2e step did not converge: %s" % r)
        g._check(L.lpm_download(g.h, capi.F_XYZ, xyz_h.ctypes.data_as(dp)))
        g._check(L.lpm_download(g.h, capi.F_PIN, pin_h.ctypes.data_as(dp)))
    t1 = time.perf_counter()
    barrier(world)
    h2d = len(bcs) * ctypes.sizeof(capi.BC)
    d2h = 2 * n * 3 * 8
    return t1 - t0, h2d, d2h


def force_assembly_rate(g, capi, reps, local):
    """Device time of the force pass (lpm_update_geometry_force) and of the
    tangent assembly (symmetric variant, BC elimination) on the lattice as
    it stands, `reps` launches each, CUDA events on the library's stream."""
    import torch
    stream = torch.cuda.ExternalStream(g.stream(), device="cuda:%d" % local)
    out = {}
    for name, fn in (("force", lambda: g.update()),
                     ("assembly", lambda: g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE))):
        fn()
        g.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        out[name] = e0.elapsed_time(e1) / reps
    return out


def adjoint_cost(g, capi, w, cg_tol, local):
    """Device time of one lpm_backward_step at the converged state: the
    gradient of the top face's z reaction with respect to every bond's Kn and
    Tv (adjoint CG on the exact Jacobian, FP64)."""
    import numpy as np
    import torch
    c = np.zeros((g.n, 3))
    c[w["top"], 2] = 1.0
    stream = torch.cuda.ExternalStream(g.stream(), device="cuda:%d" % local)
    g.backward_step(dJdpin=c, cg_tol=cg_tol)  # buffers, warm
    g.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    gk, gt, iters, relres = g.backward_step(dJdpin=c, cg_tol=cg_tol)
    e1.record(stream)
    e1.synchronize()
    return {"ms": e0.elapsed_time(e1), "cg_iters": int(iters), "relres": relres, "cg_tol": cg_tol,
            "response": "reaction of the top face along z", "parameters": "Kn and Tv of every directed bond",
            "precision": "FP64 (exact Jacobian, matrix-free)"}


def setup_cost(w, capi):
    """The set-up before the first load step, through the public API with
    host arrays: the createBonds search on the GPU (lpm_find_bonds) checked
    against the CPU generator's bonds (identical arrays required), and the
    creation of the device lattice (upload, opposite bonds, pattern and its
    sliced layout).  The CPU time is the repository's k-d tree generator;
    the reference's own search is O(N^2) and is not timed."""
    xyz, cell = w["xyz"], w["cell"]
    capi.find_bonds(xyz[:4096], cell)  # first-call costs out of the way
    t0 = time.perf_counter()
    p1, p2, layer = capi.find_bonds(xyz, cell)
    t1 = time.perf_counter()
    same = bool(np.array_equal(p1, w["p1"]) and np.array_equal(p2, w["p2"]) and np.array_equal(layer, w["layer"]))
    t2 = time.perf_counter()
    g = capi.Lattice(3, xyz, w["p1"], w["p2"], w["layer"], w["Kn"], w["Tv"], cell.particle_volume,
                     cell.nneighbors)
    g.synchronize()
    t3 = time.perf_counter()
    g.close()
    return {"bond_search_ms": (t1 - t0) * 1e3, "bond_search_bonds_per_s": len(p1) / (t1 - t0),
            "bonds_identical_to_cpu_generator": same, "cpu_kdtree_generator_ms": w["find_bonds_s"] * 1e3,
            "lattice_create_ms": (t3 - t2) * 1e3, "timing": "host wall clock, host arrays in and out"}


def fatigue_cost(capi, local, cycles=3, precond=None, tangents=False):
    """Configuration 5 at full size: the compact-tension plate (hexagonal
    lattice, W = 40 mm from the load line, 0.15 mm spacing), HCF fatigue law
    with seeded per-particle A and B, nonlocal damage rate, pin loads
    cycled between 40 and 400 N (R = 0.1).  A static step to the minimum
    load, then `cycles` simulated cycles of lpm_fatigue_run (one load increment up and
    one down, a cycle jump of 1000), mixed precision.  Device time with CUDA
    events on the library's stream."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    lat, fat = pkg.lattice, pkg.fatigue
    xyz, p1, p2, layer, cell, info = lat.ct_specimen(40.0, 0.4, 0.15)
    n = len(xyz)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(110e3, 0.34, plane_stress=True, layout="row"))
    groups = lat.ct_groups(xyz, info, 0.15)
    rng = np.random.default_rng(20261203)
    params = np.stack([rng.uniform(1.5e-4, 2.5e-4, n), rng.uniform(0.50, 0.65, n), np.full(n, 1.079),
                       np.ones(n)], axis=1)
    L = 0.3
    nl_ptr, nl_idx = lat.nonlocal_neighbors(xyz, 1.5 * L)
    g = capi.Lattice(2, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)
    g.set_law(capi.LAW_FATIGUE_HCF, params)
    (cx, cy_b), (_, cy_t) = info["holes"]
    near_pins = (np.abs(xyz[:, 0] - cx) <= info["radius"]) & ((xyz[:, 1] >= cy_t) | (xyz[:, 1] <= cy_b))
    g.set_types(np.where(near_pins, 4, 0).astype(np.int32), 4)  # the pin regions do not damage
    g.set_nonlocal(nl_ptr, nl_idx, L)
    if precond is not None:
        g.set_preconditioner(precond, 0.0)
    g.update()
    gm, gt, gb = g.add_group(groups["mid"]), g.add_group(groups["top"]), g.add_group(groups["bottom"])
    f_max, R = 400.0, 0.1
    opts = dict(tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_MIXED, max_iter=30, tol=1e-5, cg_tol=1e-10)
    fixed = [("disp", gm, 1, 0.0), ("disp", gt, 0, 0.0), ("disp", gb, 0, 0.0)]
    r = g.load_step(fixed + [("force", gt, 0.0, R * f_max, 0.0), ("force", gb, 0.0, -R * f_max, 0.0)], **opts)
    if r["status"] != 0:
        raise RuntimeError("CT static step did not converge: %s" % r)
    if tangents:
        # d/d(log A) and d/dB of every particle's HCF parameters, carried
        # through the cycles
        da = np.zeros_like(params)
        da[:, 0] = params[:, 0]
        db = np.zeros_like(params)
        db[:, 1] = 1.0
        g.tangent_begin([da, db], tol=1e-10)
    unit = fixed + [("force", gt, 0.0, 1.0, 0.0), ("force", gb, 0.0, -1.0, 0.0)]
    spectrum = fat.ca_spectrum(f_max, R, 1000 * (cycles + 1))
    fat.run_cycles(g, unit, spectrum, 1, 0.001, max_calls=1, **opts)  # warm-up cycle
    stream = torch.cuda.ExternalStream(g.stream(), device="cuda:%d" % local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    g.synchronize()
    e0.record(stream)
    g.reset_stats()
    recs = fat.run_cycles(g, unit, spectrum, 1, 0.001, max_calls=cycles, **opts)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    stats = g.stats()
    persistent = stats["persistent_solves"]
    g.close()
    if any(rc["status"] != 0 for rc in recs):
        raise RuntimeError("CT fatigue cycle did not converge")
    return {"workload": "CT hex plate W=40 mm, 0.15 mm spacing (%d particles, %d bonds), HCF law, "
                        "pin load 40-400 N" % (n, len(p1)),
            "cycles_per_s": len(recs) / (ms * 1e-3), "ms_per_cycle": ms / len(recs), "cycles": len(recs),
            "newton_iters_per_cycle": statistics.mean(rc["newton_iters"] for rc in recs),
            "cg_iters_per_cycle": statistics.mean(rc["cg_iters"] for rc in recs),
            "cycle": "1 increment up, 1 down, cycle jump 1000 (lpm_fatigue_run)", "precision": "mixed",
            "persistent_solves": persistent,
            "preconditioner": "Jacobi (the reference's)" if precond is None else
            "Jacobi plus rigid-body modes of particle boxes (lpm_set_preconditioner, automatic box)",
            **({"tangent_directions": "d/d(log A), d/dB of the HCF law", "tangent_cg_iters": stats["tangent_cg_iters"]}
               if tangents else {})}


def softening_cost(capi, local, steps=4, max_warm=15, precond=None, tangents=False):
    """Configuration 3 at full size: the single-edge-notched hexagonal plate
    (401 rows of 201/200 particles, 0.1 mm spacing, crack over 0.3 W),
    softening bond law (alpha 3) with Weibull(k = 10, lambda = 1.2e-3)
    critical stretches, one draw per undirected bond, seed 20261203.  Top
    edge pulled by 1e-4 of the height per step (static solver with damage
    rounds on the eliminated tangent, mixed precision); untimed steps until
    some bond has softened, then `steps` timed steps.  Device time with CUDA
    events on the library's stream."""
    import torch
    import __graft_entry__ as ge
    lat = ge.load_package().lattice
    xyz, p1, p2, layer, cell = lat.sent_plate(201, 401, 0.1)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(69e3, 0.3, plane_stress=True, layout="row"))
    scrit = lat.weibull_draws(p1, p2, 10.0, 1.2e-3, 20261203)[np.lexsort((layer, p1))]
    g = capi.Lattice(2, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)
    g.set_law(capi.LAW_SOFTENING, [3.0, 1.0e-3])
    g.upload(capi.B_SCRIT, scrit)
    if precond is not None:
        g.set_preconditioner(precond, 0.0)
    g.update()
    c = xyz[:, 1]
    bottom, top = np.where(c < c.min() + 1e-9)[0], np.where(c > c.max() - 1e-9)[0]
    du = 1e-4 * (c.max() - c.min())
    gb, gc, gt = g.add_group(bottom), g.add_group(bottom[:1]), g.add_group(top)
    bcs = [("disp", gb, 1, 0.0), ("disp", gc, 0, 0.0), ("disp", gt, 1, du)]
    opts = dict(solver=capi.SOLVER_STATIC_ELIMINATE, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_MIXED,
                max_iter=60, tol=1e-5, cg_tol=1e-10)
    warm = 0
    while warm < max_warm and not (g.download(capi.B_BDAMAGE) > 0).any():
        if g.load_step(bcs, **opts)["status"] != 0:
            raise RuntimeError("SENT step did not converge")
        warm += 1
    if tangents:
        # d/d(log E) and d/d(log lambda) of the Weibull scale, carried
        # through every damage round of the timed steps
        g.tangent_begin_softening([{"dKn": g.download(capi.B_KN), "dTv": g.download(capi.B_TV)},
                                   {"dscrit": g.download(capi.B_SCRIT)}], tol=1e-10)
    stream = torch.cuda.ExternalStream(g.stream(), device="cuda:%d" % local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    g.synchronize()
    g.reset_stats()
    e0.record(stream)
    recs = [g.load_step(bcs, **opts) for _ in range(steps)]
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    d = g.download(capi.B_BDAMAGE)
    stats = g.stats()
    persistent = stats["persistent_solves"]
    if tangents:
        c = xyz[:, 1]
        top_ids = np.where(c > c.max() - 1e-9)[0]
        dR = [float(g.tangent_get(k, capi.T_PIN)[top_ids, 1].sum()) for k in range(2)]
        g.tangent_end()
    g.close()
    if any(r["status"] != 0 for r in recs):
        raise RuntimeError("SENT step did not converge")
    return {"workload": "SENT hex plate 401 rows x 201/200, 0.1 mm spacing (%d particles, %d bonds), crack 0.3 W, "
                        "softening law, Weibull critical stretch" % (len(xyz), len(p1)),
            "steps_per_s": steps / (ms * 1e-3), "ms_per_step": ms / steps, "steps": steps, "untimed_steps": warm,
            "newton_iters_per_step": statistics.mean(r["newton_iters"] for r in recs),
            "damage_rounds_per_step": statistics.mean(r["damage_rounds"] for r in recs),
            "cg_iters_per_step": statistics.mean(r["cg_iters"] for r in recs),
            "softened_bonds": int((d > 0).sum()), "broken_bonds": int((d >= 1).sum()),
            "precision": "mixed", "solver": "static with damage rounds, eliminated tangent",
            "us_per_cg_iteration": 1e3 * ms / max(1, sum(r["cg_iters"] for r in recs)), "persistent_solves": persistent,
            "preconditioner": "Jacobi (the reference's)" if precond is None else
            "Jacobi plus rigid-body modes of particle boxes (lpm_set_preconditioner, automatic box)",
            **({"tangent_directions": "d/d(log E), d/d(log Weibull scale)", "dR_top": dR,
                "tangent_cg_iters": stats["tangent_cg_iters"]} if tangents else {})}


def j2_sensitivity_cost(capi, local, ncell=40, steps=4):
    """The tangent-linear sensitivity of a J2 load history (configuration 4
    form: BCC polycrystal, 20 grains, E = 110 GPa, nu = 0.34, yield 900 MPa,
    hardening 1 GPa) with respect to the yield stress and the hardening
    modulus: device time of `steps` plastic load steps without and with the
    two tangent directions carried along (mixed precision, tangent solves
    to 1e-10)."""
    import math
    import torch
    import __graft_entry__ as ge
    lat = ge.load_package().lattice
    xyz, gid = lat.bcc_polycrystal(ncell, 0.2, 20, 11)
    cell = lat.UnitCell(lat.BCC3D, 0.2 * math.sqrt(3.0) / 4.0)
    xyz = xyz[lat.prune_weak(xyz, cell, 6)]
    p1, p2, layer = lat.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(110e3, 0.34, layout="row"))
    z = xyz[:, 2]
    bottom, top = np.where(z < 0.1)[0], np.where(z > z.max() - 0.1)[0]
    du = 0.0005 * (z.max() - z.min())
    out = {}
    for tangent in (False, True):
        g = capi.Lattice(3, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)
        g.set_law(capi.LAW_J2, [110e3, 0.34, 900.0, 0.0, 1e3, 0.0, 0.0])
        g.update()
        gb, gt = g.add_group(bottom), g.add_group(top)
        bcs = [("disp", gb, 0, 0.0), ("disp", gb, 1, 0.0), ("disp", gb, 2, 0.0), ("disp", gt, 2, du)]
        opts = dict(solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_MIXED,
                    max_iter=30, tol=1e-5, cg_tol=1e-10)
        for _ in range(3):  # up to yield
            g.load_step(bcs, **opts)
        if tangent:
            g.tangent_begin([[0, 0, 1, 0, 0, 0, 0], [0, 0, 0, 0, 1, 0, 0]], tol=1e-10)
        stream = torch.cuda.ExternalStream(g.stream(), device="cuda:%d" % local)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        g.reset_stats()
        g.synchronize()
        e0.record(stream)
        for _ in range(steps):
            r = g.load_step(bcs, **opts)
            if r["status"] != 0:
                raise RuntimeError("J2 step did not converge: %s" % r)
        e1.record(stream)
        e1.synchronize()
        st = g.stats()
        out["with" if tangent else "without"] = (e0.elapsed_time(e1) / steps, st["tangent_cg_iters"] / steps)
        plastic = bool(np.abs(g.download(capi.B_DLP)).max() > 0)
        g.close()
    return {"workload": "BCC polycrystal %d^3 cells, 20 grains (%d particles), J2, plastic steps" % (ncell, len(xyz)),
            "directions": "d/d(yield stress), d/d(hardening modulus)", "forward_ms_per_step": out["without"][0],
            "with_tangents_ms_per_step": out["with"][0],
            "relative_to_forward_step": out["with"][0] / out["without"][0],
            "tangent_cg_iters_per_step": out["with"][1], "plastic": plastic}


def polycrystal_cost(capi, local, ncell=60, plastic_steps=6, unload_steps=3):
    """Configuration 4 at full size: a BCC polycrystal of 60^3 cells (0.2 mm)
    with 20 Voronoi grains of uniform SO(3) orientations (seeded), J2 law
    with E = 110 GPa, nu = 0.34, yield 900 MPa, linear isotropic hardening
    1 GPa, uniaxial tension in z at 2 % strain over 100 steps and unloading
    over 20.  Untimed steps of 0.1 % take the lattice to 0.7 % strain;
    then `plastic_steps` loading steps of 0.02 % and `unload_steps`
    unloading steps of 0.1 % are timed, without and with the two tangent
    directions (d/d yield stress, d/d hardening modulus) carried along.
    Mixed precision, BC elimination.  Device time with CUDA events."""
    import math
    import torch
    import __graft_entry__ as ge
    lat = ge.load_package().lattice
    t0 = time.perf_counter()
    xyz, gid = lat.bcc_polycrystal(ncell, 0.2, 20, 11)
    cell = lat.UnitCell(lat.BCC3D, 0.2 * math.sqrt(3.0) / 4.0)
    keep = np.arange(len(xyz))
    while True:  # drop particles with fewer than 6 bonds (lattice.prune_weak, searched on the GPU)
        q1, _, _ = capi.find_bonds(xyz[keep], cell)
        ok = np.bincount(q1, minlength=len(keep)) >= 6
        if ok.all():
            break
        keep = keep[ok]
    xyz = xyz[keep]
    p1, p2, layer = capi.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(110e3, 0.34, layout="row"))
    setup_s = time.perf_counter() - t0
    progress("polycrystal: %d particles set up" % len(xyz))
    z = xyz[:, 2]
    bottom, top = np.where(z < 0.1)[0], np.where(z > z.max() - 0.1)[0]
    L = z.max() - z.min()
    du = 0.02 * L / 100
    out = {}
    for tangent in (False, True):
        g = capi.Lattice(3, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)
        g.set_law(capi.LAW_J2, [110e3, 0.34, 900.0, 0.0, 1e3, 0.0, 0.0])
        g.update()
        gb, gt = g.add_group(bottom), g.add_group(top)
        fixed = [("disp", gb, 0, 0.0), ("disp", gb, 1, 0.0), ("disp", gb, 2, 0.0)]
        opts = dict(solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_MIXED,
                    max_iter=30, tol=1e-5, cg_tol=1e-10, cg_maxit=20000, max_cuts=2)
        for _ in range(7):
            r = g.load_step(fixed + [("disp", gt, 2, 0.001 * L)], **opts)
            if r["status"] != 0:
                raise RuntimeError("polycrystal elastic step did not converge: %s" % r)
        progress("polycrystal: elastic steps, last %s" % r)
        if tangent:
            g.tangent_begin([[0, 0, 1, 0, 0, 0, 0], [0, 0, 0, 0, 1, 0, 0]], tol=1e-10)
        stream = torch.cuda.ExternalStream(g.stream(), device="cuda:%d" % local)
        times, cgs = [], []
        for n_steps, inc in ((plastic_steps, du), (unload_steps, -5 * du)):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            g.synchronize()
            e0.record(stream)
            its = 0
            for _ in range(n_steps):
                r = g.load_step(fixed + [("disp", gt, 2, inc)], **opts)
                if r["status"] != 0:
                    raise RuntimeError("polycrystal step did not converge: %s" % r)
                its += r["cg_iters"]
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / n_steps)
            cgs.append(its / n_steps)
            progress("polycrystal: %d steps, %.1f ms each, tangents %s" % (n_steps, times[-1], tangent))
        plastic = bool(np.abs(g.download(capi.B_DLP)).max() > 0)
        out[tangent] = (times, cgs, plastic)
        g.close()
    (tl, tu), (cl, cu), plastic = out[False]
    (sl, su), _, _ = out[True]
    return {"workload": "BCC polycrystal %d^3 cells, 20 grains (%d particles, %d bonds), J2, tension to 2 %% in 100 "
                        "steps, unloading in 20" % (ncell, len(xyz), len(p1)),
            "loading_ms_per_step": tl, "unloading_ms_per_step": tu, "loading_cg_iters_per_step": cl,
            "unloading_cg_iters_per_step": cu, "steps_per_s_loading": 1e3 / tl, "plastic": plastic,
            "with_tangents_loading_ms_per_step": sl, "with_tangents_unloading_ms_per_step": su,
            "tangent_cost_relative": (sl + su) / (tl + tu), "timed_steps": [plastic_steps, unload_steps],
            "full_history_estimate_s": (100 * tl + 20 * tu) / 1e3, "setup_s": setup_s,
            "directions": "d/d(yield stress), d/d(hardening modulus)", "precision": "mixed"}


def force_bytes(nb, n):
    """Algorithmic bytes of one force pass: per directed bond the partner
    index, dis0, dLp, bdamage, Kn, Tv and the bond force written; per
    particle positions, internal force, layer sums and stress."""
    return nb * 52 + n * (24 + 24 + 64 + 48)


def column_index_bytes(g):
    """Bytes per block of the FP32 product's column index: 2 when every
    column offset of the pattern fits 16 bits (the library then reads 16-bit
    offsets), else 4."""
    import numpy as np
    cptr, cidx = g.pattern()
    rows = np.repeat(np.arange(g.n, dtype=np.int64), np.diff(cptr))
    off = np.abs(cidx.astype(np.int64) - rows)
    return 2 if off.size == 0 or off.max() <= 32767 else 4


def spmv_bytes(nblk, n, dim, value_bytes, index_bytes=4, row_sums=False, out_bytes=None):
    """Algorithmic bytes of one CG sparse-product launch: every block's
    dim*dim values and column index, each row's block count, the search
    direction read once and the product written once (out_bytes per entry:
    the FP32 product writes a double-float pair, 8 bytes), and for the FP32
    difference form each row's block row sum (dim*dim FP32 values)."""
    out = value_bytes if out_bytes is None else out_bytes
    b = nblk * (dim * dim * value_bytes + index_bytes) + n * 4 + n * dim * (value_bytes + out)
    return b + (n * dim * dim * 4 if row_sums else 0)


def mf_bytes(nb, n, dim=3, value_bytes=4, out_bytes=8):
    """Algorithmic bytes of one matrix-free product (two passes): per
    directed bond the partner word, the opposite bond's cosines and t' read
    in pass 1 and again with a' - t' in pass 2; per particle the row sums,
    S, U, V of both layers, the first pass's two sums per layer written and
    read, the input read by both passes, the output written and the
    eliminated-DOF flags read twice."""
    per_bond = 2 * 4 + (2 * dim + 3) * value_bytes
    per_particle = (dim * dim + 3 * 6 + 2 * 4) * value_bytes + 2 * dim * value_bytes + dim * out_bytes + 2 * dim
    return nb * per_bond + n * per_particle


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel_key, nblk):
    """DRAM bytes per launch of the CG sparse product: the bytes per block
    ncu measured on the 61^3 lattice (profiles/cg_spmv_sc61_traffic.json)
    times this workload's block count (traffic grows with the blocks
    processed)."""
    path = os.path.join(ROOT, "profiles", "cg_spmv_sc61_traffic.json")
    try:
        with open(path) as f:
            return float(json.load(f)["kernels"][kernel_key]["bytes_per_block"]) * nblk
    except (OSError, KeyError, ValueError):
        return None


# --------------------------------------------------------------- CPU arm
def cpu_oracle_system(w, threads):
    import __graft_entry__ as ge
    oracle = ge.load_oracle()
    oracle.lib().lo_set_threads(threads)
    o = oracle.OracleSystem(3, w["xyz"], w["p1"], w["p2"], w["layer"], w["Kn"], w["Tv"], w["cell"].particle_volume,
                            w["cell"].nneighbors)
    return oracle, o


def oracle_bcs(w, du):
    """Boundary arrays of one load step for the oracle: bottom face clamped,
    top face moved by du along z."""
    n = len(w["xyz"])
    apply = np.zeros((n, 3), np.int32)
    apply[w["bottom"], :] = 1
    apply[w["top"], 2] = 1
    dd = np.zeros((n, 3))
    dd[w["top"], 2] = du
    return apply, dd


def oracle_step(o, w, args):
    """One complete FP64 load step on the CPU oracle (symmetric tangent, BC
    elimination, Jacobi CG to cg_tol, Newton to 1e-5): wall time, Newton
    and CG iteration counts."""
    apply, dd = oracle_bcs(w, args.du)
    o.clear_log()
    t0 = time.perf_counter()
    st = o.load_step(apply, dd, sym=1, bc_elim=1, cg_tol=args.cg_tol)
    t = time.perf_counter() - t0
    if st < 0:
        raise RuntimeError("CPU oracle load step did not converge")
    log = o.log()
    return t, len(log), int(log[:, 0].sum())


REFERENCE_BUDGET_S = 100.0  # complete CPU load steps are timed until this much time is spent


def run_reference(args):
    """The reference algorithm on the host cores: complete FP64 load steps of
    the same workload on the CPU oracle with every host thread, timed one by
    one until REFERENCE_BUDGET_S is spent (at least one).  The value is the
    number of complete steps over their total time; nothing is
    extrapolated."""
    world, rank, local = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    w = workload(args.n)
    oracle, o = cpu_oracle_system(w, threads)
    o.update()
    times, newton, cg = [], [], []
    while len(times) < max(1, args.steps):
        t, ni, ci = oracle_step(o, w, args)
        times.append(t)
        newton.append(ni)
        cg.append(ci)
        if sum(times) >= REFERENCE_BUDGET_S:
            break
    total = sum(times)
    value = len(times) / total
    sample = ("%d complete FP64 load step(s) from the undeformed lattice, timed whole (%s s; %s Newton / %s CG "
              "iterations); steps are timed until %.0f s is spent" %
              (len(times), ", ".join("%.1f" % t for t in times), ", ".join(map(str, newton)),
               ", ".join(map(str, cg)), REFERENCE_BUDGET_S))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": len(times), "warmup": 0, "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": describe(w), "precision": "FP64 Jacobi CG (the reference's form)",
                       "tangent": "symmetric K_ii[1][0]", "bc": "eliminated (updateStiffnessDispBC)",
                       "cg_tol": args.cg_tol, "newton_tol": 1e-5, "threads": threads,
                       "solver": "CPU oracle (the reference algorithm restated, pinned bit for bit to it)",
                       "steps_requested": args.steps, "warmup_requested": args.warmup},
            "newton_iters_per_step": statistics.mean(newton), "cg_iters_per_step": statistics.mean(cg),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def rel_err(a, b):
    """max |a - b| / max |b|."""
    s = float(np.abs(b).max())
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0))


def headline_parity(w, args, capi):
    """The first load step of the workload, from the undeformed lattice, three
    ways: the CPU oracle in FP64 (all host threads; timed whole, the CPU
    baseline), the GPU in FP64 and the GPU in mixed precision.  Errors are
    max |u - u_ref| / max |u_ref| over the displacements, and relative errors
    of the top face's z reaction."""
    threads = os.cpu_count() or 1
    oracle, o = cpu_oracle_system(w, threads)
    o.update()
    t_cpu, ni_cpu, cg_cpu = oracle_step(o, w, args)
    xyz, top = w["xyz"], w["top"]
    u_ref = o.get(oracle.XYZ) - xyz
    R_ref = float(o.get(oracle.PIN)[top, 2].sum())
    _, nr_o, nR_o = o.residual()
    del o
    gpu = {}
    for name, prec in (("fp64", capi.PREC_FP64), ("mixed", capi.PREC_MIXED)):
        g = capi.Lattice(3, xyz, w["p1"], w["p2"], w["layer"], w["Kn"], w["Tv"], w["cell"].particle_volume,
                         w["cell"].nneighbors)
        gb, gt = g.add_group(w["bottom"]), g.add_group(top)
        bcs = [("disp", gb, 0, 0.0), ("disp", gb, 1, 0.0), ("disp", gb, 2, 0.0), ("disp", gt, 2, args.du)]
        g.update()
        r = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=prec, max_iter=30, tol=1e-5,
                        cg_tol=args.cg_tol)
        if r["status"] != 0:
            raise RuntimeError("first-step parity: GPU step did not converge: %s" % r)
        nr, nR = g.residual()
        gpu[name] = dict(u=g.download(capi.F_XYZ) - xyz, R=float(g.download(capi.F_PIN)[top, 2].sum()),
                         newton=r["newton_iters"], cg=r["cg_iters"], ratio=nr / nR)
        g.close()
    f, m = gpu["fp64"], gpu["mixed"]
    parity = {"step": "first load step from the undeformed lattice, same inputs on CPU and GPU",
              "norm": "max|u - u_ref| / max|u_ref| (displacements); |R - R_ref| / |R_ref| (top-face z reaction)",
              "fp64_vs_oracle": rel_err(f["u"], u_ref), "fp64_reaction_vs_oracle": abs(f["R"] - R_ref) / abs(R_ref),
              "mixed_vs_fp64": rel_err(m["u"], f["u"]), "mixed_reaction_vs_fp64": abs(m["R"] - f["R"]) / abs(f["R"]),
              "mixed_vs_oracle": rel_err(m["u"], u_ref),
              "newton_residual_over_reaction": {"oracle": nr_o / nR_o, "fp64": f["ratio"], "mixed": m["ratio"]},
              "newton_iters": {"oracle": ni_cpu, "fp64": f["newton"], "mixed": m["newton"]},
              "cg_iters": {"oracle": cg_cpu, "fp64": f["cg"], "mixed": m["cg"]}, "cg_tol": args.cg_tol}
    cpu = {"value": 1.0 / t_cpu, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": "one complete FP64 load step (the first, from the undeformed lattice) of the same workload on "
                     "the CPU oracle, timed whole: %.1f s, %d Newton / %d CG iterations" % (t_cpu, ni_cpu, cg_cpu)}
    return parity, cpu


def run_gb300(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    import __graft_entry__ as ge
    pkg = ge.load_package()
    capi = pkg.capi
    capi.set_device(local)
    w = workload(args.n)
    clocks = ClockSampler(local)
    results = {}
    order = ([] if args.no_fp64 else [capi.PREC_FP64]) + [capi.PREC_MIXED]
    for prec in order:
        if prec == capi.PREC_MIXED:
            clocks.start()
        progress("load steps, %s" % ("mixed" if prec == capi.PREC_MIXED else "FP64"))
        results[prec] = gpu_run(w, args, prec, world, local)
        if prec == capi.PREC_MIXED:
            clk = clocks.stop()
    mixed = results[capi.PREC_MIXED]
    value, t_mixed = aggregate(mixed["ms"] / 1e3, args.steps, world)
    g = mixed["handle"]
    # e2e through the C ABI with host buffers
    if args.no_extras:
        e2e_s, h2d, d2h = mixed["ms"] / 1e3, 0, 0
    else:
        e2e_s, h2d, d2h = e2e_run(g, mixed["bcs"], mixed["opts"], args.steps, world)
    e2e_value, _ = aggregate(e2e_s, args.steps, world)
    st = mixed["stats"]
    n, nb, nblk = g.n, g.nb, g.nblk
    launches = mixed["ktime"]["spmv32_launches"]
    avg_ms = mixed["ktime"]["spmv32_ms"] / max(launches, 1)
    byts = spmv_bytes(nblk, n, 3, 4, column_index_bytes(g), row_sums=True, out_bytes=8)
    peak, peak_kind = measured_peaks()
    achieved = byts / (avg_ms * 1e-3) / 1e9
    traffic = profiled_traffic("float", nblk)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_mixed * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 CG + f64 refinement/forces", "data": "synthetic",
            "config": {"workload": describe(w), "precision": "FP32 CG inside FP64 iterative refinement",
                       "tangent": "symmetric K_ii[1][0]", "bc": "eliminated (updateStiffnessDispBC)",
                       "cg_tol": args.cg_tol, "newton_tol": 1e-5, "l2": "inputs larger than L2 (FP32 operator %.2f GB)"
                       % (nblk * 40 / 1e9), "parallelism": "replicas x%d" % world},
            "newton_iters_per_step": statistics.mean(mixed["newton"]),
            "cg_iters_per_step": statistics.mean(mixed["cg"]),
            "cg_iters_per_s": sum(mixed["cg"]) / (mixed["ms"] / 1e3),
            "gpu_launches": int(st["kernel_launches"]),
            "roofline": {"kernel": "k_cg_spmv<float,3>", "bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "algorithmic_bytes_per_launch": byts, "avg_launch_ms": avg_ms, "launches": launches,
                         "launch_timing": "CUDA events around each launch, kernel-timing step after the timed steps",
                         "peak_kind": peak_kind + " (hbm_gbs copy bandwidth)"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}}
    if clk:
        line["clocks"] = clk
    if capi.PREC_FP64 in results:
        f = results[capi.PREC_FP64]
        fv, tf = aggregate(f["ms"] / 1e3, args.steps, world)
        sf = f["ktime"]
        avg64 = sf["spmv_ms"] / max(sf["spmv_launches"], 1)
        b64 = spmv_bytes(nblk, n, 3, 8)
        line["fp64"] = {"value": fv, "ms_per_step": tf * 1e3 / args.steps,
                        "newton_iters_per_step": statistics.mean(f["newton"]),
                        "cg_iters_per_step": statistics.mean(f["cg"]),
                        "spmv_avg_launch_ms": avg64, "spmv_achieved_gbs": b64 / (avg64 * 1e-3) / 1e9,
                        "spmv_fp64_gflops": 2 * nblk * 9 / (avg64 * 1e-3) / 1e9,
                        "mixed_speedup": value / fv}
        f["handle"].close()
    if not args.no_matrix_free:
        progress("load steps, matrix-free")
        mf = gpu_run(w, args, capi.PREC_MIXED, world, local, operator=capi.OPERATOR_MATRIX_FREE)
        mv, tm = aggregate(mf["ms"] / 1e3, args.steps, world)
        kt = mf["ktime"]
        mavg = kt["spmv32_ms"] / max(kt["spmv32_launches"], 1)
        mb = mf_bytes(nb, n)
        line["matrix_free"] = {"value": mv, "ms_per_step": tm * 1e3 / args.steps,
                               "cg_iters_per_step": statistics.mean(mf["cg"]),
                               "newton_iters_per_step": statistics.mean(mf["newton"]),
                               "product_avg_launch_ms": mavg, "product_algorithmic_bytes": mb,
                               "product_achieved_gbs": mb / (mavg * 1e-3) / 1e9,
                               "product_frac": mb / (mavg * 1e-3) / 1e9 / peak,
                               "speedup_vs_assembled": mv / value,
                               "operator": "tangent applied from bond data in two passes (lpm_set_operator), "
                                           "mixed precision, no assembly"}
        mf["handle"].close()
    if args.no_extras:
        g.close()
        if rank == 0:
            print(json.dumps(line), flush=True)
        return 0
    progress("adjoint")
    adj = adjoint_cost(g, capi, w, args.cg_tol, local)
    line["adjoint"] = dict(adj, relative_to_forward_step=adj["ms"] / (t_mixed * 1e3 / args.steps))
    fa = force_assembly_rate(g, capi, 5, local)
    fb = force_bytes(nb, n)
    line["bonds_per_s"] = {"force": world * nb / (fa["force"] * 1e-3),
                           "force_plus_assembly": world * nb / ((fa["force"] + fa["assembly"]) * 1e-3),
                           "force_ms": fa["force"], "assembly_ms": fa["assembly"], "directed_bonds": nb,
                           "force_achieved_gbs": fb / (fa["force"] * 1e-3) / 1e9,
                           "force_algorithmic_bytes": fb}
    run_leg(line, "setup", setup_cost, w, capi)
    run_leg(line, "fatigue", fatigue_cost, capi, local)
    run_leg(line, "fatigue_coarse", fatigue_cost, capi, local, precond=capi.PRECOND_COARSE)
    run_leg(line, "fatigue_sensitivity", fatigue_cost, capi, local, precond=capi.PRECOND_COARSE, tangents=True)
    fc, fs = line.get("fatigue_coarse", {}), line.get("fatigue_sensitivity", {})
    if "ms_per_cycle" in fc and "ms_per_cycle" in fs:
        fs["relative_to_forward_cycle"] = fs["ms_per_cycle"] / fc["ms_per_cycle"]
    if args.softening_steps > 0:
        run_leg(line, "softening", softening_cost, capi, local, steps=args.softening_steps)
        run_leg(line, "softening_coarse", softening_cost, capi, local, steps=args.softening_steps,
                precond=capi.PRECOND_COARSE)
        run_leg(line, "softening_sensitivity", softening_cost, capi, local, steps=args.softening_steps,
                precond=capi.PRECOND_COARSE, tangents=True)
        sf, ss = line.get("softening_coarse", {}), line.get("softening_sensitivity", {})
        if "ms_per_step" in sf and "ms_per_step" in ss:
            ss["relative_to_forward_step"] = ss["ms_per_step"] / sf["ms_per_step"]
    run_leg(line, "j2_sensitivity", j2_sensitivity_cost, capi, local)
    run_leg(line, "polycrystal", polycrystal_cost, capi, local)
    g.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        progress("CPU baseline and parity")
        line["parity"], line["cpu_baseline"] = headline_parity(w, args, capi)
    progress("done")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


ARGS = None


def profile_solve(case):
    """One mixed solve of 300 iterations on the eliminated symmetric tangent
    of a full-size plate after one FP64 load step (top edge up by 1e-3 mm),
    with a seeded right-hand side: a small case for profiling the persistent
    solve kernel (k_mx_persistent).  Device time with CUDA events."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    lat, capi = pkg.lattice, pkg.capi
    coarse = case.endswith("-coarse")
    case = case.split("-")[0]
    if case == "sent":
        xyz, p1, p2, layer, cell = lat.sent_plate(201, 401, 0.1)
        E, nu = 69e3, 0.3
    else:
        xyz, p1, p2, layer, cell, _ = lat.ct_specimen(40.0, 0.4, 0.15)
        E, nu = 110e3, 0.34
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(E, nu, plane_stress=True, layout="row"))
    g = capi.Lattice(2, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)
    y = xyz[:, 1]
    bottom, top = np.where(y < y.min() + 1e-9)[0], np.where(y > y.max() - 1e-9)[0]
    gb, gc, gt = g.add_group(bottom), g.add_group(bottom[:1]), g.add_group(top)
    g.update()
    r = g.load_step([("disp", gb, 1, 0.0), ("disp", gc, 0, 0.0), ("disp", gt, 1, 1e-3)],
                    tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64, cg_tol=1e-10)
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    if coarse:
        g.set_preconditioner(capi.PRECOND_COARSE, 0.0)
    g.upload(capi.F_RESIDUAL, np.random.default_rng(5).standard_normal(g.ndof))
    stream = torch.cuda.ExternalStream(g.stream(), device="cuda:0")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g.reset_stats()
    g.synchronize()
    e0.record(stream)
    it, rr, st = g.solve(capi.PREC_MIXED, 1e-8, maxit=300)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    out = {"profile_solve": case + ("-coarse" if coarse else ""), "particles": len(xyz), "blocks": g.nblk, "iterations": it, "ms": ms,
           "us_per_iteration": 1e3 * ms / max(it, 1), "persistent_solves": g.stats()["persistent_solves"],
           "load_step": r}
    g.close()
    print(json.dumps(out))
    return 0


def main(argv=None):
    global ARGS
    ARGS = parse_args(argv)
    if ARGS.profile_solve:
        return profile_solve(ARGS.profile_solve)
    if ARGS.impl == "reference":
        return run_reference(ARGS)
    return run_gb300(ARGS)


if __name__ == "__main__":
    sys.exit(main())
