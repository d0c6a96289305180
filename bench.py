#!/usr/bin/env python
"""bench.py — particle-iterations/s of the XPBD cloth solver on synthetic cloth grids.

One step = one frame (frame_dt = 1/60 s) of every cloth of the workload: substeps x
iterations Jacobi sweeps plus collision, hashing and normals, exactly the work
VtClothSolverGPU::Simulate does per fixed frame.  particle-iterations per step =
sum over cloths of N * substeps * iterations.

Default workload: the mixed-size batch (512 independent grid cloths, side log-uniform in
[16, 256], ~6 M particles, 5 substeps x 10 iterations, sphere + plane each, two pinned
corners).  Its working set (~3 GB) is far larger than L2, so no flush is needed between
steps.

Arms:
  --impl ours (default)  the CUDA solver through the C ABI.  `value`: device-resident
                         frames timed with CUDA events; `e2e`: the same frames with the
                         per-frame collider upload from host memory and the positions +
                         normals read back into pinned host memory inside the timed region.
                         The JSON line also carries the plain (one cloth at a time)
                         drop-in solver's rate and p50/p99 frame latency, the dominant
                         kernel's roofline, and the CPU oracle timed on a bounded sample.
  --impl reference       the CPU restatement of the reference solver (the oracle, which
                         reproduces the reference's own kernels bit for bit; those kernels
                         compile for the CPU only where the reference tree is, not on the
                         GPU machine), all host cores, one process per core, bounded sample.
  --variant fast|exact   the library build the ours arm times (default fast: contracted
                         arithmetic within the stated tolerance of the oracle; the JSON
                         line also carries the exact build's rate, `exact_build`).
Multi-GPU (torchrun): each rank runs its own copy of the workload (cloths are
independent; no collective on the data path) -> weak scaling.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-iterations/s and p99 frame latency, batched vs plain, same GB300"
UNIT = "particle-iterations/s"


# ---------------------------------------------------------------------------- helpers
def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def workload(name: str, seed: int = 0):
    from velvet_gb300 import workloads as W

    if name == "batched":
        return W.batched(512, seed=seed)
    if name == "small":
        return W.small()
    if name == "small32":  # the small configuration's setting on a 32x32 cloth
        wl = W.small()
        spec = wl.cloths[0]
        wl.cloths[0] = W.ClothSpec(32, spec.spacing, W.horizontal_cloth(32, spec.spacing, 0.8), [0, 31],
                                   spec.colliders)
        wl.name = "small_32x32"
        return wl
    if name == "large":
        return W.large()
    if name == "stress":
        return W.stress(seed=seed)
    if name == "grid1024":
        wl = W.stress(seed=seed)
        spec = wl.cloths[0]
        spec.attached = [0, spec.side - 1]
        wl.name = "grid_1024x1024_two_corners"
        return wl
    raise SystemExit(f"unknown workload {name}")


def pits_per_frame(wl) -> int:
    return sum(c.num_particles for c in wl.cloths) * wl.substeps * wl.iterations


def iteration_bytes(wl) -> float:
    """Algorithmic bytes of one Jacobi iteration over every cloth:
    12*C_s + 20*C_b + 12*C_a + 28*N (constraint streams at information size, predicted
    position read 12 B + inverse mass 4 B + write 12 B per particle).  C_a counts only
    cloths whose LRA rest distances are kept per particle (at most GRID_LRA_CACHED slots):
    with more slots the kernel recomputes them instead of streaming a table, and that
    term is reported apart (lra_roofline)."""
    b = 0.0
    for c in wl.cloths:
        V = c.side
        Cs = 2 * V * (V - 1) + 2 * (V - 1) ** 2
        Cb = (V - 1) ** 2
        Ca = len(c.attached) * V * V if len(c.attached) <= GRID_LRA_CACHED else 0
        b += 12 * Cs + 20 * Cb + 12 * Ca + 28 * V * V
    return b


# FP32 operations per (particle, LRA slot) pair of an iteration when the rest distance is
# recomputed: |slot0 - x0| (3 sub, 3 mul, 2 add, sqrt), times the stretchiness, the
# inverse-mass test, |p - slot| (3 sub, 3 mul, 2 add, sqrt) and the comparison.
LRA_OPS_PER_PAIR = 21
GRID_LRA_CACHED = 4  # slots whose rest distances the tile kernel keeps per particle


def lra_roofline(wl, t_iter_ms: float, clock_info) -> dict | None:
    """Cloths with more LRA slots than the tile kernel caches (the stress configuration's
    whole attached row): the (particle, slot) pairs of an iteration as an equivalent
    rate.  The kernel skips every group of slots whose bounding boxes prove that none of
    its pairs fires (exactly: a skipped pair contributes nothing), so most pairs are never
    evaluated and the equivalent FP32 rate is compared with the SMs' FP32 issue rate only
    to show how much work the bound removes; it is not a roofline fraction."""
    import torch

    pairs = sum(c.side * c.side * len(c.attached) for c in wl.cloths if len(c.attached) > GRID_LRA_CACHED)
    if not pairs or t_iter_ms <= 0:
        return None
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clock_info or {}).get("sm_mhz") or (clock_info or {}).get("sm_max_mhz") or 2070.0
    peak = sms * 128 * mhz * 1e6 / 1e12
    eq = pairs * LRA_OPS_PER_PAIR / (t_iter_ms / 1000.0) / 1e12
    return {"pairs_per_iteration": pairs, "pairs_per_second": pairs / (t_iter_ms / 1000.0),
            "ops_per_pair_if_evaluated": LRA_OPS_PER_PAIR, "equivalent_tflops": eq,
            "fp32_issue_peak_tflops": peak, "equivalent_over_peak": eq / peak,
            "peak_source": f"{sms} SMs x 128 FP32 lanes x {mhz:.0f} MHz (nominal issue rate at the sampled clock)",
            "note": "groups of slots (16, more above 1,024 slots) proven quiet by bounding boxes are "
                    "skipped; an equivalent rate above the issue peak is the work the bound removes, "
                    "not an achieved rate"}


def frame_bytes(wl, k_mean: float, interleaved_hash: int = 3) -> float:
    """Algorithmic bytes of one frame over every cloth (compulsory traffic, vec3 = 12 B,
    index = 4 B, each datum once per kernel phase): per substep predict 48 + SDF 36 +
    finalize 48 + collide 40 + 4(k+1) per particle, per hash 20 + 16 ceil(bits/8) + 4 + 8
    + 8 + 28 + 4(k+1) per particle (keys, sort passes, ranges, neighbour lists), per frame
    pre-SDF 24 + 24 + normals 24 per particle, plus the iterations' bytes."""
    hashes = -(-wl.substeps // interleaved_hash)  # substeps 0, I_h, 2 I_h, ...
    b = wl.substeps * wl.iterations * iteration_bytes(wl)
    for c in wl.cloths:
        n = c.side * c.side
        bits = max(1, math.ceil(math.log2(2 * n)))
        b += wl.substeps * n * (48 + 36 + 48 + 40 + 4 * (k_mean + 1))
        b += hashes * n * (20 + 16 * math.ceil(bits / 8) + 4 + 8 + 8 + 28 + 4 * (k_mean + 1))
        b += n * (24 + 24 + 24)
    return b


def mean_cached_neighbours(solvers, max_particles: int = 400_000) -> float | None:
    """k: entries per particle in the neighbour lists of a size-preserving sample of
    simulated plain solvers (the same lists the batched form builds)."""
    import velvet_gb300 as vg

    total, count = 0, 0
    step = max(1, int(math.ceil(sum(s[1].num_particles for s in solvers) / max_particles)))
    for s, spec, _ in solvers[::step]:
        nb = s.debug_view(vg._abi.DEBUG_NEIGHBORS).reshape(-1, spec.num_particles)
        filled = nb != 0xFFFFFFFF
        # entries before each column's terminator (a full list has none)
        first_empty = np.where(filled.all(0), nb.shape[0], np.argmin(filled, axis=0))
        total += int(first_empty.sum())
        count += spec.num_particles
    return total / count if count else None


# DRAM traffic of one plain k_grid_iter launch on the 512-cloth mix (fast build, 15x15 x4):
# ncu dram__bytes_read.sum + dram__bytes_write.sum = 330.89 + 91.80 MB over 6,865,422
# particles (the mix's arrays exceed L2, so the written positions reach DRAM too); other
# grid workloads are scaled from it by the particles a launch covers.
GRID_ITER_DRAM_BYTES_PER_PARTICLE = (330.8864e6 + 91.799552e6) / 6865422
GRID_ITER_DRAM_SOURCE_PARTICLES = 6865422


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int = 0, pci_bus_id: str | None = None):
        self.rows: list[list[str]] = []
        sel = ["-i", pci_bus_id] if pci_bus_id else ["-i", str(device_index)]
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", *sel], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 8 for k in range(4)
                          if r[4 + k].lower() == "active"})
        pw = [float(r[2]) for r in self.rows if len(r) >= 8 and r[2].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm), "power_w_max": max(pw) if pw else None}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------- oracle legs
def _oracle_worker(args):
    """Runs `frames` frames of the given cloths on the CPU oracle; returns (pits, seconds)."""
    idx, wl_name, seed, frames = args
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle import Oracle
    from velvet_gb300 import workloads as W

    wl = workload(wl_name, seed)
    pits, secs = 0, 0.0
    for i in idx:
        spec = wl.cloths[i]
        o = Oracle()
        W.build_plain(spec, o)
        d = spec.particle_diameter()
        t0 = time.perf_counter()
        for f in range(frames):
            o.update_colliders(spec.colliders(f))
            o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, d)
        secs += time.perf_counter() - t0
        pits += spec.num_particles * wl.substeps * wl.iterations * frames
        o.close()
    return pits, secs


def sample_indices(wl, budget_particles: int) -> list[int]:
    """Every k-th cloth, preserving the size distribution, up to ~budget particles."""
    n = len(wl.cloths)
    total = sum(c.num_particles for c in wl.cloths)
    k = max(1, int(math.ceil(total / max(1, budget_particles))))
    return list(range(0, n, k))


def cpu_baseline_single(wl_name: str, seed: int, budget_s: float = 15.0) -> dict:
    """The oracle on one core over a bounded sample of the workload."""
    wl = workload(wl_name, seed)
    idx = sample_indices(wl, 250_000)
    pits, secs = _oracle_worker((idx, wl_name, seed, 1))
    frames = max(1, min(4, int(budget_s / max(secs, 1e-3))))
    if frames > 1:
        p2, s2 = _oracle_worker((idx, wl_name, seed, frames))
        pits, secs = p2, s2
    return {"value": pits / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{len(idx)} of {len(wl.cloths)} cloths (every {len(wl.cloths) // max(1, len(idx))}th), "
                      f"{frames} frame(s), {pits / 1e6:.1f} M particle-iterations in {secs:.1f} s"}


def cpu_reference_solver_single(budget_s: float = 8.0) -> dict:
    """The reference's own CPU solver (VtClothSolverCPU, restated in oracle/vt_cpu_solver.c:
    a different, Gauss-Seidel algorithm) on one core, on its own CPU configuration: one
    64x64 cloth, 5 substeps x 10 iterations."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle import CpuSolver
    from velvet_gb300 import workloads as W

    wl = W.small()
    s = CpuSolver(wl.cloths[0])
    frames, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s and frames < 300:
        s.simulate(float(W.FRAME_DT), wl.substeps, wl.iterations)
        frames += 1
    secs = time.perf_counter() - t0
    s.close()
    pits = wl.num_particles * wl.substeps * wl.iterations * frames
    return {"value": pits / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"VtClothSolverCPU restated: 64x64 cloth, {frames} frames in {secs:.1f} s"}


def _cpu_solver_worker(args):
    """VtClothSolverCPU (restated) on the given cloths of a workload, `frames` frames each;
    returns (pits, seconds)."""
    idx, wl_name, seed, frames = args
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle import CpuSolver

    wl = workload(wl_name, seed)
    pits, secs = 0, 0.0
    for i in idx:
        spec = wl.cloths[i]
        s = CpuSolver(spec)
        t0 = time.perf_counter()
        for _ in range(frames):
            s.simulate(wl.frame_dt, wl.substeps, wl.iterations)
        secs += time.perf_counter() - t0
        pits += spec.num_particles * wl.substeps * wl.iterations * frames
        s.close()
    return pits, secs


def cpu_reference_solver_all_cores(wl_name: str, seed: int) -> dict:
    """VtClothSolverCPU on every host core, one independent cloth at a time per process,
    over a size-preserving sample of the workload (cloths are independent, so the cores
    share nothing): aggregate particle-iterations / wall time."""
    import multiprocessing as mp

    sys.path.insert(0, str(ROOT / "tests"))
    import oracle

    oracle.cpu_solver_lib()  # build once here, before the workers load it
    wl = workload(wl_name, seed)
    cores = os.cpu_count() or 1
    idx = sample_indices(wl, 150_000 * cores)
    chunks = [c for c in (idx[k::cores] for k in range(cores)) if c]
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(chunks)) as pool:
        t0 = time.perf_counter()
        res = pool.map(_cpu_solver_worker, [(c, wl_name, seed, 2) for c in chunks])
        wall = time.perf_counter() - t0
    pits = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    return {"value": pits / busy, "unit": UNIT, "cores": len(chunks), "kind": "port",
            "sample": f"VtClothSolverCPU restated: {len(idx)} of {len(wl.cloths)} cloths, 2 frames each, "
                      f"{len(chunks)} processes, {pits / 1e6:.1f} M particle-iterations, slowest process "
                      f"{busy:.1f} s of simulation ({wall:.1f} s with process start-up)"}


def host_info() -> dict:
    """Core count and CPU model of the host the bench ran on."""
    model = platform.processor() or platform.machine()
    try:
        fields: dict[str, str] = {}
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if ":" in line:
                k, v = line.split(":", 1)
                fields.setdefault(k.strip().lower(), v.strip())
        if "model name" in fields:
            model = fields["model name"]
        elif "cpu part" in fields:  # Arm: implementer / part codes (0x41 / 0xd4f = Arm Neoverse V2)
            model = f"Arm implementer {fields.get('cpu implementer', '?')} part {fields['cpu part']}"
    except OSError:
        pass
    return {"nproc": os.cpu_count(), "cpu_model": model, "machine": platform.machine()}


def run_reference(args) -> None:
    rank, world, _ = env_rank()
    if rank != 0:
        return
    import multiprocessing as mp

    sys.path.insert(0, str(ROOT / "tests"))
    import oracle

    oracle.lib()  # build once here, before the workers load it
    wl = workload(args.workload, args.seed)
    cores = os.cpu_count() or 1
    idx = sample_indices(wl, 400_000 * max(1, cores // 4))
    chunks = [idx[k::cores] for k in range(cores)]
    chunks = [c for c in chunks if c]
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(chunks)) as pool:
        step_times, step_pits = [], []
        for s in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_oracle_worker, [(c, args.workload, args.seed, 1) for c in chunks])
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                step_times.append(dt)
                step_pits.append(sum(r[0] for r in res))
    value = sum(step_pits) / sum(step_times)
    sample = (f"{len(idx)} of {len(wl.cloths)} cloths (size distribution kept), one frame per step "
              f"on {len(chunks)} processes")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * statistics.mean(step_times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic grid cloths (seeded), CPU restatement of the reference GPU solver "
                "(bit-identical to the reference's own kernels run on the CPU)",
        "config": {"workload": wl.name, "cloths_sampled": len(idx), "substeps": wl.substeps,
                   "iterations": wl.iterations},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": len(chunks), "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------- GPU arm
# --csr-kernels: grid cloths solved by the general CSR kernels (k_bend + k_solve) instead
# of the implicit-topology tile kernel (same results; for profiling that path)
CSR_KERNELS = False


def new_solver(spec):
    import velvet_gb300 as vg
    from velvet_gb300 import workloads as W

    s = vg.ClothSolver()
    W.build_plain(spec, s)
    if CSR_KERNELS:
        vg._abi.check(vg.lib().vt_solver_use_grid_kernel(s.handle, 0), "vt_solver_use_grid_kernel")
    return s


def build_plain_solvers(wl, graphs=True):
    import velvet_gb300 as vg

    solvers = []
    for spec in wl.cloths:
        s = new_solver(spec)
        vg._abi.check(vg.lib().vt_solver_use_graphs(s.handle, 1 if graphs else 0), "vt_solver_use_graphs")
        solvers.append((s, spec, spec.particle_diameter()))
    return solvers


def build_batch(wl):
    import velvet_gb300 as vg

    batch = vg.BatchSolver()
    for spec in wl.cloths:
        s = new_solver(spec)
        batch.add(s)
        s.close()
    return batch


def plain_frame(wl, solvers, frame, stream, upload_colliders):
    for s, spec, d in solvers:
        if upload_colliders:
            s.update_colliders(spec.colliders(frame))
        s.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                   wl.collision_margin, d, stream)


def batch_frame(wl, batch, frame, stream, upload_colliders):
    if upload_colliders:
        for k, spec in enumerate(wl.cloths):
            batch.update_colliders(k, spec.colliders(frame))
    batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                   wl.collision_margin, None, stream)


def launch_total(solvers) -> int:
    import ctypes as C

    import velvet_gb300 as vg

    tot = 0
    for s, _, _ in solvers:
        v = C.c_uint64()
        vg._abi.check(vg.lib().vt_solver_launch_count(s.handle, C.byref(v)), "vt_solver_launch_count")
        tot += v.value
    return tot


def profile_frames(args) -> None:
    """Builds the workload and runs `--profile-frames` frames on the default stream:
    the command ncu captures (nothing else launches kernels)."""
    import torch

    wl = workload(args.workload, args.seed)
    if args.form == "plain":
        solvers = build_plain_solvers(wl, graphs=False)
        for f in range(args.profile_frames):
            plain_frame(wl, solvers, f, None, upload_colliders=False)
        for s, _, _ in solvers:
            s.sync()
    else:
        batch = build_batch(wl)
        batch.use_graphs(False)
        for f in range(args.profile_frames):
            batch_frame(wl, batch, f, None, upload_colliders=False)
        batch.sync()
    torch.cuda.synchronize()
    print(json.dumps({"profiled_frames": args.profile_frames, "workload": wl.name, "form": args.form,
                      "particles": wl.num_particles}))


def timed_device(step_fn, steps, warmup, stream, dist_sync):
    import torch

    for f in range(warmup):
        step_fn(f)
    torch.cuda.synchronize()
    dist_sync()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    for k in range(steps):
        step_fn(warmup + k)
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    dist_sync()
    per = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
    return ev[0].elapsed_time(ev[steps]), per


def pct(v, q):
    s = sorted(v)
    return s[min(len(s) - 1, int(q * len(s)))]


def serving_legs(args, duration: float, plain_seconds: float) -> tuple[dict, dict]:
    """Served form: Poisson arrivals (args.rate req/s for `duration` s), each request one
    grid cloth with side log-uniform in [16, 512] and a frame count uniform in [30, 300],
    admitted by the HBM budget (--budget-gb) and an active-particle cap, one frame for all
    active requests per tick.  Requests wait in a front-end backlog and enter the
    server's queue as it drains.  Returns the served leg (aggregate particle-iterations/s
    over the wall time, p50/p99 frame latency, request latency from arrival to admission
    and to completion) and the plain solver run one request at a time on the same
    arrival stream for `plain_seconds`.  Both legs are timed alike: registration of a
    request's cloth on the host is outside both timed regions (the served leg's payloads
    are built before its loop; the plain leg's registration time is measured and taken
    out), and neither leg synchronises per frame (the plain leg records an event pair per
    frame and reads them once per request)."""
    import torch

    import velvet_gb300 as vg
    from velvet_gb300 import workloads as W

    rng = np.random.default_rng(args.seed)
    n_req = int(args.rate * duration * 1.5) + 16
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, n_req))
    sides = np.rint(np.exp(rng.uniform(math.log(16), math.log(512), n_req))).astype(int)
    frames = rng.integers(30, 301, n_req)
    S, It = 5, 10
    templates: dict[int, object] = {}

    def spec_of(side):
        return W.ClothSpec(side, 0.02, W.horizontal_cloth(side, 0.02, 0.8), [0, side - 1],
                           W.static_colliders([W.sphere((0.0, 0.3, 0.0), 0.3), W.plane(0.0)]))

    def template(side):
        if side not in templates:
            spec = spec_of(side)
            s = vg.ClothSolver()
            W.build_plain(spec, s)
            templates[side] = (s, spec)
        return templates[side]

    described: dict[int, tuple] = {}

    def submit(srv, side, frames):
        if args.described:  # the cloth is described; the server builds it on the device
            if side not in described:
                spec = spec_of(side)
                described[side] = (spec, spec.particle_diameter(), spec.colliders(0))
            spec, d, cols = described[side]
            return srv.submit_grid(spec.resolution, spec.spacing * spec.resolution, spec.model, d,
                                   spec.attached, cols, frames)
        s, _ = template(side)
        return srv.submit(s, frames)

    # registered requests arrive with their cloth already registered (the client's
    # work): build the payload of every size that can arrive before the timed loop
    tb = time.perf_counter()
    if not args.described:
        for side in sorted(set(int(v) for v in sides[: int(args.rate * duration * 1.2) + 16])):
            template(side)
    build_s = time.perf_counter() - tb
    stream = torch.cuda.Stream()
    srv = vg.ClothServer(int(args.budget_gb * (1 << 30)), max_cloths=4096,
                         max_active_particles=args.max_active_particles, substeps=S, iterations=It)
    # warm-up: one small request through the whole path
    submit(srv, 16, 3)
    while srv.tick(stream).active or srv.stats().requests_done < 1:
        pass
    base = srv.stats()
    k = 0
    backlog: list[int] = []
    ticks, admitted, active_samples = 0, 0, []
    outstanding: dict[int, int] = {}  # request id -> arrival index
    t_admit, t_done = {}, {}
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        if now >= duration:
            break
        while k < n_req and arrivals[k] <= now:
            backlog.append(k)
            k += 1
        info_q = 0
        while backlog and info_q < 2:
            j = backlog.pop(0)
            outstanding[submit(srv, int(sides[j]), int(frames[j]))] = j
            info_q += 1
        info = srv.tick(stream)
        ticks += 1
        admitted += info.admitted
        active_samples.append(info.active_particles)
        now = time.perf_counter() - t0
        for rid in list(outstanding):
            state, _ = srv.poll(rid)
            j = outstanding[rid]
            if state != 0 and j not in t_admit:  # left the queue
                t_admit[j] = now
            if state >= 2:  # done, failed or cancelled
                t_done[j] = now
                del outstanding[rid]
    wall = time.perf_counter() - t0
    st = srv.stats()
    pits = st.particle_iterations - base.particle_iterations
    wait = [t_admit[j] - arrivals[j] for j in t_admit]
    resp = [t_done[j] - arrivals[j] for j in t_done]
    served = {"value": pits / wall, "unit": UNIT, "wall_s": wall, "ticks": ticks,
              "p50_frame_ms": st.p50_frame_ms, "p99_frame_ms": st.p99_frame_ms,
              "frame_latency": "event-timed GPU time of the tick's frame, weighted by its requests",
              "arrived": k, "admitted": admitted, "completed": int(st.requests_done - base.requests_done),
              "backlog_at_end": len(backlog),
              "request_wait_s": {"p50": statistics.median(wait) if wait else None,
                                 "p99": pct(wait, 0.99) if wait else None,
                                 "what": "arrival to admission (queueing; the stream asks for more than one "
                                         "GPU sustains, so the backlog grows through the run)"},
              "request_latency_s": {"p50": statistics.median(resp) if resp else None,
                                    "p99": pct(resp, 0.99) if resp else None, "what": "arrival to last frame"},
              "mean_active_particles": float(np.mean(active_samples)) if active_samples else 0.0,
              "gpu_busy_frac": (st.gpu_ms - base.gpu_ms) / 1000.0 / wall,
              "payload_build_s_untimed": build_s, "distinct_sizes": len(templates) or len(described),
              "submission": "described grid cloths, built on the device at admission" if args.described
              else "registered solvers (host-built constraint arrays)"}
    srv.close()
    for s, _ in templates.values():
        s.close()

    # the plain solver, one request at a time, same stream of requests, bounded time;
    # host registration of each request is measured and taken out of the wall time
    p_pits, p_frames, reg_s = 0, [], 0.0
    pool = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(301)]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    j = 0
    while time.perf_counter() - t1 - reg_s < plain_seconds and j < n_req:
        tr = time.perf_counter()
        spec = spec_of(int(sides[j]))
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        d = spec.particle_diameter()
        reg_s += time.perf_counter() - tr
        nf = int(frames[j])
        for f in range(nf):
            pool[f][0].record(stream)
            s.simulate(float(W.FRAME_DT), S, It, 1.0, 0.1, 0.06, d, stream)
            pool[f][1].record(stream)
            p_pits += spec.num_particles * S * It
        pool[nf - 1][1].synchronize()
        p_frames.extend(pool[f][0].elapsed_time(pool[f][1]) for f in range(nf))
        s.close()
        j += 1
    p_wall = time.perf_counter() - t1 - reg_s
    plain = {"value": p_pits / p_wall, "unit": UNIT, "wall_s": p_wall, "requests": j,
             "registration_s_excluded": reg_s,
             "p50_frame_ms": statistics.median(p_frames), "p99_frame_ms": pct(p_frames, 0.99)}
    return served, plain


def served_mix_leg(args, wl, plain_value: float | None) -> dict:
    """The served form on the mixed-size workload itself: every cloth of the mix arrives at
    once as a request of --served-mix-frames frames (registered beforehand, untimed), the
    server admits them under its budget and active-particle cap and runs them by continuous
    batching until the last one finishes.  Reports particle-iterations/s over the wall
    time, the frame latency distribution and the ratio to the plain solver on the same
    mix."""
    import torch

    import velvet_gb300 as vg

    frames = args.served_mix_frames
    S, It = wl.substeps, wl.iterations
    solvers = [new_solver(spec) for spec in wl.cloths]
    stream = torch.cuda.Stream()
    srv = vg.ClothServer(int(args.budget_gb * (1 << 30)), max_cloths=2 * len(wl.cloths),
                         max_active_particles=args.max_active_particles, substeps=S, iterations=It)
    # warm-up: one small cloth through the whole path
    srv.submit(solvers[0], 2)
    while srv.tick(stream).active or srv.stats().requests_done < 1:
        pass
    base = srv.stats()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ids = [srv.submit(s, frames) for s in solvers]
    ticks = 0
    while True:
        info = srv.tick(stream)
        ticks += 1
        if info.active == 0 and info.queued == 0:
            break
    wall = time.perf_counter() - t0
    st = srv.stats()
    done = sum(1 for r in ids if srv.poll(r)[0] == 2)
    pits = st.particle_iterations - base.particle_iterations
    out = {"value": pits / wall, "unit": UNIT, "wall_s": wall, "ticks": ticks, "requests": len(ids),
           "completed": done, "frames_per_request": frames,
           "p50_frame_ms": st.p50_frame_ms, "p99_frame_ms": st.p99_frame_ms,
           "max_active_particles": args.max_active_particles,
           "what": "every cloth of the mix submitted at once (registered, untimed), admitted under the cap, "
                   "run to completion by continuous batching; frame latency = a tick's event-timed GPU time, "
                   "weighted by its requests"}
    if plain_value:
        out["over_plain"] = out["value"] / plain_value
    srv.close()
    for s in solvers:
        s.close()
    return out


def run_serving(args) -> None:
    """--workload serving: the served and plain legs for --duration / --plain-seconds."""
    import torch

    torch.cuda.set_device(0)
    served, plain = serving_legs(args, args.duration, args.plain_seconds)
    S, It = 5, 10
    line = {"metric": METRIC, "value": served["value"], "unit": UNIT, "n_gpus": 1, "steps": served["ticks"],
            "warmup": 1, "ms_per_step": 1000 * served["wall_s"] / max(1, served["ticks"]), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic Poisson request stream, seed {args.seed}",
            "config": {"workload": "serving", "rate_per_s": args.rate, "duration_s": args.duration,
                       "side": "log-uniform [16, 512]", "frames": "uniform [30, 300]",
                       "budget_gb": args.budget_gb, "max_active_particles": args.max_active_particles,
                       "substeps": S, "iterations": It, "library": os.environ.get("VT_VARIANT", "exact")},
            "served": served, "plain": plain, "served_over_plain": served["value"] / plain["value"],
            "p50_frame_ms": served["p50_frame_ms"], "p99_frame_ms": served["p99_frame_ms"]}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="batched")
    ap.add_argument("--form", choices=["batched", "plain"], default="batched",
                    help="form run by --profile-frames")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--csr-kernels", action="store_true",
                    help="solve grid cloths with the general CSR kernels instead of the tile kernel")
    ap.add_argument("--grid-tile", type=int, default=-1,
                    help="pin a grid kernel variant (velvet_gb300.GRID_VARIANTS index); -1 = autotune")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain solver")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="only run this many frames of the workload and exit (for ncu captures)")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serving: seconds of arrivals")
    ap.add_argument("--described", action="store_true",
                    help="serving: submit grid cloths by description (built on the device)")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="serving: device-memory budget")
    ap.add_argument("--max-active-particles", type=int, default=3_500_000,
                    help="serving: admission stops above this many active particles")
    ap.add_argument("--plain-seconds", type=float, default=15.0,
                    help="serving: seconds of the one-request-at-a-time plain comparison")
    ap.add_argument("--variant", choices=["fast", "exact"], default="fast",
                    help="library build: fast (contracted arithmetic, within the stated tolerance of the "
                         "oracle) or exact (bit-identical to the oracle)")
    ap.add_argument("--served-seconds", type=float, default=12.0,
                    help="batched run: seconds of the served leg (Poisson stream at --rate)")
    ap.add_argument("--served-plain-seconds", type=float, default=8.0,
                    help="batched run: seconds of the served leg's plain comparison")
    ap.add_argument("--no-served", action="store_true", help="skip the served legs")
    ap.add_argument("--served-mix-frames", type=int, default=6,
                    help="frames per request when the served form runs the mixed-size workload")
    ap.add_argument("--tile-loads", choices=["tma", "cp_async"], default="cp_async",
                    help="how the grid kernel stages its tiles (same results)")
    ap.add_argument("--substep-clusters", choices=["on", "restaging", "off"], default="on",
                    help="small grid cloths: a substep's iterations as one launch of thread-block clusters "
                         "(on: positions resident in shared memory where cloths fit 64x64; restaging: "
                         "tiles re-read from global memory each iteration)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end legs")
    ap.add_argument("--no-exact-build", action="store_true",
                    help="skip timing the exact build beside the fast one")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    os.environ["VT_VARIANT"] = args.variant  # read when velvet_gb300 is first imported
    if args.impl == "reference":
        run_reference(args)
        return
    global CSR_KERNELS
    CSR_KERNELS = args.csr_kernels
    if args.grid_tile >= 0:
        import velvet_gb300 as vg

        vg._abi.check(vg.lib().vt_tuning_set_grid_tile(args.grid_tile), "vt_tuning_set_grid_tile")
    if args.tile_loads == "tma":
        import velvet_gb300 as vg

        vg._abi.check(vg.lib().vt_tuning_set_tile_loads(1), "vt_tuning_set_tile_loads")
    if args.substep_clusters != "on":
        import velvet_gb300 as vg

        mode = {"off": 0, "restaging": 2}[args.substep_clusters]
        vg._abi.check(vg.lib().vt_tuning_set_substep_clusters(mode), "vt_tuning_set_substep_clusters")
    if args.profile_frames:
        profile_frames(args)
        return
    if args.workload == "serving":
        run_serving(args)
        return

    import torch

    import velvet_gb300 as vg
    from velvet_gb300 import _abi

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def dist_sync():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        t = torch.tensor([x], device="cuda", dtype=torch.float64)
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def sum_over_ranks(x: float) -> float:
        t = torch.tensor([x], device="cuda", dtype=torch.float64)
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())

    # weak scaling: every rank simulates its own mix of cloths (seed + rank)
    wl = workload(args.workload, args.seed + rank)
    stream = torch.cuda.Stream()
    pits = pits_per_frame(wl)
    job_pits = sum_over_ranks(pits)  # every rank's cloths differ (seed + rank)
    n_tot = wl.num_particles
    props = torch.cuda.get_device_properties(local)
    bus = getattr(props, "pci_bus_id", None)
    pci = None
    if bus is not None:
        pci = f"{getattr(props, 'pci_domain_id', 0):08x}:{bus:02x}:{getattr(props, 'pci_device_id', 0):02x}.0"

    # ---- batched form: every cloth advanced by one CUDA graph launch per frame
    batch = build_batch(wl)
    bstep = lambda f: batch_frame(wl, batch, f, stream, upload_colliders=False)  # noqa: E731
    for f in range(args.warmup):
        bstep(f)
    torch.cuda.synchronize()
    l0 = batch.launch_count()
    clocks = ClockSampler(local, pci)
    total_ms, per = timed_device(bstep, args.steps, 0, stream, dist_sync)
    clock_info = clocks.stop()
    launches_timed = batch.launch_count() - l0
    total_ms = max_over_ranks(total_ms)
    value = job_pits * args.steps / (total_ms / 1000.0)

    # ---- roofline of the dominant stage: one Jacobi iteration (bend + solve), events
    # around each launch on the launching stream (graphs off while profiling)
    _abi.profiler_reset()
    _abi.profiler_enable(True)
    for k in range(2):
        bstep(args.warmup + args.steps + k)
    torch.cuda.synchronize()
    prof = _abi.profiler_read()
    _abi.profiler_enable(False)
    solve, bend = prof.get("solve", (0, 0.0)), prof.get("bend", (0, 0.0))
    grid_it = prof.get("grid_iter", (0, 0.0))
    roofline = None
    peak, peak_kind = measured_peak_hbm()
    iters = 2 * wl.substeps * wl.iterations
    t_iter_ms = (solve[1] + bend[1] + grid_it[1]) / iters if (solve[0] or grid_it[0]) else 0.0
    if t_iter_ms > 0:
        ach = iteration_bytes(wl) / (t_iter_ms / 1000.0) / 1e9
        grid_only = grid_it[0] and not solve[0]
        kern = "k_grid_iter" if grid_only else "k_bend + k_solve"
        traffic = GRID_ITER_DRAM_BYTES_PER_PARTICLE * n_tot if grid_only else None
        roofline = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                    "traffic": traffic,
                    "traffic_source": (("ncu on batched_512: dram__bytes_read.sum + dram__bytes_write.sum of one "
                                        "plain k_grid_iter launch" if n_tot == GRID_ITER_DRAM_SOURCE_PARTICLES else
                                        "ncu on batched_512, scaled by particles") if traffic else None),
                    "kernel": f"{kern}: one Jacobi iteration over all cloths",
                    "algorithmic_bytes_per_launch": iteration_bytes(wl),
                    "avg_iteration_ms": t_iter_ms, "peak_source": f"{peak_kind} hbm_gbs",
                    "stage_ms_per_frame": {k: round(v[1] / 2, 4) for k, v in prof.items()}}
        lra = lra_roofline(wl, t_iter_ms, clock_info)
        if lra is not None:
            roofline["lra"] = lra

    grid_tile = vg.grid_variant_name(batch.grid_tile())
    batch.close()

    # ---- end to end through the C ABI: colliders from host memory every frame, all
    # positions + normals read back into pinned host memory every frame.  Synchronous
    # form: each step waits for its own read-back.  Pipelined form (the headline): frame
    # k+1 is enqueued while frame k's read-back copies run on a second stream, the host
    # waits for frame k's copies before enqueuing frame k+2, and every copy completes
    # inside the timed region.  Each form runs on a freshly built batch over the same
    # frames as the device-resident loop (the cost of a frame changes as the cloths fall
    # onto their colliders), so the forms differ only in how the host drives them.
    e2e = None
    if not args.no_e2e:
        host_pos = [torch.empty((n_tot, 3), dtype=torch.float32, pin_memory=True) for _ in range(2)]
        host_nrm = [torch.empty((n_tot, 3), dtype=torch.float32, pin_memory=True) for _ in range(2)]
        sh = vg.stream_handle(stream)
        copy_stream = torch.cuda.Stream()
        ch = vg.stream_handle(copy_stream)
        copied = [torch.cuda.Event(), torch.cuda.Event()]

        def e2e_step(b, f):
            batch_frame(wl, b, f, stream, upload_colliders=True)
            _abi.check(vg.lib().vt_batch_all_get(b.handle, 0, host_pos[0].data_ptr(), 1, sh), "all_get")
            _abi.check(vg.lib().vt_batch_all_get(b.handle, 1, host_nrm[0].data_ptr(), 1, sh), "all_get")
            stream.synchronize()

        host_enqueue_s = [0.0]

        def e2e_pipelined(b, f):
            t = time.perf_counter()
            batch_frame(wl, b, f, stream, upload_colliders=True)
            _abi.check(vg.lib().vt_batch_all_get_async(b.handle, 0, host_pos[f % 2].data_ptr(), ch), "all_get_async")
            _abi.check(vg.lib().vt_batch_all_get_async(b.handle, 1, host_nrm[f % 2].data_ptr(), ch), "all_get_async")
            copied[f % 2].record(copy_stream)
            host_enqueue_s[0] += time.perf_counter() - t
            if f > 0:
                copied[(f - 1) % 2].synchronize()  # frame f-1 is in host memory

        e2e_steps = args.steps
        batch = build_batch(wl)
        for f in range(args.warmup):
            e2e_step(batch, f)
        dist_sync()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            e2e_step(batch, args.warmup + k)
        e2e_sync_s = max_over_ranks(time.perf_counter() - t0)
        batch.close()
        batch = build_batch(wl)
        for f in range(args.warmup):
            e2e_pipelined(batch, f)
        copy_stream.synchronize()
        dist_sync()
        host_enqueue_s[0] = 0.0
        e_first, e_last = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e2e_clocks = ClockSampler(local, pci)
        t0 = time.perf_counter()
        e_first.record(stream)
        for k in range(e2e_steps):
            e2e_pipelined(batch, args.warmup + k)
        e_last.record(stream)
        copy_stream.synchronize()
        stream.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
        e2e_clock_info = e2e_clocks.stop()
        e2e_device_ms = e_first.elapsed_time(e_last) / e2e_steps
        e2e_value = job_pits * e2e_steps / e2e_s
        e2e_sync_value = job_pits * e2e_steps / e2e_sync_s
        ncol = sum(len(c.colliders(0)) for c in wl.cloths)
        h2d = ncol * 208 + len(wl.cloths) * 128  # collider blocks + per-cloth parameter blocks
        d2h = n_tot * 24
        batch.close()
        e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "mode": "pipelined: frame k+1 computes while frame k's positions and normals copy to pinned "
                       "host memory (vt_batch_all_get_async); all copies inside the timed region",
               "synchronous_value": e2e_sync_value, "steps": e2e_steps,
               "wall_ms_per_frame": 1000.0 * e2e_s / e2e_steps,
               "device_ms_per_frame": e2e_device_ms,
               "host_enqueue_ms_per_frame": 1000.0 * host_enqueue_s[0] / e2e_steps,
               "clocks": e2e_clock_info}

    # ---- the plain drop-in solver on the same workload, one cloth at a time
    plain = None
    if not args.no_plain:
        solvers = build_plain_solvers(wl)
        pstep = lambda f: plain_frame(wl, solvers, f, stream, upload_colliders=False)  # noqa: E731
        psteps = max(3, args.steps // 4)
        p_ms, p_per = timed_device(pstep, psteps, args.warmup, stream, dist_sync)
        p_ms = max_over_ranks(p_ms)
        plain = {"value": job_pits * psteps / (p_ms / 1000.0), "unit": UNIT, "steps": psteps,
                 "ms_per_step": p_ms / psteps, "p50_frame_ms": statistics.median(p_per),
                 "p99_frame_ms": pct(p_per, 0.99), "form": "one vt_simulate per cloth per frame, CUDA graphs"}
        k_mean = mean_cached_neighbours(solvers)
        if roofline is not None and k_mean is not None:
            fb = frame_bytes(wl, k_mean)
            ach = fb / (total_ms / args.steps / 1000.0) / 1e9
            roofline["frame"] = {"bytes_per_particle_iteration": fb / pits, "k_mean_measured": k_mean,
                                 "bytes_per_frame": fb, "achieved": ach, "frac": ach / peak,
                                 "model": "per-frame compulsory bytes (iterations + predict, SDF, collide, "
                                          "finalize, hash, normals) / event-timed frame"}
        for s, _, _ in solvers:
            s.close()

    # the served form on the mixed-size workload itself, against the plain solver on it
    served_mix = None
    if rank == 0 and world == 1 and not args.no_served:
        served_mix = served_mix_leg(args, wl, plain["value"] if plain else None)

    # the served form on a bounded Poisson stream, and its plain comparison (one GPU)
    served = None
    if rank == 0 and world == 1 and not args.no_served:
        sv, sp = serving_legs(args, args.served_seconds, args.served_plain_seconds)
        served = {**sv, "plain": sp, "served_over_plain": sv["value"] / sp["value"],
                  "config": {"rate_per_s": args.rate, "duration_s": args.served_seconds,
                             "side": "log-uniform [16, 512]", "frames": "uniform [30, 300]",
                             "budget_gb": args.budget_gb, "max_active_particles": args.max_active_particles}}

    # the exact build (bit-identical to the oracle) on the same batched frames, in a child
    # process (the library is chosen per process)
    exact = None
    if rank == 0 and world == 1 and args.variant == "fast" and not args.no_exact_build:
        r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--variant", "exact", "--workload", args.workload,
                            "--steps", str(args.steps), "--warmup", str(args.warmup), "--no-plain",
                            "--no-cpu-baseline", "--no-served", "--no-e2e", "--seed", str(args.seed)]
                           + (["--grid-tile", str(args.grid_tile)] if args.grid_tile >= 0 else []),
                           capture_output=True, text=True, timeout=900)
        try:
            ex = json.loads(r.stdout.strip().splitlines()[-1])
            exact = {"value": ex["value"], "ms_per_step": ex["ms_per_step"], "p99_frame_ms": ex["p99_frame_ms"],
                     "roofline_frac": (ex.get("roofline") or {}).get("frac"),
                     "avg_iteration_ms": (ex.get("roofline") or {}).get("avg_iteration_ms"),
                     "what": "libvelvet_gb300.so: bit-identical to the oracle (no contraction, IEEE division "
                             "and square root)"}
        except (ValueError, IndexError, KeyError):
            exact = {"error": (r.stdout[-300:] + r.stderr[-300:])}

    # the CPU legs run once, at one GPU: at N > 1 the other ranks' GPUs would wait on them
    cpu, cpu_ref_solver, cpu_ref_solver_all = None, None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_single(args.workload, args.seed)
        cpu_ref_solver = cpu_reference_solver_single()
        cpu_ref_solver_all = cpu_reference_solver_all_cores(args.workload, args.seed)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic grid cloths generated from the config (seeded), no dataset",
            "config": {"workload": wl.name, "form": "batched (one graph launch per frame for all cloths)",
                       "library": f"libvelvet_gb300{'_fast' if args.variant == 'fast' else ''}.so",
                       "tile_loads": args.tile_loads, "substep_clusters": args.substep_clusters,
                       "cloths_per_gpu": len(wl.cloths), "particles_per_gpu": n_tot,
                       "substeps": wl.substeps, "iterations": wl.iterations,
                       "grid_tile": None if CSR_KERNELS else grid_tile,
                       "kernels": "CSR (k_bend + k_solve)" if CSR_KERNELS else "grid tile (k_grid_iter)",
                       "l2": "inputs larger than L2 (working set ~%.1f GB)" % (n_tot * 500 / 1e9),
                       "parallelism": f"independent cloths per GPU x {world} GPU(s)"},
            "p50_frame_ms": statistics.median(per), "p99_frame_ms": pct(per, 0.99),
            "plain": plain,
            "batched_over_plain": (value / plain["value"]) if plain else None,
            "clocks": clock_info,
            "e2e": e2e,
            "gpu_launches": launches_timed,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "cpu_reference_cpu_solver": cpu_ref_solver,
            "cpu_reference_cpu_solver_all_cores": cpu_ref_solver_all,
            "served_mix": served_mix,
            "served": served,
            "exact_build": exact,
            "host": host_info(),
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
