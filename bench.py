#!/usr/bin/env python
"""Benchmark of the PCISPH particle step on GB300 (one JSON line on rank 0).

Workload: the 1,048,576-particle PCISPH dam break (128 x 64 x 128 cubic lattice at
spacing 0.008, +-0.1 spacing jitter, 2 x 1 x 1.2 box), FP32 state, tolerance-mode
corrector (max density error < 1 % of rho0, at most 20 iterations), substep dt at the
CFL speed limit of scale 5, 1,000 substeps.  A step is one substep: grid rebuild,
density, non-pressure force, the corrector to tolerance, integration with colliders.
The first `--prep` (200) substeps run the plain corrector; the learned variant trains
its warm-start MLP online on their (features, converged pressure) pairs.  After
`--warmup` more substeps the timed window covers the remaining `--steps` substeps.

  value      particle-updates/s over the timed substeps, inputs resident in HBM, L2
             flushed (256 MB write) between steps, CUDA events on the launching stream
  e2e        the same metric through the C ABI with host buffers: upload positions and
             velocities (and the carried pressure for warm starts) from pinned memory,
             one substep, download them, every step
  roofline   dominant kernel: algorithmic bytes per launch / its average duration
  kernel_bounds  every neighbour pass against its HBM bound and its issue-rate bound
             (warp instructions from the committed ncu summary / duration / issue slots)
  cpu_baseline  the CPU oracle (restatement of the reference's CPU path) on the box's
             host cores, on a bounded sample of the same workload
  config.plain_same_window  the plain (zero-start) corrector timed on the same substeps
             (as CUDA graphs, and in the reference's launch sequence: plain_host_loop_value)

`--impl reference` times the reference's CPU implementation of the path (the oracle
port, all host threads) on the same workload and prints the same line with
"impl": "reference".  Under torchrun every rank runs an independent replica of the
scene ("replicas only": the step has no exchange); rank 0 prints the aggregate.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-updates/s PCISPH 1M, learned+batched vs plain at ≤1% density err"
UNIT = "particle-updates/s"
L2_FLUSH_BYTES = 256 << 20

# Algorithmic (compulsory) HBM bytes per particle per launch: every FP32 SoA array a
# kernel reads or writes counted once; neighbour re-reads are served by L1/L2.
def alg_bytes(list_len):
    """Compulsory DRAM bytes per particle of each kernel: the particle's own fields read
    and written once, its member list (`list_len` 4-byte ids on average) read or written
    once; neighbours' fields are re-reads of data other threads already brought on chip
    (cell-sorted order) and are not counted."""
    L = 4.0 * list_len
    return {
        "k_hash_count": 16 + 4 + 4,                        # pos in; cell, arrival index out
        "k_place": 4 + 4 + 4 + 4 + 8,                      # cell, index, start, id in; (id, slot) out
        "k_rank_gather": 8 + 4 + 4 + 32 + 32 + 4 + 4 + 4 + 4 + 4,  # + pressure in, previous pressure out
        "k_density": 16 + 4 + 4 + 4 + 4 + 4 + L,          # pos, cell in; rho, 1/rho, vel.w, count, list out
        "k_non_pressure": 16 + 16 + 4 + 4 + 16 + 4 + 16 + 16 + L,  # pos, vel, cell, count, list; F, p, Fp, x* out
        "k_pred_density": 16 + 4 + 4 + 4 + 4 + 4 + 4 + 4 + L,     # x*, cell, count, list, p; p, rho*, err, pos.w
        "k_pressure_force": 16 + 16 + 4 + 4 + 16 + 16 + 16 + L,   # pos, vel, cell, count, list, F; Fp, x* out
        "k_sph_forces": 16 + 16 + 4 + 4 + 16 + 32 + L,
        "k_integrate": 16 + 16 + 16 + 32,
    }


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_profile_figures(workload_key, tag):
    """Per-particle figures of each kernel from the committed ncu summary: lines
    `<tag>: <kernel> <value>` (DRAM bytes per launch, warp instructions per launch)."""
    path = os.path.join(ROOT, "profiles", "%s_ncu.md" % workload_key)
    out = {}
    if os.path.exists(path):
        for line in open(path):
            parts = line.split()
            if len(parts) == 3 and parts[0] == tag + ":":
                out[parts[1]] = float(parts[2])
    return out


def load_traffic(workload_key):
    """Per-particle DRAM bytes per launch from the committed ncu summary."""
    return load_profile_figures(workload_key, "traffic_bytes_per_particle")


def kernel_bounds(prof, table, n, peak, inst_table, sm_count, sm_mhz):
    """Each neighbour pass against both of its bounds: algorithmic HBM bytes / duration as a
    fraction of the measured copy bandwidth, and warp instructions (ncu count per particle,
    scaled to the launch) / duration as a fraction of the SMs' issue rate (4 schedulers per
    SM, one warp instruction each per cycle, at the median SM clock sampled under load)."""
    out = {}
    for k, (ms, cnt) in prof.items():
        if k not in table or cnt == 0:
            continue
        avg_s = ms / cnt / 1e3
        e = {"avg_launch_us": avg_s * 1e6, "hbm_frac": table[k] * n / avg_s / 1e9 / peak}
        if k in inst_table and sm_mhz:
            e["issue_frac"] = inst_table[k] * n / avg_s / (sm_count * 4 * sm_mhz * 1e6)
        e["bound"] = "issue" if e.get("issue_frac", 0.0) > e["hbm_frac"] else "hbm"
        out[k] = e
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if s[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def aggregate(dist, units, seconds):
    """Whole-job throughput: units summed over ranks / the slowest rank's time."""
    if dist is None:
        return units / seconds, seconds, units
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([seconds], dtype=torch.float64, device=dev)
    u = torch.tensor([units], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return u.item() / t.item(), t.item(), u.item()


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_oracle_rate(scene, pos, vel, budget_s, threads, max_steps=50):
    """Time the CPU oracle on substeps of (scene, pos, vel) until `budget_s` (at least one)."""
    from oracle import oracle as O
    sim = O.OracleSim(scene, pos, vel, variant="f32", threads=threads)
    steps, iters, t = 0, 0, 0.0
    while steps < max_steps and (steps == 0 or t < budget_s):
        t0 = time.perf_counter()
        it, _ = sim.pcisph_substep(scene["dt"], scene["max_density_error_ratio"],
                                   scene["max_iterations"], O.PCISPH_TOLERANCE)
        t += time.perf_counter() - t0
        steps += 1
        iters += it
    sim.close()
    return len(pos) * steps / t, steps, iters, t


def slab(pos, block, depth):
    """The first `depth` z-layers of the lattice block (x fastest, then y, then z)."""
    nx, ny, nz = block
    return pos.reshape(nz, ny, nx, 3)[:depth].reshape(-1, 3)


def run_reference(args, scene, pos):
    """Reference arm: the oracle port of the reference CPU path, all host threads."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if scene.get("batch"):
        # the reference has no batching: it would run the scenes one after the other; the
        # sample is the median-size scene
        scene, sample, _, what = cpu_sample(scene, pos, None, 0)
    else:
        block = scene["block"]
        # size the per-step sample so the whole run stays within ~150 s of CPU time
        probe = slab(pos, block, 8)
        rate, _, _, _ = cpu_oracle_rate(scene, probe, None, 0.0, threads, max_steps=1)
        per_step_budget = 150.0 / max(1, args.prep + args.steps + args.warmup)
        depth = int(np.clip((per_step_budget * rate) / (block[0] * block[1]) // 8 * 8, 8, block[2]))
        sample = slab(pos, block, depth)
        what = "%d-layer slab of the dam-break block" % depth
    from oracle import oracle as O
    sim = O.OracleSim(scene, sample, None, variant="f32", threads=threads)
    for _ in range(args.prep + args.warmup):
        sim.pcisph_substep(scene["dt"], scene["max_density_error_ratio"], scene["max_iterations"],
                           O.PCISPH_TOLERANCE)
    t, iters = 0.0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        it, _ = sim.pcisph_substep(scene["dt"], scene["max_density_error_ratio"],
                                   scene["max_iterations"], O.PCISPH_TOLERANCE)
        t += time.perf_counter() - t0
        iters += it
    sim.close()
    value = len(sample) * args.steps / t
    desc = ("%s (%d particles), one tolerance-mode substep per step after %d preparation and "
            "%d warm-up substeps, %.2f corrector iterations per substep"
            % (what, len(sample), args.prep, args.warmup, iters / max(1, args.steps)))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": scene["workload"], "variant": "plain", "solver": "pcisph",
                   "tolerance": scene["max_density_error_ratio"],
                   "max_iterations": scene["max_iterations"], "dt": scene["dt"],
                   "parallelism": "cpu threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def make_solver(bb, scene, pos, device):
    """The solver of a configuration: one scene, or a batch of scenes (`pos` a list)."""
    if scene.get("batch"):
        return bb.BatchSolver(scene, scene["boxes"], pos, device=device)
    return bb.Solver(scene, pos=pos, device=device)


def one_scene(scene, pos, index):
    """Scene `index` of a batch as a single-scene configuration (its own container)."""
    lo, hi = scene["boxes"][index]
    ext = tuple(float(b - a) for a, b in zip(lo, hi))
    center = tuple(float(a + b) / 2 for a, b in zip(lo, hi))
    sc = dict(scene, domain_min=tuple(lo), domain_max=tuple(hi), batch=False,
              colliders=[{"type": "box", "size": ext, "center": center, "reverse": True}])
    return sc, pos[index]


def cpu_sample(scene, pos, vel, depth):
    """Bounded CPU sample: the first `depth` z-layers of the lattice block, or for a batch
    the scene whose size is the median of the batch."""
    if scene.get("batch"):
        sizes = [len(p) for p in pos]
        k = int(np.argsort(sizes)[len(sizes) // 2])
        sc, p = one_scene(scene, pos, k)
        v = vel[k] if vel is not None else None
        return sc, p, v, "scene %d of the batch (%d particles)" % (k, len(p))
    block = scene["block"]
    if depth >= block[2]:
        return scene, pos, vel, "the whole block"
    return (scene, slab(pos, block, depth), slab(vel, block, depth) if vel is not None else None,
            "a %d-layer slab of the block" % depth)


def launches_per_substep(scene, variant, iters, worklist=1):
    """Kernels one graph-launched PCISPH substep runs: 5 for the grid rebuild (hash and
    count, 2 scan kernels, place, rank and gather), 2 for density (the pair-record copy and
    the pass), non-pressure, 3 per corrector iteration (predicted density, pressure force,
    loop control), plus the warm start (one kernel; learned: features and the MLP); 2 more
    when pseudo-viscosity is active.  A batch adds the scenes' slot ranges and, with a work
    list, its rebuild before each iteration."""
    pv = 2 if scene.get("pseudo_viscosity", 10.0) * scene["dt"] > 0.1 else 0
    extra = {"plain": 0, "warm": 1, "learned": 2}[variant]
    batch = (1 + (iters if worklist else 0)) if scene.get("batch") else 0
    return 8 + extra + 3 * iters + pv + batch


def sample_substeps(first, total, k):
    """k substep indices spread evenly over [first, total): the timed sample of the run."""
    span = total - first
    return [first + (i * span) // k for i in range(k)]


def timed_event(stream, flush, fn):
    """Device time (ms) of fn() on `stream`, L2 flushed before and outside the events."""
    import torch
    flush.zero_()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    fn()
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b)


class StepLog:
    """Per-substep corrector statistics of one arm of the timed sample."""

    def __init__(self):
        self.ms, self.iters, self.errs = [], [], []
        self.not_converged = self.out_of_grid = self.crowded = 0

    def add(self, ms, st):
        self.ms.append(ms)
        self.iters.append(st["iterations"])
        self.errs.append(st["max_density_error_ratio"])
        self.not_converged += st["not_converged"]
        self.out_of_grid = max(self.out_of_grid, st["out_of_grid"])
        self.crowded = max(self.crowded, st["crowded"])


def frame_io(bb, g, scene, n, device, reps=5):
    """Particle frames of the final state in the reference's text format, end to end through
    the C ABI: the device writer formats and packs the frame and delivers its bytes to host
    memory (SerializerSaveSphDataSet3's block); the device reader takes the bytes back
    (SerializerLoadSphDataSet3) into a second solver.  Median of `reps` calls each; the CPU
    leg times the oracle's restatement of the reference serializer and reader (single
    thread, as the reference) on a slice of the same frame and scales it per particle."""
    from oracle import oracle as O
    flags = bb.FRAME_POSITION | bb.FRAME_VELOCITY | bb.FRAME_DENSITY | bb.FRAME_MASS
    size = len(g.frame_text(flags))
    out = bytearray(size)
    w = []
    for _ in range(reps + 1):
        t0 = time.perf_counter()
        g.frame_text(flags, out=out)
        w.append(time.perf_counter() - t0)
    text = bytes(out)
    r = bb.Solver(dict(scene), capacity=n, device=device)
    rd = []
    for _ in range(reps + 1):
        t0 = time.perf_counter()
        r.frame_load(text)
        rd.append(time.perf_counter() - t0)
    r.close()
    w, rd = float(np.median(w[1:])), float(np.median(rd[1:]))
    # CPU: a slice of 131,072 particles of the same frame
    fl, cnt, p, v, d, _ = O.frame_parse(text)
    m = min(len(p), 131072)
    mass = g.scalars()["mass"]
    t0 = time.perf_counter()
    sub = O.frame_text(p[:m], v[:m], d[:m], mass, scene["spacing"], flags)
    cw = (time.perf_counter() - t0) * len(p) / m
    t0 = time.perf_counter()
    O.frame_parse(sub)
    cr = (time.perf_counter() - t0) * len(p) / m
    return {"particles": n, "flags": "pvdm", "bytes": size,
            "write_ms": 1e3 * w, "write_gb_per_s": size / w / 1e9,
            "read_ms": 1e3 * rd, "read_gb_per_s": size / rd / 1e9,
            "cpu": {"kind": "port", "cores": 1, "write_ms": 1e3 * cw, "read_ms": 1e3 * cr,
                    "sample": "%d particles of the same frame, scaled per particle" % m},
            "measured": "host wall clock around the C-ABI calls (frame bytes in pageable host memory)"}


def seeding(bb, scene, final_pos, device, reps=3):
    """Particle seeding on the device, end to end through the C ABI, beside the oracle's
    restatement of the reference's CPU code (single thread, as the reference):
    - VolumeParticleEmitter3: a jittered BCC sphere of about 0.7 M particles at the
      scene's spacing (the rand() jitter sequence is drawn on the host, as in the reference);
    - MapGridEmit: the final state mapped, every particle moved half a spacing, the mapped
      cells refilled (capacity twice the particle count)."""
    import ctypes
    from oracle import oracle as O
    libc = ctypes.CDLL(None)
    sp = scene["spacing"]
    n = len(final_pos)
    out = {}
    shape = {"type": "sphere", "radius": 0.35 * (sp / 0.008), "center": (0.0, 0.0, 0.0)}
    s = bb.Solver(dict(scene), capacity=2 * n, device=device)
    t = []
    for _ in range(reps + 1):
        libc.srand(42)
        t0 = time.perf_counter()
        k = s.emit_volume(shape, sp, jitter=0.2)
        t.append(time.perf_counter() - t0)
    libc.srand(42)
    t0 = time.perf_counter()
    want, _ = O.emit_volume(shape, sp, jitter=0.2, capacity=k + 1)
    cpu = time.perf_counter() - t0
    out["volume_emitter"] = {"particles": k, "ms": 1e3 * float(np.median(t[1:])),
                             "cpu_ms": 1e3 * cpu, "cpu_kind": "port", "cpu_cores": 1,
                             "same_as_oracle": bool(len(want) == k)}
    # continuous emission on the final state
    s.upload(final_pos)
    s.setup()
    s.map_grid()
    moved = (final_pos + np.float32(0.5 * sp) * np.array([0.0, -1.0, 0.0], np.float32)).astype(np.float32)
    s.set(bb.FIELD_POSITION, moved)
    t0 = time.perf_counter()
    added = s.map_grid_emit(0.5 * sp)
    gpu = time.perf_counter() - t0
    s.close()
    o = O.OracleSim(scene, final_pos)
    o.update_grid_distribution()
    o.map_grid()
    o.set(O.POSITION, moved)
    t0 = time.perf_counter()
    ref = o.map_grid_emit(0.5 * sp)
    cpu = time.perf_counter() - t0
    o.close()
    out["map_grid_emit"] = {"particles": n, "added": added, "ms": 1e3 * gpu, "cpu_ms": 1e3 * cpu,
                            "cpu_kind": "port", "cpu_cores": 1, "same_as_oracle": bool(len(ref) == added)}
    # GenerateShapeSDF of a triangle mesh: a torus of 1,152 triangles on a grid of 0.55M nodes
    nu, nv = 32, 18
    u, w = np.meshgrid(2 * np.pi * np.arange(nu) / nu, 2 * np.pi * np.arange(nv) / nv, indexing="ij")
    big, small = 0.3, 0.1
    verts = np.stack([(big + small * np.cos(w)) * np.cos(u), (big + small * np.cos(w)) * np.sin(u),
                      small * np.sin(w)], axis=-1).reshape(-1, 3).astype(np.float32)
    tris = []
    for i in range(nu):
        for j in range(nv):
            a, b = i * nv + j, ((i + 1) % nu) * nv + j
            c, d = ((i + 1) % nu) * nv + (j + 1) % nv, i * nv + (j + 1) % nv
            tris += [(a, b, c), (a, c, d)]
    s2 = bb.Solver(dict(scene), capacity=16, device=device)
    s2.upload(final_pos[:16])
    t = []
    for _ in range(2):
        t0 = time.perf_counter()
        nodes, _, _, vals, _, stuck = s2.mesh_sdf(verts, np.array(tris, np.int32), dx=0.0075, margin=0.1)
        t.append(time.perf_counter() - t0)
    s2.close()
    out["mesh_sdf"] = {"triangles": len(tris), "nodes": int(np.prod(nodes)), "ms": 1e3 * min(t),
                       "inside_nodes": int((vals < 0).sum()), "stuck_rays": stuck,
                       "note": "tiles of 64 and sub-tiles of 8 triangles culled by their boxes (distance over a Morton-ordered copy, rays in index order)"}
    out["measured"] = "host wall clock around the C-ABI calls (single call; emitter median of %d)" % reps
    return out


def postprocess(bb, scene, final_pos, device):
    """Post-processing on the grid, end to end through the C ABI (host wall clock, result
    copied back), beside the oracle's restatement of the reference's CPU code (single
    thread):
    - boundary classification of the final state: LNMBoundary (fast), LNMBoundarySingle,
      LNMBoundaryExtended (5 levels), XiaoweiBoundary and LNMBoundary with the Xiaowei L2
      filter, on the same grid distribution and densities;
    - DiltsSpokeBoundary of a jittered BCC sphere of about 95 K particles at the spacing;
    - MarchingCubes of two overlapping spheres' distance on a 256^3 vertex grid (no CPU
      leg: the reference's own MarchingCubes is not part of the oracle)."""
    import ctypes
    from oracle import oracle as O
    sp = scene["spacing"]
    out = {}
    o = O.OracleSim(scene, final_pos)
    o.update_grid_distribution()
    o.compute_density(0)
    rho = o.get(O.DENSITY)
    s = bb.Solver(dict(scene), pos=final_pos, device=device)
    s.update_grid_distribution()
    s.set(bb.FIELD_DENSITY, rho)
    runs = {"lnm": (lambda: s.lnm_boundary(sp), lambda: o.lnm(sp)),
            "lnm_single": (lambda: s.lnm_boundary_single(sp), lambda: o.lnm_single(sp)),
            "lnm_extended": (lambda: s.lnm_boundary_extended(sp, 5), lambda: o.lnm_extended(sp, 5)),
            "xiaowei": (lambda: s.boundary_test("xiaowei", sp), lambda: o.xiaowei(sp)),
            "lnm_xiaowei": (lambda: s.lnm_boundary_geometric(sp, "xiaowei")[0],
                            lambda: o.lnm_geometric(sp, 1)[0])}
    for name, (dev, cpu) in runs.items():
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            got = dev()
            t.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        want = cpu()
        c = time.perf_counter() - t0
        out[name] = {"particles": len(final_pos), "ms": 1e3 * min(t[1:]), "cpu_ms": 1e3 * c,
                     "same_as_oracle": bool(np.array_equal(got, want))}
    s.close()
    o.close()
    ctypes.CDLL(None).srand(3)
    ball, _ = O.emit_volume({"type": "sphere", "center": (0.0, 0.0, 0.0), "radius": 0.18 * (sp / 0.008)}, sp,
                            jitter=0.2)
    s = bb.Solver(dict(scene), pos=ball, device=device)
    s.update_grid_distribution()
    t = []
    for _ in range(2):
        t0 = time.perf_counter()
        got = s.boundary_test("dilts")
        t.append(time.perf_counter() - t0)
    o = O.OracleSim(scene, ball)
    o.update_grid_distribution()
    t0 = time.perf_counter()
    want = o.dilts()
    c = time.perf_counter() - t0
    o.close()
    out["dilts"] = {"particles": len(ball), "boundary": int(got.sum()), "ms": 1e3 * min(t), "cpu_ms": 1e3 * c,
                    "same_as_oracle": bool(np.array_equal(got, want))}
    # marching cubes of two overlapping spheres on 256^3 nodes
    m = 256
    ax = np.linspace(-1.0, 1.0, m, dtype=np.float32)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")   # x fastest in memory
    d1 = np.sqrt((x - 0.2) ** 2 + y ** 2 + z ** 2) - 0.5
    d2 = np.sqrt((x + 0.3) ** 2 + (y - 0.1) ** 2 + z ** 2) - 0.4
    vals = np.minimum(d1, d2).astype(np.float32).ravel()
    del x, y, z, d1, d2
    spacing = float(ax[1] - ax[0])
    t = []
    for _ in range(3):
        t0 = time.perf_counter()
        pts, _, tris = s.marching_cubes((m, m, m), (-1.0, -1.0, -1.0), (spacing,) * 3, vals, 0.0)
        t.append(time.perf_counter() - t0)
    s.close()
    out["marching_cubes"] = {"nodes": m ** 3, "points": len(pts), "triangles": len(tris), "ms": 1e3 * min(t[1:]),
                             "note": "field upload, both passes and the mesh download included"}
    # the surface app on the final state: Zhu-Bridson field (kernel 2 x spacing, cells of
    # 2 x spacing) and marching cubes, beside the oracle's field
    sc = bb.surface_scene(final_pos, sp)
    s = bb.Solver(sc, pos=final_pos, device=device)
    t = []
    for _ in range(3):
        t0 = time.perf_counter()
        s.update_grid_distribution()
        nodes, org, spc, vals = s.particle_sdf("zhu", 2 * sp, sp)
        pts, _, tris = s.marching_cubes(nodes, org, spc, vals, 0.0)
        t.append(time.perf_counter() - t0)
    s.close()
    o = O.OracleSim(sc, final_pos)
    o.update_grid_distribution()
    t0 = time.perf_counter()
    want = o.particle_sdf(0, 2 * sp, sp)
    c = time.perf_counter() - t0
    o.close()
    out["surface_zhu_bridson"] = {"particles": len(final_pos), "field_nodes": int(np.prod(nodes)),
                                  "triangles": len(tris), "ms": 1e3 * min(t[1:]), "cpu_field_ms": 1e3 * c,
                                  "same_field_as_oracle": bool(np.array_equal(vals.view(np.uint32),
                                                                              want[3].view(np.uint32))),
                                  "note": "distribution, field, marching cubes and mesh download; the CPU leg is "
                                          "the field alone"}
    out["measured"] = "host wall clock around the C-ABI calls (best of the repeats after the first)"
    return out


def sph_config1(bb, device, stream, advances=200):
    """Config 1, the plain SPH dam break of 16,384 particles (SphSolver3, fixed dt 1e-3,
    200 Advance calls of 7 CFL substeps each), on the device with CUDA events around the
    Advance calls, beside the CPU oracle (the reference's SPH step restated, Jacobi order,
    all host threads) on the first 5 Advance calls from the same start."""
    import torch
    from bubbles_gb300 import scenes
    from oracle import oracle as O
    sc, pos = scenes.sph_16k(seed=0)
    g = bb.Solver(sc, pos=pos, device=device)
    g.set_stream(stream)
    for _ in range(3):
        g.advance(sc["dt"])
    g.upload(pos)
    g.setup()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    substeps = 0
    a.record(stream)
    for _ in range(advances):
        substeps += g.advance(sc["dt"])["substeps"]
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b)
    g.close()
    threads = os.cpu_count() or 1
    o = O.OracleSim(sc, pos, variant="f32", threads=threads)
    t0 = time.perf_counter()
    cpu_sub = sum(o.advance_sph(sc["dt"]) for _ in range(5))
    cpu_s = time.perf_counter() - t0
    o.close()
    n = len(pos)
    return {"workload": sc["workload"], "particles": n, "advances": advances, "substeps": substeps,
            "ms_per_advance": ms / advances, "us_per_substep": 1e3 * ms / substeps,
            "particle_updates_per_s": n * substeps / (ms / 1e3),
            "cpu": {"kind": "port", "cores": threads, "advances": 5, "substeps": cpu_sub,
                    "particle_updates_per_s": n * cpu_sub / cpu_s},
            "measured": "CUDA events on the solver's stream around the Advance calls (each reads its CFL "
                        "count back to the host)"}


def batched_config4(bb, device, stream, flush, samples=10, prep=200):
    """Config 4, 64 dam breaks of uneven sizes in one batch (3.7 M particles), learned warm
    start against the plain corrector: `prep` plain substeps (the MLP trains on them), then
    `samples` substeps spread evenly over the rest of the 500-substep run, each timed from
    the run's state with both correctors (CUDA events, L2 flushed before each)."""
    from bubbles_gb300 import autotune, scenes
    sc, pos = scenes.config("batched_64", seed=0)
    tuned = autotune.load("batched_64")
    if tuned is not None:
        sc = dict(sc, grid_spacing_scale=tuned["grid_spacing_scale"])
    scl = dict(sc, pressure_init="learned", mlp={"train_substeps": prep})
    scp = dict(sc, pressure_init="zero")
    g, gp = make_solver(bb, scl, pos, device), make_solver(bb, scp, pos, device)
    for s_ in (g, gp):
        if tuned is not None:
            s_.set_tuning(**tuned["tuning"])
        s_.set_stream(stream)
    dt, n = sc["dt"], sum(len(p) for p in pos)
    for _ in range(prep):
        g.advance_time_step(dt)
    learned, plain = StepLog(), StepLog()
    cur = prep
    for idx in sample_substeps(prep + 5, sc["steps"], samples):
        while cur < idx:
            g.advance_time_step(dt)
            cur += 1
        p, v = g.download()
        pr, dv = g.get(bb.FIELD_PRESSURE), g.get(bb.FIELD_DIVERGENCE)
        gp.upload(p, v)
        plain.add(timed_event(stream, flush, lambda: gp.advance_time_step(dt)), gp.stats())
        g.upload(p, v)
        g.set(bb.FIELD_PRESSURE, pr)
        g.set(bb.FIELD_DIVERGENCE, dv)
        learned.add(timed_event(stream, flush, lambda: g.advance_time_step(dt)), g.stats())
        cur += 1
    g.close()
    gp.close()
    lv, pv = n * samples / (sum(learned.ms) / 1e3), n * samples / (sum(plain.ms) / 1e3)
    return {"workload": sc["workload"], "particles": n, "samples": samples,
            "window": "substeps %d..%d of the %d-substep run" % (prep + 5, sc["steps"] - 1, sc["steps"]),
            "learned_value": lv, "plain_value": pv, "speedup_vs_plain": lv / pv,
            "corrector_iterations_learned_slowest_scene": float(np.mean(learned.iters)),
            "corrector_iterations_plain_slowest_scene": float(np.mean(plain.iters)),
            "not_converged_learned": learned.not_converged, "not_converged_plain": plain.not_converged,
            "unit": UNIT, "measured": "CUDA events on the launching stream, one substep per sample from the run's state"}


def energy_log(g, scene, substeps, path=None, every=10):
    """FP64 mass and energy of the state every `every` substeps of a run after the timed
    region (device reductions, bbg_energy), as JSONL records; optionally written to `path`."""
    dt = scene["dt"]
    recs = []
    for k in range(substeps + 1):
        if k % every == 0:
            e = g.energy()
            recs.append({"substep": k, "mass": e["mass"], "kinetic": e["kinetic"], "potential": e["potential"],
                         "total": e["kinetic"] + e["potential"], "momentum": [float(x) for x in e["momentum"]]})
        if k < substeps:
            g.advance_time_step(dt)
    if path:
        with open(path, "w") as f:
            for r in recs:
                f.write(json.dumps(r) + "\n")
    tot = [r["total"] for r in recs]
    return {"every": every, "substeps": substeps, "records": recs,
            "mass_change": recs[-1]["mass"] - recs[0]["mass"], "energy_change": tot[-1] - tot[0],
            "measured": "FP64 device reductions after the timed region (gravity potential against the origin)"}


def run_ours(args, scene, pos):
    import torch

    import bubbles_gb300 as bb

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = init_dist(world, "nccl")
    n = sum(len(p) for p in pos) if scene.get("batch") else len(pos)
    dt = scene["dt"]
    variant = args.variant
    stream = torch.cuda.Stream(device=local)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    warm = variant != "plain"
    learned = variant == "learned"
    compare = warm and not args.no_plain
    total = max(int(scene.get("steps", 0)), args.prep + args.warmup + args.steps)
    samples = sample_substeps(args.prep + args.warmup, total, args.steps)
    with torch.cuda.stream(stream):
        tuned = None
        if not args.no_tuning:
            from bubbles_gb300 import autotune
            tuned = autotune.load(args.config)
            if tuned is not None and scene.get("batch"):
                scene = dict(scene, grid_spacing_scale=tuned["grid_spacing_scale"])

        overrides = {k: int(v) for k, v in (kv.split("=", 1) for kv in args.tune)}

        def solver(sc):
            s = make_solver(bb, sc, pos, local)
            if tuned is not None:
                s.set_tuning(**tuned["tuning"])
            if overrides:
                s.set_tuning(**overrides)
            s.set_stream(stream)
            return s
        g = solver(scene)
        tuning_used = g.tuning()
        gp = solver(dict(scene, pressure_init="zero")) if compare else None
        # host copies of a sampled substep's input state (pinned): the e2e step reads them,
        # and every other timed arm is restored from them
        pos_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
        vel_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
        pr_h = torch.empty((n,), dtype=torch.float32, pin_memory=True).numpy()
        dv_h = torch.empty((n,), dtype=torch.float32, pin_memory=True).numpy()
        pos_o = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
        vel_o = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
        pr_o = torch.empty((n,), dtype=torch.float32, pin_memory=True).numpy()
        dv_o = torch.empty((n,), dtype=torch.float32, pin_memory=True).numpy()

        def snapshot():
            g.download(pos_h, vel_h)
            if warm:
                g.get(bb.FIELD_PRESSURE, out=pr_h)
            if learned:
                g.get(bb.FIELD_DIVERGENCE, out=dv_h)

        def restore(s, carried):
            s.upload(pos_h, vel_h)
            if carried:
                s.set(bb.FIELD_PRESSURE, pr_h)
                if learned:
                    s.set(bb.FIELD_DIVERGENCE, dv_h)

        def e2e_step():
            # end to end through the C ABI: the substep's inputs from pinned host memory,
            # its outputs back to host memory, one synchronisation
            if scene.get("batch"):
                g.upload(pos_h, vel_h)
                if warm:
                    g.set(bb.FIELD_PRESSURE, pr_h)
                if learned:
                    g.set(bb.FIELD_DIVERGENCE, dv_h)
                g.advance_time_step(dt)
                g.download(pos_o, vel_o)
                if warm:
                    g.get(bb.FIELD_PRESSURE, out=pr_o)
                if learned:
                    g.get(bb.FIELD_DIVERGENCE, out=dv_o)
                return
            g.step_host(dt, pos_h, vel_h, pr_h if warm else None, dv_h if learned else None,
                        pos_o, vel_o, pr_o if warm else None, dv_o if learned else None)

        # the first `prep` substeps of the run: plain corrector; the learned variant trains
        # its model on their (features, converged pressure) pairs
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.prep):
            g.advance_time_step(dt)
        torch.cuda.synchronize()
        prep_s = time.perf_counter() - t0
        mlp = g.mlp_status() if learned else None
        # warm-up: the run's next substeps, plus every timed arm once from the first
        # sampled state's predecessor (graph capture, first-use allocations), state restored
        for k in range(args.warmup):
            if k == args.warmup - 1:
                snapshot()
                if gp is not None:
                    restore(gp, False)
                    gp.advance_time_step(dt)
                    restore(gp, False)
                    gp.use_cuda_graphs(False)
                    gp.advance_time_step(dt)
                    gp.use_cuda_graphs(True)
                e2e_step()
                restore(g, warm)
                g.profiler_enable(True)
                g.advance_time_step(dt)
                g.profiler_enable(False)
                g.profiler_report()
                restore(g, warm)
            g.advance_time_step(dt)
        torch.cuda.synchronize()
        list_len = float(np.minimum(g.neighbor_counts() - 1, 64).mean())
        barrier(dist)

        sampler = ClockSampler(local)
        sampler.start()
        barrier(dist)
        # the timed sample: at each sampled substep of the run, from the run's state there,
        #   plain: the zero-start corrector (a second solver given the same state);
        #   kernels: the learned substep launched kernel by kernel with per-kernel events;
        #   e2e: the learned substep through bbg_step_host (host buffers, wall clock);
        #   value: the learned substep replayed as a CUDA graph (device events), which
        #   also carries the run forward.
        dev, pln, pln_host = StepLog(), StepLog(), StepLog()
        e2e_s, e2e_iters, e2e_ms = 0.0, [], []
        cur = args.prep + args.warmup
        for idx in samples:
            while cur < idx:
                g.advance_time_step(dt)
                cur += 1
            snapshot()
            if gp is not None:
                restore(gp, False)
                pln.add(timed_event(stream, flush, lambda: gp.advance_time_step(dt)), gp.stats())
                # the same plain substep in the reference's launch sequence: one launch per
                # pass, the host reading each iteration's error before the next
                restore(gp, False)
                gp.use_cuda_graphs(False)
                pln_host.add(timed_event(stream, flush, lambda: gp.advance_time_step(dt)), gp.stats())
                gp.use_cuda_graphs(True)
            restore(g, warm)
            g.profiler_enable(True)
            flush.zero_()
            g.advance_time_step(dt)
            g.profiler_enable(False)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2e_step()
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
            e2e_s += e2e_ms[-1] / 1e3
            e2e_iters.append(g.stats()["iterations"])
            restore(g, warm)
            dev.add(timed_event(stream, flush, lambda: g.advance_time_step(dt)), g.stats())
            cur += 1
        torch.cuda.synchronize()
        barrier(dist)
        sampler.stop()
        prof, _ = g.profiler_report()
        total_s = sum(dev.ms) / 1e3
        value, tmax, _ = aggregate(dist, float(n * args.steps), total_s)
        e2e_value, _, _ = aggregate(dist, float(n * args.steps), e2e_s)
        launches_timed = int(sum(launches_per_substep(scene, variant, it, tuning_used.get("batch_worklist", 1))
                                 for it in dev.iters))
        plain = None
        if gp is not None:
            pv, _, _ = aggregate(dist, float(n * args.steps), sum(pln.ms) / 1e3)
            plain = {"value": pv, "ms_per_step": sum(pln.ms) / args.steps,
                     "corrector_iterations_mean": float(np.mean(pln.iters)),
                     "max_density_error_ratio_max": float(np.max(pln.errs)),
                     "not_converged": pln.not_converged}
            ph, _, _ = aggregate(dist, float(n * args.steps), sum(pln_host.ms) / 1e3)
            plain["host_loop"] = {
                "value": ph, "ms_per_step": sum(pln_host.ms) / args.steps,
                "corrector_iterations_mean": float(np.mean(pln_host.iters)),
                "launches": "one launch per pass, the host reading each corrector iteration's "
                            "max error before launching the next (the reference's GPU loop)"}
            gp.close()
        final_pos, final_vel = g.download()
        batch_offsets = g.layout() if scene.get("batch") else None
        energy = None
        steps_e = args.energy_steps if args.energy_steps >= 0 else (100 if args.config == "pcisph_4m" else 0)
        if steps_e > 0 and rank == 0:
            energy = energy_log(g, scene, steps_e, args.energy_log)
        frames = seeds = post = sph1 = batch4 = None
        if not scene.get("batch") and not args.no_frames and rank == 0:
            frames = frame_io(bb, g, scene, n, local)
            seeds = seeding(bb, scene, final_pos, local)
            post = postprocess(bb, scene, final_pos, local)
        g.close()
        if not scene.get("batch") and not args.no_frames and rank == 0:
            sph1 = sph_config1(bb, local, stream)
            batch4 = batched_config4(bb, local, stream, flush)

    if rank != 0:
        barrier(dist)
        return

    # roofline of the dominant kernel
    peak, peak_kind = load_peaks()
    traffic_table = load_traffic(args.config)
    table = alg_bytes(list_len)
    kern = {k: v for k, v in prof.items() if k in table}
    top = max(kern, key=lambda k: kern[k][0]) if kern else None
    roof = None
    if top:
        ms, cnt = kern[top]
        avg_s = ms / cnt / 1e3
        alg = table[top] * n
        achieved = alg / avg_s / 1e9
        tr = traffic_table.get(top)
        roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": tr * n if tr is not None else None,
                "algorithmic_bytes": alg, "avg_launch_us": avg_s * 1e6,
                "share_of_step": ms / sum(v[0] for v in prof.values()),
                "measured": "per-launch CUDA events on the launching stream over the sampled substeps "
                            "(launched kernel by kernel from the same states; the timed arm replays the "
                            "same kernels as graphs)"}

    # CPU baseline: oracle on the host cores, bounded sample of the same state
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        if scene.get("batch"):
            cuts = np.cumsum([len(p) for p in pos])[:-1]
            fp, fv = np.split(final_pos, cuts), np.split(final_vel, cuts)
            # the e2e buffers hold packed coordinates: take each scene back out
            fp = [a - batch_offsets[i].astype(np.float32) for i, a in enumerate(fp)]
        else:
            fp, fv = final_pos, final_vel
        sc_c, sample_p, sample_v, what = cpu_sample(scene, fp, fv, args.cpu_slab)
        rate, steps_c, iters_c, t_c = cpu_oracle_rate(sc_c, np.asarray(sample_p, np.float64),
                                                      np.asarray(sample_v, np.float64),
                                                      args.cpu_budget, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": ("%d substep(s) (%.1f s, %.2f corrector iterations each) of %s "
                          "(%d particles) from the same state, FP32 oracle, plain corrector, %d threads"
                          % (steps_c, t_c, iters_c / max(1, steps_c), what, len(sample_p), threads))}

    per_kernel = {k: {"ms_total": v[0], "launches": v[1], "avg_us": 1e3 * v[0] / max(1, v[1])}
                  for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    first, last = samples[0], samples[-1]
    config = {"workload": scene["workload"], "variant": variant, "solver": "pcisph",
              "particles_per_gpu": n, "dt": dt, "tolerance": scene["max_density_error_ratio"],
              "max_iterations": scene["max_iterations"],
              "window": ("%d substeps sampled evenly over substeps %d..%d of the %d-substep run (%d preparation "
                         "+ %d warm-up substeps first); each timed from the run's state at that substep"
                         % (len(samples), first, last, total, args.prep, args.warmup)),
              "corrector_iterations_mean": float(np.mean(dev.iters)),
              "corrector_iterations_mean_e2e": float(np.mean(e2e_iters)),
              "e2e_ms_per_sample": [round(x, 3) for x in e2e_ms],
              "max_density_error_ratio_max": float(np.max(dev.errs)),
              "substeps_at_max_iterations_above_tolerance": dev.not_converged,
              "state_checks": {"out_of_grid_max": dev.out_of_grid, "crowded_max": dev.crowded},
              "member_list_mean": list_len,
              "preparation_s": prep_s,
              "regions": "at every sampled substep the plain, per-kernel, e2e and timed arms start "
                         "from the same state (host copy of the run's state, uploaded outside the timing)",
              "l2": "flushed before every timed substep (256 MB write, outside the events)",
              "tuning": dict({"source": ("bubbles_gb300/tuned/%s.json" % args.config) if tuned is not None
                              else "defaults",
                              "grid_spacing_scale": scene.get("grid_spacing_scale", 2.0)}, **tuning_used),
              "parallelism": "replicas" if world > 1 else "single gpu"}
    if variant == "warm":
        config["warm_start"] = "previous substep's pressure x 0.5, monotone corrector update"
    if variant == "learned":
        config["warm_start"] = ("MLP 4-64-64-1 GELU, BF16 tensor-core inference; estimate x 0.9, "
                                "monotone corrector update")
        config["mlp"] = {"trained_substeps": mlp["trained_substeps"], "adam_steps": mlp["adam_steps"],
                         "last_training_loss": mlp["last_loss"],
                         "training": "online during the %d preparation substeps" % args.prep}
    config["iterations_per_sample"] = [int(x) for x in dev.iters]
    if plain is not None:
        plain["iterations_per_sample"] = [int(x) for x in pln.iters]
        config["plain_same_window"] = plain
    clocks = sampler.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tmax / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config,
        # the comparison the metric names, flat: this variant against the plain (zero-start,
        # reference) corrector on the same substeps from the same states
        "variant": variant,
        "corrector_iterations": float(np.mean(dev.iters)),
        "not_converged": dev.not_converged,
        "max_density_error_ratio": float(np.max(dev.errs)),
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": n * (24 + (4 if warm else 0) + (4 if variant == "learned" else 0)),
                "d2h_bytes_per_step": n * (24 + (4 if warm else 0) + (4 if variant == "learned" else 0))},
        "roofline": roof,
        "cpu_baseline": cpu,
        "gpu_launches": launches_timed,
        "clocks": clocks,
        "kernels": per_kernel,
        # a batch's corrector passes run over the unconverged scenes' tiles only, while
        # the fractions count every particle: for batches they overstate those passes
        "kernel_bounds": kernel_bounds(prof, table, n, peak,
                                       load_profile_figures(args.config, "warp_instructions_per_particle"),
                                       torch.cuda.get_device_properties(local).multi_processor_count,
                                       clocks.get("sm_mhz")),
    }
    if roof is not None and roof["kernel"] in line["kernel_bounds"]:
        # the dominant kernel's other bound: its share of the SMs' issue slots
        roof["issue_frac"] = line["kernel_bounds"][roof["kernel"]].get("issue_frac")
    if plain is not None:
        line.update({"plain_value": plain["value"], "speedup_vs_plain": value / plain["value"],
                     "plain_host_loop_value": plain["host_loop"]["value"],
                     "speedup_vs_plain_host_loop": value / plain["host_loop"]["value"],
                     "corrector_iterations_plain": plain["corrector_iterations_mean"],
                     "not_converged_plain": plain["not_converged"],
                     "max_density_error_ratio_plain": plain["max_density_error_ratio_max"]})
    if sph1 is not None:
        line["sph_config1"] = sph1
        line["sph_config1_value"] = sph1["particle_updates_per_s"]   # flat copies of the extras' figures
    if batch4 is not None:
        line["batched_config4"] = batch4
        line["batched_config4_value"] = batch4["learned_value"]
        line["batched_config4_plain_value"] = batch4["plain_value"]
        line["batched_config4_speedup_vs_plain"] = batch4["speedup_vs_plain"]
    if frames is not None:
        line["frame_io"] = frames
    if seeds is not None:
        line["seeding"] = seeds
        line["postprocess"] = post
    if energy is not None:
        line["energy_log"] = energy
    print(json.dumps(line), flush=True)
    barrier(dist)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=795,
                    help="timed substeps (default: the rest of the 1,000-substep run)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--prep", type=int, default=200,
                    help="substeps run before warm-up (the learned variant trains during them)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="pcisph_1m")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--cpu-slab", type=int, default=32, help="z-layers of the block for the CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--energy-steps", type=int, default=-1,
                    help="substeps of FP64 mass/energy logging after the timed region (every 10); "
                         "default 100 for pcisph_4m, else none")
    ap.add_argument("--energy-log", default=None, help="JSONL file for the mass/energy records")
    ap.add_argument("--mlp", action="append", default=[], metavar="KEY=VALUE",
                    help="learned warm start settings (bbg_mlp_desc fields, e.g. expectile=0.4)")
    ap.add_argument("--warm-scale", type=float, default=None,
                    help="start pressure = scale x estimate for warm starts (default: the library's, 0.9 learned)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-corrector comparison")
    ap.add_argument("--tune", action="append", default=[], metavar="KEY=VALUE",
                    help="launch tuning override after the tuned file (bbg_tuning fields, e.g. block_size=64)")
    ap.add_argument("--max-iterations", type=int, default=None,
                    help="corrector iteration cap of both arms (default: the configuration's)")
    ap.add_argument("--no-frames", action="store_true",
                    help="skip the particle-frame and seeding timings (frame writer / reader, emitters)")
    ap.add_argument("--no-tuning", action="store_true",
                    help="ignore bubbles_gb300/tuned/<config>.json (autotuner output)")
    ap.add_argument("--variant", default="learned", choices=["plain", "warm", "learned"],
                    help="corrector start: plain = zero pressure (reference), warm = the previous "
                         "substep's pressure, learned = the MLP estimate")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    from bubbles_gb300 import scenes
    rank, _, _ = dist_env()
    scene, pos = scenes.config(args.config, seed=args.seed + rank)
    scene["pressure_init"] = {"plain": "zero", "warm": "previous", "learned": "learned"}[args.variant]
    if args.variant == "learned":
        scene["mlp"] = dict(scene.get("mlp_training", {}), train_substeps=args.prep)
        for kv in args.mlp:
            k, v = kv.split("=", 1)
            scene["mlp"][k] = float(v) if "." in v or "e" in v else int(v)
    if args.warm_scale is not None:
        scene["warm_scale"] = args.warm_scale
    if args.max_iterations is not None:
        scene["max_iterations"] = args.max_iterations
    if args.impl == "reference":
        run_reference(args, scene, pos)
    else:
        run_ours(args, scene, pos)


if __name__ == "__main__":
    main()
