"""Benchmark of the GB300 per-substep cloth step (vertex-substeps/s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One step = one frame = ClothSolverBase::SimulateSwift (num_substeps substeps).  The default
workload is the batched configuration: 512 garments (vertex counts log-uniform in [2k, 100k],
14.19 M vertices in all), each draped on its own animated 6,890-vertex tube body, stepped by one
context in one launch per phase, 10 substeps x 10 iterations, stretch + bend + LRA, obstacle and
particle self contact.  Inputs are synthetic and seeded (xrtailor_gb300/scenes.py).

Output: one JSON line (rank 0).  `value` times K frames with CUDA events on the library's stream,
inputs resident in HBM, L2 flushed (a 512 MiB write) between frames outside the timed events;
`e2e` times K frames through the public API with host buffers (obstacle targets in from pinned
memory, cloth positions out, per frame) by wall clock; `roofline` is the dominant phase's
algorithmic bytes per launch over its launch time, timed by CUDA event-record nodes inside a
replayed frame graph; `plain_per_garment` / `batched_over_plain` time a sample of the same
garments each alone in its own context; `cpu_baseline` is the oracle (OpenMP CPU restatement)
on a bounded garment sample; `plain_garment` holds the 256 x 256 garment's numbers.
`--impl reference` times that CPU restatement alone on a garment sample per step: the reference's
own path is CUDA-only and cannot be built here (no glm / vcglib / GLFW sources), so the oracle
port stands in for it.  Other workloads: --workload garment|small|heavy|diff|lbvh|impact.
Several GPUs (torchrun) run independent replicas.
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

HBM_FALLBACK = 6800.0
METRIC = "vertex-substeps/s"


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


def _workload(name):
    from xrtailor_gb300 import scenes
    if name == "garment":
        return scenes.plain_garment(256)
    if name == "small":
        return scenes.plain_small(64)
    if name == "heavy":
        return scenes.plain_heavy(1024)
    raise SystemExit(f"unknown workload {name}")


def _mesh_counts(mesh):
    """(vertices, edges, bend elements) of a triangle mesh: undirected edges, and one bend
    element per edge shared by two triangles."""
    t = np.asarray(mesh.triangles, np.int64)
    e = np.sort(np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e[:, 0] * (int(t.max()) + 1) + e[:, 1], return_counts=True)
    return len(mesh.positions), len(cnt), int((cnt == 2).sum())


L2_NOTE = "flushed between frames (512 MiB write, outside the timed events)"


def _plain_config(workload, p, quality=False, fem=False):
    """The workload's description, the same for both arms (a function of the scene only)."""
    sc = _workload(workload)
    V, E, B = _mesh_counts(sc.cloth)
    att = sc.cloth.attached_indices
    slots = 0 if att is None else len(att)
    return {"workload": f"plain_{workload}" + ("_quality" if quality else ("_fem" if fem else "")),
            "quality": ("FEM fabric, imminent + PBD repulsion, impact-zone collision step "
                        "per substep, no particle hash") if quality else None,
            "fabric": "FEM strain + isometric bending" if fem else "XPBD stretch + dihedral bend",
            "vertices": V, "edges": E, "bends": B, "lra": slots * V,
            "obstacle_triangles": len(sc.obstacle.triangles) if sc.obstacle is not None else 0,
            "substeps": p.num_substeps, "iterations": p.num_iterations,
            "collision_passes": p.num_collision_passes,
            "self_collision": bool(p.enable_self_collision), "l2": L2_NOTE}


def _batched_config(instances, p):
    """The batched workload's description, the same for both arms (a function of the seeded
    draw only)."""
    from xrtailor_gb300 import scenes
    rng_sizes = scenes.batched_sizes(instances)
    nxy = scenes.batched_grid_dims(instances)
    E = int(sum(nx * (ny - 1) + ny * (nx - 1) + (nx - 1) * (ny - 1) for nx, ny in nxy))
    B = E - int(sum(2 * (nx - 1) + 2 * (ny - 1) for nx, ny in nxy))
    V = int(rng_sizes.sum())
    return {"workload": f"batched_{instances}", "instances": instances, "vertices": V,
            "edges": E, "bends": B, "lra": 2 * V,
            "obstacle_triangles": instances * len(scenes.TubeBody().triangles),
            "substeps": p.num_substeps, "iterations": p.num_iterations,
            "collision_passes": p.num_collision_passes,
            "self_collision": bool(p.enable_self_collision), "l2": L2_NOTE}


def _setup(solver, sc):
    solver.add_cloth(sc.cloth, particle_diameter=sc.particle_diameter)
    if sc.obstacle is not None:
        solver.add_obstacle(sc.obstacle)
    solver.start()


def _targets(sc, frames):
    if sc.body is None:
        return None
    return [sc.body.pose((f + 1) / 60.0) for f in range(frames)]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def bytes_per_substep(s, p, has_obstacle):
    """Algorithmic bytes of one substep (fp32, vec3 = 12 B, index = 4 B):
    V*52 + I*[V*28 + E*24 + B*24 + L*12 + Nb*72 + C_solve] + P*C_gen, with
    C_solve = V*32 + E*48 + V*32 and C_gen = V*24 + V*32 + E*48 per collision pass."""
    V, E, B, L, Nb = s.num_vertices, s.num_edges, s.num_bends, s.num_lra, s.num_bindings
    I = p.num_iterations
    c_solve = (V * 32 + E * 48 + V * 32) if has_obstacle else 0
    c_gen = (V * 24 + V * 32 + E * 48) if has_obstacle else 0
    passes = p.num_collision_passes / p.num_substeps
    return V * 52 + I * (V * 28 + E * 24 + B * 24 + L * 12 + Nb * 72 + c_solve) + passes * c_gen


# Algorithmic bytes per processed unit of each phase's launch: records read + vertices read and
# written (float4 = 16 B).  stretch: 16 B record + 8 B lambda r/w + 2 x 32 B vertex r/w;
# bend: 16 B indices + 8 B (angle, compliance) + 4 x 32 B; collide: x, x0 read + x write (48 B);
# vf_solve: x r/w + two contact records (32 B + 16 B) ; ee_apply: x read + write (32 B) + the
# vertex's edge list entries are data dependent and not counted.
BYTES_PER_UNIT = {"stretch": 88, "bend": 152, "collide": 48, "vf_solve": 64, "ee_apply": 32,
                  "predict_finalize": 64, "lra": 32}
# The frame formula's per-unit terms for the tile-local stretch and bend launches: a constraint
# record (stretch: 2 indices, rest, compliance + multiplier read and written; bend: 4 indices,
# rest angle, compliance) and a vertex touched once (position read + written, inverse mass).
RECORD_BYTES = 24
VERTEX_BYTES = 28
# FEM fabric (the phases keep the names stretch / bend): strain = 3 indices + inverse rest
# matrix + area (36 B); isometric bending = 4 indices + 4x4 Hessian + multiplier read and
# written (88 B).
FEM_RECORD_BYTES = {"stretch": 36, "bend": 88}


def run_ours(args, rank, local_rank, world):
    import torch
    from xrtailor_gb300 import ClothSolver, build as xb, scenes
    xb.build()
    torch.cuda.set_device(local_rank)
    sc = _workload(args.workload)
    p = scenes.scene_params(sc)
    if args.quality:
        _quality(p)
    fem = args.material == "fem" or args.quality
    frames_needed = args.warmup + 2 * args.steps + 8
    tg = _targets(sc, frames_needed)
    dev_targets = None
    if tg is not None:
        dev_targets = torch.tensor(np.stack(tg), device=f"cuda:{local_rank}")
        torch.cuda.synchronize()

    def make(tile):
        q = ClothSolver(p, device=local_rank)
        if tile is not None:
            q.set_tile_vertices(tile)
        if fem:
            q.set_fem_material(ClothSolver.fem_material())
        _setup(q, sc)
        return q

    # launch configuration of a single-garment workload: autotuned on the workload itself
    tuned, trials, tune_s = None, [], 0.0
    if args.tile_vertices is None and args.tune_instances > 0 and not args.quality:
        from xrtailor_gb300 import autotune
        t0 = time.perf_counter()
        tuned, trials = autotune.tune(
            make, tiles=(128, 256, 512), frames=8, warmup=3, vertex_blocks=(64, 128, 256),
            targets=(None if dev_targets is None else
                     (lambda k: dev_targets[k % frames_needed].data_ptr())))
        tune_s = time.perf_counter() - t0
    solver = make(args.tile_vertices if tuned is None else tuned["tile_vertices"])
    if tuned is not None:
        solver.set_dependent_launch(tuned["dependent_launch"])
        solver.set_vertex_block(tuned["vertex_block"])
    s = solver.sizes()
    V, S = s.num_vertices, p.num_substeps
    _, _, stream_ptr = solver.device_state()
    stream = torch.cuda.ExternalStream(stream_ptr, device=f"cuda:{local_rank}")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local_rank}")
    lib = solver._lib
    fi = 0

    def set_targets_dev(k):
        if dev_targets is not None:
            lib.xrt_set_obstacle_targets_device(solver._h, dev_targets[k].data_ptr())

    for _ in range(args.warmup):
        set_targets_dev(fi)
        solver.step()
        fi += 1
    solver.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                set_targets_dev(fi)
                fi += 1
                starts[k].record(stream)
                solver.step()
                ends[k].record(stream)
                flush.zero_()
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    solver.synchronize()
    s = solver.sizes()  # launches_per_frame is known once the frame graph exists
    frame_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    t_dev = sum(frame_ms) / 1e3
    if world > 1:
        tt = torch.tensor([t_dev], device=f"cuda:{local_rank}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
        t_dev = float(tt.item())
    units = V * S * args.steps * world
    value = units / t_dev

    # end to end through the C ABI with host buffers (pinned)
    from xrtailor_gb300 import _lib as L
    host_targets = None
    if tg is not None:
        host_targets = torch.from_numpy(np.stack(tg)).pin_memory().numpy()
    out = torch.empty((V, 3), dtype=torch.float32).pin_memory().numpy()
    h2d = (host_targets[0].nbytes if host_targets is not None else 0)
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for k in range(args.steps):
        if host_targets is not None:
            solver.set_obstacle_targets(host_targets[fi % len(host_targets)])
        fi += 1
        solver.step()
        L.check(lib.xrt_get_positions(solver._h, L.fptr(out)), solver._h, "read")
    e2e_t = time.perf_counter() - e0
    e2e = V * S * args.steps / e2e_t

    # per-phase profile (eager frames with CUDA events around every launch)
    solver.set_profiling(True)
    for _ in range(3):
        set_targets_dev(fi % frames_needed)
        fi += 1
        solver.step()
    prof = solver.profile()
    solver.set_profiling(False)
    phases = {k: v for k, v in prof.items() if k != "frames"}
    total_ms = sum(v["ms"] for v in phases.values())
    dom = max((k for k in phases if k in BYTES_PER_UNIT), key=lambda k: phases[k]["ms"])
    d = phases[dom]
    peak, peak_src = _peaks()
    per_launch_bytes = BYTES_PER_UNIT[dom] * d["units"] / max(d["launches"], 1)
    accounting = "per constraint: record + every vertex read and written (BYTES_PER_UNIT)"
    tiles = {"stretch": (s.num_stretch_tile_colors, s.stretch_footprint_vertices),
             "bend": (s.num_bend_tile_colors, s.bend_footprint_vertices)}.get(dom)
    if tiles and tiles[0]:
        # the frame formula's terms for one tile-color launch: the constraints' records (24 B
        # each: indices, rest value, compliance, multiplier) and each footprint vertex once
        # (28 B: position read and written, inverse mass read); a tile color's footprints are
        # disjoint, so a launch touches footprint / tile colors vertices on average
        record = FEM_RECORD_BYTES[dom] if fem else RECORD_BYTES
        per_launch_bytes = (record * d["units"] / max(d["launches"], 1) +
                            VERTEX_BYTES * tiles[1] / tiles[0])
        accounting = (f"frame formula: {record} B per constraint record + {VERTEX_BYTES} B per "
                      "footprint vertex of the launch")
    per_launch_s = d["ms"] / 1e3 / max(d["launches"], 1)
    achieved = per_launch_bytes / per_launch_s / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            key = args.workload + ("_fem" if fem else "")
            tr = json.load(open(tpath)).get(key, {}).get(dom)
            if tr:
                traffic = tr["bytes_per_unit"] * d["units"] / max(d["launches"], 1)
        except Exception:
            traffic = None
    frame_bytes = bytes_per_substep(s, p, sc.obstacle is not None) * S
    result = {
        "metric": METRIC, "value": value, "unit": "vertex-substeps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generators, xrtailor_gb300/scenes.py)",
        "config": dict(_plain_config(args.workload, p, args.quality, fem),
                       parallelism="replicas" if world > 1 else "single"),
        "schedule": {"stretch_colors": s.num_stretch_colors, "bend_colors": s.num_bend_colors},
        "launch": tuned or {"tile_vertices": args.tile_vertices or 256},
        "autotune": {"seconds": round(tune_s, 1),
                     "trials_ms_per_frame": [[t, d, b, round(ms, 3)] for t, d, b, ms in trials]},
        "e2e": {"value": e2e, "unit": "vertex-substeps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(out.nbytes)},
        "gpu_launches": int(s.launches_per_frame) * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_src, "bytes_per_launch": per_launch_bytes,
                     "accounting": accounting,
                     "us_per_launch": per_launch_s * 1e6,
                     "share_of_frame": d["ms"] / total_ms if total_ms else None},
        "frame_bandwidth_gbs": frame_bytes / (t_dev / args.steps / world) / 1e9,
        "phase_ms_per_frame": {k: round(v["ms"] / max(prof["frames"], 1), 4) for k, v in phases.items()},
        "clocks": clocks.summary(),
        "wall_s": wall,
    }
    return result


def _phase_roofline(prof, sz, fem=False):
    """The dominant phase of a per-phase profile (xrt_get_profile) and its roofline terms:
    algorithmic bytes per launch over the launch's average time.  Tile-local stretch and bend
    launches are accounted in the frame formula's terms (record bytes per constraint + 28 B per
    footprint vertex of the launch); other phases by BYTES_PER_UNIT."""
    phases = {k: v for k, v in prof.items() if k != "frames" and v["launches"]}
    total_ms = sum(v["ms"] for v in phases.values())
    dom = max((k for k in phases if k in BYTES_PER_UNIT), key=lambda k: phases[k]["ms"])
    d = phases[dom]
    per_launch_bytes = BYTES_PER_UNIT[dom] * d["units"] / max(d["launches"], 1)
    accounting = "per constraint: record + every vertex read and written (BYTES_PER_UNIT)"
    tiles = {"stretch": (sz.num_stretch_tile_colors, sz.stretch_footprint_vertices),
             "bend": (sz.num_bend_tile_colors, sz.bend_footprint_vertices)}.get(dom)
    if tiles and tiles[0]:
        # a tile color's footprints are disjoint, so one launch touches footprint / tile colors
        # vertices; its records are the launch's constraints
        record = FEM_RECORD_BYTES[dom] if fem else RECORD_BYTES
        per_launch_bytes = (record * d["units"] / max(d["launches"], 1) +
                            VERTEX_BYTES * tiles[1] / tiles[0])
        accounting = (f"frame formula: {record} B per constraint record + {VERTEX_BYTES} B per "
                      "footprint vertex of the launch")
    per_launch_s = d["ms"] / 1e3 / max(d["launches"], 1)
    return dom, d, per_launch_bytes, per_launch_s, accounting, (d["ms"] / total_ms if total_ms else None)


def _traffic(key, dom, units_per_launch):
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        tr = json.load(open(tpath)).get(key, {}).get(dom)
        if tr:
            return tr["bytes_per_unit"] * units_per_launch
    except Exception:
        pass
    return None


def run_batched(args, local_rank):
    """The batched workload: `--instances` garments (default 512), each on its own body, stepped
    by one context in one launch per phase; then a sample of the same garments stepped one
    context each (the plain step per garment) on the same GPU, frames timed the same way."""
    import torch
    from xrtailor_gb300 import ClothSolver, build as xb, scenes
    xb.build()
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    from xrtailor_gb300 import autotune
    t_gen = time.perf_counter()
    gs = scenes.batched_garments(args.instances)
    p = scenes._params(**scenes.BATCHED_PARAMS)
    S = p.num_substeps
    nframes = args.warmup + 2 * args.steps + 4
    ov = [len(g.body.rest) for g in gs]
    obase = np.concatenate([[0], np.cumsum(ov)])
    # obstacle targets of every frame, on the device (timed frames) and in pinned host memory
    # (frames through the public API with host buffers)
    tg_host = torch.empty((nframes, int(obase[-1]), 3), dtype=torch.float32).pin_memory()
    for f in range(nframes):
        tg_host[f] = torch.from_numpy(np.concatenate([g.body.pose((f + 1) / 60.0) for g in gs]))
    tg = tg_host.to(dev)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t_gen

    def comps(idx):
        return np.concatenate([np.full(gs[i].num_edges, gs[i].stretch_compliance, np.float32)
                               for i in idx])

    def make(tile, idx):
        q = ClothSolver(p, device=local_rank)
        if tile is not None:
            q.set_tile_vertices(tile)
        for i in idx:
            q.add_instance(gs[i].cloth, gs[i].body.mesh)
        q.set_compliance(0, comps(idx))
        q.start()
        return q

    # launch configuration: autotuned on an evenly spaced subset of the garments
    tuned, trials, tune_s = None, [], 0.0
    if args.tile_vertices is None and args.tune_instances > 0:
        t0 = time.perf_counter()
        sub = autotune.subset(len(gs), args.tune_instances)
        tg_sub = torch.cat([tg[:, int(obase[i]):int(obase[i + 1])] for i in sub], dim=1)
        tuned, trials = autotune.tune(lambda t: make(t, sub), frames=2, warmup=1,
                                      targets=lambda k: tg_sub[k % nframes].data_ptr())
        del tg_sub
        tune_s = time.perf_counter() - t0
    t_setup = time.perf_counter()
    tile = args.tile_vertices if tuned is None else tuned["tile_vertices"]
    s = make(tile, range(len(gs)))
    if tuned is not None:
        s.set_dependent_launch(tuned["dependent_launch"])
        s.set_vertex_block(tuned["vertex_block"])
    setup_s = time.perf_counter() - t_setup
    sz = s.sizes()
    V = sz.num_vertices
    _, _, sp = s.device_state()
    stream = torch.cuda.ExternalStream(sp, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    lib = s._lib
    fi = 0
    for _ in range(args.warmup):
        lib.xrt_set_obstacle_targets_device(s._h, tg[fi].data_ptr())
        fi += 1
        s.step()
    s.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for a, b in ev:
                lib.xrt_set_obstacle_targets_device(s._h, tg[fi].data_ptr())
                fi += 1
                a.record(stream)
                s.step()
                b.record(stream)
                flush.zero_()
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    s.synchronize()
    t_batch = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    value = V * S * args.steps / t_batch
    launches = s.sizes().launches_per_frame
    sz = s.sizes()

    # end to end through the public API: the frame's obstacle targets from pinned host memory,
    # the step, the cloth positions back into host memory, every frame
    from xrtailor_gb300 import _lib as L
    out = torch.empty((V, 3), dtype=torch.float32).pin_memory().numpy()
    h2d = int(tg_host[0].numel() * 4)
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        s.set_obstacle_targets(tg_host[fi].numpy())
        fi += 1
        s.step()
        L.check(lib.xrt_get_positions(s._h, L.fptr(out)), s._h, "read")
    e2e_t = time.perf_counter() - e0
    e2e = V * S * args.steps / e2e_t

    # per-phase profiles of one frame each: replayed graph with an event pair per phase group
    # (the roofline's launch time) and eager frames with an event pair per launch
    prof = {}
    for mode, graph in (("graph", True), ("eager", False)):
        s.set_profiling(True, graph=graph)
        lib.xrt_set_obstacle_targets_device(s._h, tg[fi % nframes].data_ptr())
        fi += 1
        s.step()
        prof[mode] = s.profile()
        s.set_profiling(False)
    dom, d, per_launch_bytes, per_launch_s, accounting, share = _phase_roofline(prof["graph"], sz)
    peak, peak_src = _peaks()
    achieved = per_launch_bytes / per_launch_s / 1e9
    units_per_launch = d["units"] / max(d["launches"], 1)
    phases = {m: {k: round(v["ms"] / max(pr["frames"], 1), 3) for k, v in pr.items()
                  if k != "frames" and v["launches"]} for m, pr in prof.items()}
    s.close()
    del s
    torch.cuda.empty_cache()

    # the plain step per garment: one context per garment, frames timed with events on its stream
    sample = autotune.subset(len(gs), args.plain_sample) if args.plain_sample > 0 else []
    plain_t, plain_units = 0.0, 0
    t_plain_wall = time.perf_counter()
    for i in sample:
        g = gs[i]
        q = ClothSolver(p, device=local_rank)
        if args.tile_vertices is not None:
            q.set_tile_vertices(args.tile_vertices)
        q.add_cloth(g.cloth)
        q.add_obstacle(g.body.mesh)
        q.set_compliance(0, np.full(g.num_edges, g.stretch_compliance, np.float32))
        q.start()
        _, _, qsp = q.device_state()
        qs = torch.cuda.ExternalStream(qsp, device=dev)
        o0, o1 = int(obase[i]), int(obase[i + 1])
        lib.xrt_set_obstacle_targets_device(q._h, tg[0, o0:o1].data_ptr())
        q.step()  # warm-up (captures the frame graph)
        q.synchronize()
        pe = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.plain_frames)]
        with torch.cuda.stream(qs):
            for k, (a, b) in enumerate(pe):
                lib.xrt_set_obstacle_targets_device(q._h, tg[1 + k, o0:o1].data_ptr())
                a.record(qs)
                q.step()
                b.record(qs)
        torch.cuda.synchronize()
        plain_t += sum(a.elapsed_time(b) for a, b in pe) / 1e3 / args.plain_frames
        plain_units += len(g.cloth.positions) * S
        q.close()
    plain_wall = time.perf_counter() - t_plain_wall
    plain_value = plain_units / plain_t if plain_t > 0 else None
    res = {
        "metric": METRIC, "value": value, "unit": "vertex-substeps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_batch / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded: xrtailor_gb300/scenes.py batched_garments)",
        "config": dict(_batched_config(len(gs), p), parallelism="single"),
        "launch": tuned or {"tile_vertices": tile},
        "e2e": {"value": e2e, "unit": "vertex-substeps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(out.nbytes),
                "path": "ClothSolver.set_obstacle_targets + step + xrt_get_positions, pinned "
                        "host buffers"},
        "gpu_launches": int(launches) * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": _traffic(f"batched_{len(gs)}", dom, units_per_launch),
                     "peak_source": peak_src, "bytes_per_launch": per_launch_bytes,
                     "accounting": accounting, "us_per_launch": per_launch_s * 1e6,
                     "timing": "replayed frame graph, CUDA event-record nodes around each "
                               "iteration's launches of the phase",
                     "share_of_frame": share},
        "frame_bandwidth_gbs": bytes_per_substep(sz, p, True) * S / (t_batch / args.steps) / 1e9,
        "plain_per_garment": {
            "value": plain_value, "unit": "vertex-substeps/s",
            "garments_timed": len(sample), "frames_each": args.plain_frames,
            "wall_s": round(plain_wall, 1),
            "method": "evenly spaced garments, each alone in its own context (graph replay), "
                      "CUDA events per frame; throughput = sum of vertex-substeps / sum of "
                      "frame times"},
        "batched_over_plain": value / plain_value if plain_value else None,
        "phase_ms_per_frame": phases,
        "setup_s": {"scenes": round(gen_s, 1), "autotune": round(tune_s, 1),
                    "context": round(setup_s, 1), "plain_sample": round(plain_wall, 1)},
        "autotune_trials_ms_per_frame": [[t, dd, vb, round(ms, 2)] for t, dd, vb, ms in trials],
        "clocks": clocks.summary(),
        "wall_s": wall,
    }
    return res


def _cpu_garment_sample(count):
    """Evenly spaced garments of the batched draw for the CPU legs (indices)."""
    from xrtailor_gb300 import autotune
    return autotune.subset(512, count)


def run_cpu_batched(args, frames_per_garment=1, threads=0, sample=8):
    """The oracle (OpenMP port of the plain step) on `sample` evenly spaced garments of the
    batched draw, each in its own oracle solver, `frames_per_garment` frames each after one
    warm-up frame: the sum of vertex-substeps over the sum of frame times."""
    from oracle.oracle import OracleSolver, default_params, lib
    from xrtailor_gb300 import scenes
    idx = _cpu_garment_sample(sample)
    gs = scenes.batched_garments(args.instances, only=idx)
    p = default_params(**scenes.BATCHED_PARAMS)
    t_sum, units = 0.0, 0
    for g in gs:
        o = OracleSolver(p, threads=threads)
        o.add_cloth(g.cloth)
        o.add_obstacle(g.body.mesh)
        o.set_compliance(0, np.full(g.num_edges, g.stretch_compliance, np.float32))
        o.start()
        o.set_obstacle_targets(g.body.pose(1 / 60.0))
        o.step()
        t0 = time.perf_counter()
        for f in range(frames_per_garment):
            o.set_obstacle_targets(g.body.pose((f + 2) / 60.0))
            o.step()
        t_sum += time.perf_counter() - t0
        units += len(g.cloth.positions) * p.num_substeps * frames_per_garment
        o.close()
    return units / t_sum, lib().orc_num_threads(), t_sum, idx


def run_diff(args, local_rank):
    """The differentiation workload: `--diff-instances` sheets of `--diff-n`^2 vertices in one
    batched context, each pinned along its top edge and falling onto its own sphere, rolled out
    `--diff-frames` frames of 10 substeps.  The target rollout uses the seeded ground truth
    (per-edge stretch and per-bend compliance, masses); each timed step is one gradient
    evaluation from a uniform guess: the forward rollout with per-frame checkpoints, the L2 loss
    against the target on the host, and the reverse pass (xrt_backward: replay + adjoint)."""
    import torch
    from xrtailor_gb300 import ClothSolver, build as xb, scenes
    from xrtailor_gb300.diff import rollout as torch_rollout
    xb.build()
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    insts = scenes.diff_batch(args.diff_instances, args.diff_n)
    p = scenes._params(**scenes.DIFF_PARAMS)
    S, F = p.num_substeps, args.diff_frames
    s = ClothSolver(p, device=local_rank)
    for d in insts:
        s.add_instance(d.cloth, d.sphere)
    s.start()
    sz = s.sizes()
    V, E, B = sz.num_vertices, sz.num_edges, sz.num_bends
    cat = lambda f: np.concatenate([f(d) for d in insts])  # noqa: E731
    x0, v0 = cat(lambda d: d.cloth.positions), cat(lambda d: d.velocity)
    comp_true, bcomp_true = cat(lambda d: d.stretch_compliance), cat(lambda d: d.bend_compliance)
    mass = cat(lambda d: d.mass)
    assert (len(comp_true), len(bcomp_true)) == (E, B)
    pinned = s.inv_mass() == 0.0
    w = np.where(pinned, 0.0, 1.0 / mass).astype(np.float32)
    comp_guess = np.full(E, 1e-6, np.float32)
    bcomp_guess = np.full(B, 100.0, np.float32)
    _, _, sp = s.device_state()
    stream = torch.cuda.ExternalStream(sp, device=dev)

    def forward(comp, bcomp, record):
        s.set_compliance(0, comp)
        s.set_compliance(1, bcomp)
        s.set_inv_mass(w)
        s.set_state(x0, v0)
        if record:
            s.diff_begin()
        s.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            s.step(F)
            b.record(stream)
        torch.cuda.synchronize()
        return s.host_positions(), a.elapsed_time(b) / 1e3

    x_target, _ = forward(comp_true, bcomp_true, False)

    def evaluate():
        xf, t_fwd = forward(comp_guess, bcomp_guess, True)
        dL = 2.0 * (xf - x_target)
        loss = float((dL * dL).sum() / 4.0)
        t0 = time.perf_counter()
        g = s.backward(dL)
        t_bwd = time.perf_counter() - t0
        return loss, g, t_fwd, t_bwd

    for _ in range(args.warmup):
        evaluate()
    _, t_plain = forward(comp_guess, bcomp_guess, False)
    rec = []
    with ClockSampler(local_rank) as clocks:
        for _ in range(args.steps):
            loss, g, t_fwd, t_bwd = evaluate()
            rec.append((t_fwd, t_bwd))
    # per-phase profile of one more evaluation (eager frames, CUDA events around each phase)
    s.set_profiling(True)
    evaluate()
    prof = s.profile()
    s.set_profiling(False)
    phases = {k: round(v["ms"] / F, 3) for k, v in prof.items()
              if k != "frames" and v["launches"]}
    s.diff_end()
    t_fwd = float(np.mean([r[0] for r in rec]))
    t_bwd = float(np.mean([r[1] for r in rec]))
    units = V * S * F
    value = units / (t_fwd + t_bwd)
    # end to end: the torch.autograd binding with host tensors (uploads, reverse pass, readback)
    tt = {k: torch.tensor(a, requires_grad=True) for k, a in
          (("x0", x0), ("v0", v0), ("mass", mass), ("comp", comp_guess), ("bcomp", bcomp_guess))}
    xt = torch.from_numpy(x_target)
    t0 = time.perf_counter()
    xf, _ = torch_rollout(s, F, tt["x0"], tt["v0"], tt["mass"], tt["comp"], tt["bcomp"])
    ((xf - xt) ** 2).sum().backward()
    t_e2e = time.perf_counter() - t0
    s.diff_end()
    grads = {"stretch_compliance": g["stretch_compliance"], "bend_compliance": g["bend_compliance"],
             "mass": g["mass"][~pinned], "velocity": g["velocity"]}
    s.close()
    return {
        "metric": "vertex-substeps/s (forward + reverse)", "value": value,
        "unit": "vertex-substeps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * (t_fwd + t_bwd), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded: xrtailor_gb300/scenes.py diff_batch)",
        "config": {"workload": f"diff_{len(insts)}x{args.diff_n}", "instances": len(insts),
                   "vertices": V, "edges": E, "bends": B, "frames": F, "substeps": S,
                   "iterations": p.num_iterations, "collision_passes": p.num_collision_passes,
                   "checkpoint": "every frame (10 substeps)",
                   "l2": "working set (tape) far larger than L2", "parallelism": "single"},
        "forward_s": t_fwd, "forward_plain_s": t_plain, "backward_s": t_bwd,
        "backward_over_forward": t_bwd / t_plain,
        "backward_over_recorded_forward": t_bwd / t_fwd,
        "loss": loss,
        "phase_ms_per_frame": phases,
        "grad_norms": {k: float(np.linalg.norm(v)) for k, v in grads.items()},
        "grads_finite": bool(all(np.isfinite(v).all() for v in grads.values())),
        "e2e": {"value": units / t_e2e, "unit": "vertex-substeps/s",
                "h2d_bytes_per_step": int(4 * (2 * 3 * V + V + E + B) + 4 * 3 * V),
                "d2h_bytes_per_step": int(4 * (3 * V + 3 * V + V + E + B + 3 * V)),
                "path": "xrtailor_gb300.diff.rollout + torch backward, host tensors"},
        "clocks": clocks.summary(),
    }


# Algorithmic bytes per object of the LBVH (fp32, index 4 B): build = primitive read 36 + leaf
# box 24 + Morton code 4 + radix sort (key + value, read + write, 4 passes of 8 bits) 128 +
# node 16 + internal box 24; refit = predicted primitive read 36 + leaf box 24 + internal box 24.
LBVH_BUILD_BYTES = 36 + 24 + 4 + 2 * (4 + 4) * 4 * 2 + 16 + 24
LBVH_REFIT_BYTES = 36 + 24 + 24


def run_lbvh(args, local_rank):
    """The LBVH of the 1024 x 1024 sheet (2,093,058 triangles): BVH::UpdateData + Construct and
    the per-pass refit (BVH::RefitMidstep) from device buffers.  One step = one build + one
    refit, each timed with CUDA events on its own stream; L2 flushed (512 MiB write) before each
    launch group, outside the events."""
    import torch
    from xrtailor_gb300 import Lbvh, build as xb, scenes
    xb.build()
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    sc = scenes.plain_heavy(1024)
    pos = sc.cloth.positions.astype(np.float32)
    tri = sc.cloth.triangles.astype(np.int64)
    prims = torch.from_numpy(pos[tri].reshape(-1, 9).copy()).to(dev)
    n = prims.shape[0]
    rng = np.random.default_rng(3)
    shift = torch.from_numpy(rng.uniform(-1e-3, 1e-3, size=(len(pos), 3)).astype(np.float32))
    pred = torch.from_numpy((pos + shift.numpy())[tri].reshape(-1, 9).copy()).to(dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    b = Lbvh(local_rank)
    for _ in range(max(args.warmup, 1)):
        b.build_device(prims.data_ptr(), n, pred.data_ptr(), 0.0, sp)
        b.refit_device(pred.data_ptr(), sp)
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    with ClockSampler(local_rank) as clocks:
        for e in ev:
            flush.zero_()
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e[0].record(stream)
                b.build_device(prims.data_ptr(), n, pred.data_ptr(), 0.0, sp)
                e[1].record(stream)
            torch.cuda.synchronize()
            flush.zero_()
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e[2].record(stream)
                b.refit_device(pred.data_ptr(), sp)
                e[3].record(stream)
            torch.cuda.synchronize()
    t_build = statistics.median(e[0].elapsed_time(e[1]) for e in ev) / 1e3
    t_refit = statistics.median(e[2].elapsed_time(e[3]) for e in ev) / 1e3
    peak, peak_kind = _peaks()
    gb_build = n * LBVH_BUILD_BYTES / t_build / 1e9
    gb_refit = n * LBVH_REFIT_BYTES / t_refit / 1e9
    b.close()
    return {
        "metric": "LBVH build GB/s (algorithmic bytes)", "value": gb_build, "unit": "GB/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * (t_build + t_refit), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 boxes, u32 codes",
        "data": "synthetic (seeded: xrtailor_gb300/scenes.py plain_heavy, 1024 x 1024 sheet)",
        "config": {"workload": "lbvh_1024x1024", "objects": n,
                   "l2": "flushed before each build and each refit (512 MiB write)",
                   "parallelism": "single"},
        "build": {"ms": 1e3 * t_build, "objects_per_s": n / t_build, "GB/s": gb_build,
                  "bytes_per_object": LBVH_BUILD_BYTES},
        "refit": {"ms": 1e3 * t_refit, "objects_per_s": n / t_refit, "GB/s": gb_refit,
                  "bytes_per_object": LBVH_REFIT_BYTES},
        "roofline": {"bound": "hbm", "achieved": gb_build, "peak": peak, "unit": "GB/s",
                     "frac": gb_build / peak, "peak_kind": peak_kind,
                     "refit_frac": gb_refit / peak},
        "clocks": clocks.summary(),
    }


def _impact_state(n, solver):
    """The impact-zone workload: an n x n sheet (two pinned corners) draped for 4 frames over the
    radius-0.3 icosphere, then predicted positions 0.12 below: every vertex over the sphere's cap
    crosses it within the step."""
    from xrtailor_gb300 import scenes
    cloth = scenes.grid_cloth(n, 1.0, origin=(0.0, 0.35, 0.0), jitter=1e-3, seed=1)
    cloth.fixed_indices = scenes.two_corner_pins(n)
    solver.add_cloth(cloth)
    solver.add_obstacle(scenes.icosphere(2, 0.3, center=(0.5, 0.0, 0.5)))
    solver.start()
    for _ in range(4):
        solver.step()
    x = solver.host_positions()
    pred = x.copy()
    pred[:, 1] -= 0.12
    return pred


def _impact_params():
    from xrtailor_gb300 import scenes
    return scenes._params(num_substeps=2, num_iterations=3, solve_bending=0,
                          num_collision_passes=2, enable_self_collision=0)


def run_impact(args, local_rank):
    """ImpactZoneOptimization::CollisionStep (xrt_collision_step): one step = restore the crossing
    predicted positions, then the whole collision step (passes of pairs + CCD + zone solves until
    no impact remains).  Host-driven (impact counts are read back per pass, as in the reference),
    so it is timed on the wall clock around synchronised calls."""
    import torch
    from xrtailor_gb300 import ClothSolver, build as xb
    xb.build()
    torch.cuda.set_device(local_rank)
    g = ClothSolver(_impact_params(), device=local_rank)
    pred = _impact_state(args.impact_n, g)
    for _ in range(args.warmup):
        g.set_predicted(pred)
        st = g.collision_step()
    g.synchronize()
    times = []
    with ClockSampler(local_rank) as clocks:
        for _ in range(args.steps):
            g.set_predicted(pred)
            g.synchronize()
            t0 = time.perf_counter()
            st = g.collision_step()
            g.synchronize()
            times.append(time.perf_counter() - t0)
    # end to end: host positions in, collision step, host positions out
    e0 = time.perf_counter()
    for _ in range(args.steps):
        g.set_predicted(pred)
        g.collision_step()
        out = g.predicted()
    e2e_s = (time.perf_counter() - e0) / args.steps
    step_s = sum(times) / len(times)
    V = g.sizes().num_vertices
    res = {"metric": "impact-zone collision steps per second", "value": 1.0 / step_s,
           "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "replicas only",
           "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded sheet and icosphere, bench.py _impact_state)",
           "config": {"workload": f"impact_zone_sheet{args.impact_n}", "vertices": V,
                      "obstacle": "icosphere(2), r = 0.3", "crossing": "0.12 below x0",
                      "stats": st},
           "e2e": {"value": 1.0 / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": int(pred.nbytes),
                   "d2h_bytes_per_step": int(out.nbytes)},
           "gpu_launches": None, "roofline": None, "clocks": clocks.summary()}
    if not args.no_cpu_baseline:
        from oracle.oracle import OracleSolver, lib
        o = OracleSolver(_impact_params())
        opred = _impact_state(args.impact_n, o)
        o.set_predicted(opred)
        c0 = time.perf_counter()
        so = o.collision_step()
        ct = time.perf_counter() - c0
        res["cpu_baseline"] = {"value": 1.0 / ct, "unit": "steps/s", "cores": 1, "kind": "port",
                               "sample": f"1 collision step of the same state ({ct:.1f} s)",
                               "same_stats": so == st}
    return res


def _quality(p):
    """SimulateQuality's configuration on top of a workload's parameters (the FEM fabric is set
    by the caller): imminent + PBD repulsion, the impact-zone step, no particle hash."""
    p.enable_self_collision = 0
    p.imminent_repulsion = 1
    p.pbd_repulsion = 1
    p.impact_zone = 1


def _oracle_params(sc, quality=False):
    """The scene's parameters over the oracle's own restatement of the reference defaults, so a
    CPU-only run loads nothing from the CUDA library."""
    from oracle.oracle import default_params
    p = default_params(**sc.params)
    if quality:
        _quality(p)
    return p


def run_cpu(workload, frames, warmup=1, threads=0, fem=False, quality=False):
    from oracle.oracle import OracleSolver, default_fem_material, lib
    sc = _workload(workload)
    p = _oracle_params(sc, quality)
    fem = fem or quality
    o = OracleSolver(p, threads=threads)
    if fem:
        o.set_fem_material(default_fem_material())
    _setup(o, sc)
    tg = _targets(sc, warmup + frames)
    V = o.sizes()["num_vertices"]
    fi = 0
    for _ in range(warmup):
        if tg is not None:
            o.set_obstacle_targets(tg[fi])
        fi += 1
        o.step()
    t0 = time.perf_counter()
    for _ in range(frames):
        if tg is not None:
            o.set_obstacle_targets(tg[fi])
        fi += 1
        o.step()
    t = time.perf_counter() - t0
    return V * p.num_substeps * frames / t, lib().orc_num_threads(), t


def _garment_summary(args, local_rank):
    """The 256 x 256 garment (plain step) as extra keys of the batched line."""
    import copy
    a = copy.copy(args)
    a.workload, a.quality, a.material, a.tile_vertices = "garment", False, "swift", None
    a.steps = min(args.steps, 20)
    r = run_ours(a, 0, local_rank, 1)
    keep = ("value", "ms_per_step", "e2e", "roofline", "frame_bandwidth_gbs", "clocks", "config",
            "launch", "autotune")
    out = {k: r[k] for k in keep}
    out["steps"] = a.steps
    return out


def run_reference(args):
    """The reference arm: the oracle (OpenMP port of the reference's plain step; the reference's
    own path is CUDA-only and cannot be built here) on the host cores, each step a bounded sample
    of the workload.  Batched: one frame of each of 8 evenly spaced garments of the batch, each in
    its own solver (the reference steps one scene per solver)."""
    from oracle.oracle import OracleSolver, default_params, lib
    from xrtailor_gb300 import scenes
    steps, warmup = max(args.steps, 1), max(args.warmup, 0)
    if args.workload == "batched":
        idx = _cpu_garment_sample(8)
        gs = scenes.batched_garments(args.instances, only=idx)
        p = default_params(**scenes.BATCHED_PARAMS)
        solvers = []
        for g in gs:
            o = OracleSolver(p)
            o.add_cloth(g.cloth)
            o.add_obstacle(g.body.mesh)
            o.set_compliance(0, np.full(g.num_edges, g.stretch_compliance, np.float32))
            o.start()
            solvers.append(o)
        poses = [[g.body.pose((f + 1) / 60.0) for f in range(warmup + steps)] for g in gs]
        units_step = sum(len(g.cloth.positions) for g in gs) * p.num_substeps
        for f in range(warmup):
            for o, ps in zip(solvers, poses):
                o.set_obstacle_targets(ps[f])
                o.step()
        t0 = time.perf_counter()
        for f in range(warmup, warmup + steps):
            for o, ps in zip(solvers, poses):
                o.set_obstacle_targets(ps[f])
                o.step()
        t = time.perf_counter() - t0
        value = units_step * steps / t
        sample = (f"each step one frame of each of 8 evenly spaced garments of the batch "
                  f"(garments {idx}, {units_step // p.num_substeps} vertices), one oracle "
                  f"solver per garment")
        config = dict(_batched_config(args.instances, p), parallelism="single")
    else:
        fem = args.material == "fem" or args.quality
        value, cores_, t = run_cpu(args.workload, steps, warmup=warmup, fem=fem,
                                   quality=args.quality)
        cfg_p = _oracle_params(_workload(args.workload), args.quality)
        config = dict(_plain_config(args.workload, cfg_p, args.quality, fem), parallelism="single")
        sample = f"{steps} full frames of {config['workload']}"
    cores = lib().orc_num_threads()
    return {"metric": METRIC, "value": value, "unit": "vertex-substeps/s", "n_gpus": 0,
            "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * t / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generators, xrtailor_gb300/scenes.py)",
            "config": config, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "vertex-substeps/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "vertex-substeps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["garment", "small", "heavy", "batched", "diff", "lbvh", "impact"])
    ap.add_argument("--impact-n", type=int, default=128, help="impact workload: sheet size")
    ap.add_argument("--quality", action="store_true",
                    help="plain workloads in SimulateQuality's configuration: FEM fabric, "
                         "imminent + PBD repulsion, impact zones per substep, no particle hash")
    ap.add_argument("--cpu-frames", type=int, default=24,
                    help="frames of the CPU baseline sample (~10 s of the garment on 16 cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--instances", type=int, default=512, help="batched workload: garments")
    ap.add_argument("--no-garment", action="store_true",
                    help="batched workload: skip the 256 x 256 garment's extra keys")
    ap.add_argument("--plain-sample", type=int, default=128,
                    help="batched workload: garments timed alone (evenly spaced)")
    ap.add_argument("--plain-frames", type=int, default=2)
    ap.add_argument("--tune-instances", type=int, default=32,
                    help="batched workload: garments the launch autotuner times (0: library "
                         "defaults)")
    ap.add_argument("--diff-instances", type=int, default=16)
    ap.add_argument("--diff-n", type=int, default=128)
    ap.add_argument("--diff-frames", type=int, default=60)
    ap.add_argument("--material", default="swift", choices=["swift", "fem"],
                    help="plain workloads: the Swift fabric (XPBD stretch + dihedral bend) or "
                         "the FEM fabric (strain + isometric bending, include/xrt_fem.h)")
    ap.add_argument("--tile-vertices", type=int, default=None,
                    help="tile size of the Gauss-Seidel schedule (library default if omitted)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return

    if args.workload == "batched":
        if world > 1:
            # independent replicas of the batch, one per GPU (instances would shard with no
            # exchange step; every GPU runs the whole batch here)
            import torch
            torch.distributed.init_process_group("nccl")
        res = run_batched(args, local_rank)
        if world > 1:
            import torch
            tt = torch.tensor([res["ms_per_step"]], device=f"cuda:{local_rank}")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            res["ms_per_step"] = float(tt.item())
            res["value"] = (res["config"]["vertices"] * res["config"]["substeps"] * world /
                            (res["ms_per_step"] / 1e3))
            res["n_gpus"] = world
            res["config"]["parallelism"] = f"replicas x{world}"
            torch.distributed.destroy_process_group()
        if rank == 0 and not args.no_cpu_baseline:
            v, cores, t, idx = run_cpu_batched(args, frames_per_garment=3, sample=16)
            res["cpu_baseline"] = {"value": v, "unit": "vertex-substeps/s", "cores": cores,
                                   "kind": "port",
                                   "sample": f"3 frames each of 16 evenly spaced garments of the "
                                             f"batch (garments {idx}), one oracle solver per "
                                             f"garment ({t:.1f} s)"}
        if rank == 0 and not args.no_garment:
            res["plain_garment"] = _garment_summary(args, local_rank)
        if rank == 0:
            print(json.dumps(res))
        return
    if args.workload == "diff":
        if rank == 0:
            print(json.dumps(run_diff(args, local_rank)))
        return
    if args.workload == "lbvh":
        if rank == 0:
            print(json.dumps(run_lbvh(args, local_rank)))
        return
    if args.workload == "impact":
        if rank == 0:
            print(json.dumps(run_impact(args, local_rank)))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, local_rank, world)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        frames = 1 if args.quality else args.cpu_frames
        v, cores, t = run_cpu(args.workload, frames, fem=args.material == "fem",
                              quality=args.quality)
        res["cpu_baseline"] = {"value": v, "unit": "vertex-substeps/s", "cores": cores,
                               "kind": "port",
                               "sample": f"{frames} frames of {res['config']['workload']} "
                                         f"({t:.1f} s)"}
    if rank == 0:
        print(json.dumps(res))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
