#!/usr/bin/env python
"""Benchmark: reinitialize_2nd_order node-iterations/s on one GB300, mixed precision vs FP64.

Workload (the 3D flower configuration): octree on [-1,1]^3, levels 5-10, refined where
|phi_exact| <= 1.2*diag(cell) (refine_levelset_cf with lip = 2.4) around r = 0.5 + 0.1 sin(5 theta)
sin(4 phi); phi0 = (r - r_s)(0.2 + |x - (0.1,-0.2,0.15)|^2); reinitialize_2nd_order, 50 iterations.
A step is one 50-iteration reinitialisation of the whole grid; a node-iteration is one node through
one RK2 pseudo-time iteration. Synthetic data (no dataset); the working set (tables + fields, >1 GB)
is far larger than L2, so no L2 flush is needed between steps.

Prints one JSON line (rank 0). `--impl reference` times the CPU restatement of the reference loops
(oracle/, the reference itself needs p4est/PETSc/MPI) on all host cores instead.
"""
from __future__ import annotations

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

ITERS = 50
LEVELS = (5, 10)
METRIC = "reinit node-iters/s on 1 GB300: mixed vs FP64 at stated band L\u221e error; HBM %"
CPU_SAMPLE_ITERS = 10  # bounded CPU sample: about 10 s of 16-core work on the full grid
LIP = 2.4


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--levels", type=int, nargs=2, default=list(LEVELS))
    p.add_argument("--iters", type=int, default=ITERS)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--workload", default="reinit3d", choices=["reinit3d", "reinit2d", "transport3d", "batch2d", "large3d"],
                   help="reinit3d: the headline reinitialisation line; reinit2d: the 2D quadtree configuration (FP64, 20 "
                        "iterations, error against r - 0.5); transport3d: the level-set transport run "
                        "(semi-Lagrangian step + host regrid + 5 reinitialisation iterations per step; --steps time steps); "
                        "batch2d: 256 quadtrees reinitialised together (--steps timed batch calls)")
    p.add_argument("--batch", type=int, default=256, help="batch2d: number of quadtrees")
    p.add_argument("--large-levels", type=int, nargs=2, default=[6, 11], help="large3d: min and max level")
    p.add_argument("--stage-config", default=None,
                   help="reinit3d, large3d: fixed launch shape of the mixed stage instead of the autotuner's, as five to seven "
                        "integers threads_per_block,uniform_blocks,regular_blocks,uniform_depth,window_halo[,streams[,priority]] "
                        "(e.g. 256,0,0,3,512 or 256,912,304,1,512,1)")
    args = p.parse_args()
    if args.fp64_steps < 1:
        p.error("--fp64-steps must be at least 1")
    return args


def parse_stage_config(text):
    v = [int(x) for x in text.split(",")]
    if len(v) not in (5, 6, 7):
        raise SystemExit("--stage-config takes five to seven integers")
    return {"threads_per_block": v[0], "uniform_blocks": v[1], "regular_blocks": v[2], "uniform_depth": v[3], "window_halo": v[4],
            "streams": v[5] if len(v) > 5 else 2, "priority": v[6] if len(v) > 6 else 2}


def build_grid(levels):
    import casl_p4est_gb300 as G
    from casl_p4est_gb300 import shapes
    f = G.my_p4est_brick_new([1, 1, 1], [-1, -1, -1], [1, 1, 1])
    f.refine_levelset(shapes.flower([0, 0, 0], 0.5, 0.1, 5, 4), levels[0], levels[1], lip=LIP)
    f.build_nodes()
    phi0 = f.sample(shapes.flower([0, 0, 0], 0.5, 0.1, 5, 4, scale=(0.2, (0.1, -0.2, 0.15))))
    return f, phi0


def workload_config(args, N, world=1):
    return {"workload": f"3D flower octree [-1,1]^3 levels {args.levels[0]}-{args.levels[1]} (lip 2.4), "
                        f"{N} nodes, reinitialize_2nd_order {args.iters} iterations",
            "nodes": N, "iterations": args.iters,
            "l2": "working set > L2 (no flush needed)", "parallelism": "replicas" if world > 1 else "single GPU"}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic_per_node(kernel):
    """DRAM bytes per node of one launch, from the committed ncu summary (profiles/), if present."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_flower3d.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_node:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
              "clocks.mem,clocks.max.mem,temperature.gpu")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons, mem, mmax, temp = [], [], set(), [], [], []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
            try:
                mem.append(float(parts[9]))
                mmax.append(float(parts[10]))
                temp.append(float(parts[11]))
            except (IndexError, ValueError):
                pass
        if not sm:
            return None
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons), "samples": len(sm)}
        if mem:
            out.update(mem_mhz=statistics.median(mem), mem_max_mhz=max(mmax), temp_c=max(temp))
        return out


def gpu_info(gpu_index):
    """Read-only description of the GPU (which board, its ECC, power-limit and application-clock settings), so that
    lines from different GPUs of the same kind can be told apart."""
    fields = ["name", "uuid", "pci.bus_id", "vbios_version", "driver_version", "ecc.mode.current", "power.limit",
              "clocks.applications.graphics", "clocks.applications.memory", "compute_mode", "mig.mode.current"]
    try:
        out = subprocess.run(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + ",".join(fields), "--format=csv,noheader"],
                             stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=20).stdout.strip()
        vals = [v.strip() for v in out.splitlines()[0].split(",")]
        return dict(zip(fields, vals)) if len(vals) == len(fields) else None
    except Exception:
        return None


def box_copy_bandwidth(stream):
    """Device-to-device copy bandwidth of this GPU (1 GiB, read + written bytes per second), beside the pool's
    measured peak: GPUs of the same kind differ by several percent, and so do the memory-bound kernels on them."""
    import torch
    n = 1 << 28
    x = torch.empty(n, dtype=torch.float32, device="cuda")
    y = torch.empty_like(x)
    x.fill_(1.0)
    for _ in range(3):
        y.copy_(x)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(10):
        y.copy_(x)
    e1.record(stream)
    torch.cuda.synchronize()
    gbs = 10 * 2 * x.numel() * 4 / (e0.elapsed_time(e1) / 1e3) / 1e9
    del x, y
    return gbs


def cpu_reinit_sample(f, phi0, iters, nthreads):
    """The oracle (CPU restatement of reinitialize_2nd_order, its grid and stencils from its own construction)
    on the same grid: `iters` iterations. Returns (seconds, result)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    og = O.OracleGrid.from_forest(f)
    phi = phi0.copy()
    t = time.perf_counter()
    og.reinitialize(phi, 2, 2, iterations=iters, nthreads=nthreads)
    return time.perf_counter() - t, phi


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement of the reference loops (the reference itself needs p4est, PETSc
    and MPI), its grid and stencils from its own construction, on all host cores; every timed step is the
    full workload (all nodes, args.iters iterations); warm-up steps are one iteration each."""
    if rank != 0:
        return
    f, phi0 = build_grid(args.levels)
    N = f.num_nodes
    cores = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    og = O.OracleGrid.from_forest(f)
    for _ in range(args.warmup):
        phi = phi0.copy()
        og.reinitialize(phi, 2, 2, iterations=1, nthreads=cores)
    times = []
    for _ in range(args.steps):
        phi = phi0.copy()
        t = time.perf_counter()
        og.reinitialize(phi, 2, 2, iterations=args.iters, nthreads=cores)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = N * args.iters * args.steps / total
    out = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "node-iters/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, N),
        "cpu_baseline": {"value": value, "unit": "node-iters/s", "cores": cores, "kind": "port",
                         "sample": f"the full workload per timed step: reinitialize_2nd_order, {args.iters} iterations x {N} nodes, "
                                   f"{cores} threads, FP64; CPU restatement of reinitialize_one_iteration/compute_derivatives "
                                   "(oracle/, bit-identical to the reference's own code built from its sources); warm-up steps are "
                                   "1 iteration each"},
        "e2e": {"value": value, "unit": "node-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def negative_volume(f, phi):
    """Volume of {phi < 0}: phi linear on the Kuhn simplices of every leaf (6 tetrahedra in 3D, 2
    triangles in 2D); the fraction of a simplex with vertex values f_i is
    (-1)^(n+1) sum_i max(0,-f_i)^n / prod_{j != i}(f_i - f_j) (Hermite-Genocchi)."""
    import itertools
    dim = f.dim
    tree, level, _ = f.leaves()
    ln = f.local_nodes()
    fv = phi[ln].astype(np.float64)
    span = (np.array(f.xyz_max[:dim]) - np.array(f.xyz_min[:dim])) / np.array(f.n_xyz[:dim])
    vol = np.prod(span) * (0.5 ** level.astype(np.float64)) ** dim
    scale = np.max(np.abs(fv), axis=1, keepdims=True) + 1e-300
    fv = fv + 1e-12 * scale * np.arange(fv.shape[1])[None, :]  # separate equal values
    frac = np.zeros(len(level))
    for perm in itertools.permutations(range(dim)):
        verts = [0]
        for a in perm:
            verts.append(verts[-1] | (1 << a))
        fs = fv[:, verts]
        acc = np.zeros(len(level))
        for i in range(dim + 1):
            den = np.ones(len(level))
            for j in range(dim + 1):
                if j != i:
                    den *= fs[:, i] - fs[:, j]
            acc += np.maximum(0.0, -fs[:, i]) ** dim / den
        frac += (acc if dim % 2 == 0 else -acc)
    n_simplex = 6 if dim == 3 else 2
    return float(np.sum(vol * frac / n_simplex))


def run_transport(args):
    """Level-set transport (3D): octree levels 5-9 on [0,1]^3 around the sphere R = 0.15 at
    (0.35,0.35,0.35); single-vortex velocity u = 2 sin^2(pi x) sin(2 pi y) sin(2 pi z) cos(pi t/T), ...,
    T = 3; dt = dx_min; per step update_p4est (semi-Lagrangian RK2 backtrace with quadratic node
    interpolation + host regrid until the grid settles, velocity at the step's midpoint), a new level
    set on the new grid, and 5 reinitialisation iterations; mixed and FP64 runs side by side. The fields
    stay on the GPU: node numbering, node coordinates, refinement tags and the node-neighbour tables are
    computed there, and only the tags (one byte per leaf) go to the host for its regrid passes."""
    import math

    import torch
    import casl_p4est_gb300 as G
    torch.cuda.set_device(0)
    lmin, lmax, T = 5, 9, 3.0
    sphere = G.shapes.sphere([0.35, 0.35, 0.35], 0.15)
    f0 = G.my_p4est_brick_new([1, 1, 1], [0, 0, 0], [1, 1, 1])
    f0.refine_levelset(sphere, lmin, lmax, lip=1.2)
    f0.build_nodes()
    dmin = 1.0 / (1 << lmax)
    dt = dmin

    def gpu_loop(prec, steps):
        f = f0.copy()
        phi_h = f.sample(sphere)
        vol0 = negative_volume(f, phi_h)
        phi = torch.from_numpy(phi_h).cuda()
        t = 0.0
        times = {"update_p4est": 0.0, "level_set_setup": 0.0, "reinit": 0.0}
        nodes = []
        ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), device_build=True)
        regrid_iters = 0
        torch.cuda.synchronize()
        t_all = time.perf_counter()
        for step in range(steps):
            t0 = time.perf_counter()
            sl = G.my_p4est_semi_lagrangian_t(f.copy(), ls, splitting=(lmin, lmax, 1.2))
            phi = sl.update_p4est(G.VortexVelocity(math.cos(math.pi * (t + 0.5 * dt) / T)), dt, phi)  # device fields
            regrid_iters += sl.iterations
            f = sl.forest_np1
            t1 = time.perf_counter()
            ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), device_build=True)
            ls.set_stream(torch.cuda.current_stream().cuda_stream)
            t2 = time.perf_counter()
            ls.reinitialize_2nd_order(phi, 5, precision=prec)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            times["update_p4est"] += t1 - t0
            times["level_set_setup"] += t2 - t1
            times["reinit"] += t3 - t2
            nodes.append(f.num_nodes)
            t += dt
        wall = time.perf_counter() - t_all
        phi = phi.cpu().numpy()
        return {"forest": f, "phi": phi, "ls": ls, "vol0": vol0, "vol": negative_volume(f, phi), "wall_s": wall,
                "times_s": times, "nodes_mean": float(np.mean(nodes)), "nodes_last": nodes[-1],
                "regrid_iterations": regrid_iters, "t_final": t}

    def cpu_loop(steps, nthreads):
        """The same steps on the host: the CPU restatement of the semi-Lagrangian step and of the
        reinitialisation (oracle/) on all host cores, the regrid and node numbering by the host forest code,
        the node-neighbour construction by the restatement."""
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        f = f0.copy()
        phi = f.sample(sphere)
        og = O.OracleGrid.from_forest(f)
        t = 0.0
        t_all = time.perf_counter()
        for step in range(steps):
            scale = math.cos(math.pi * (t + 0.5 * dt) / T)
            g = f.copy()
            while True:
                new = og.sl_advect_vortex(g.node_xyz(), dt, scale, phi, nthreads=nthreads)
                if not g.refine_and_coarsen(lmin, lmax, new, lip=1.2):
                    break
                g.build_nodes()
            f, phi = g, new
            og = O.OracleGrid.from_forest(f)
            og.reinitialize(phi, 2, 2, iterations=5, nthreads=nthreads)
            t += dt
        return f, phi, time.perf_counter() - t_all

    results = {prec: gpu_loop(prec, args.steps) for prec in ("mixed", "fp64")}
    m, d = results["mixed"], results["fp64"]
    # FP64 result on the mixed run's final nodes (quadratic node interpolation), compared in the band
    interp = G.my_p4est_interpolation_nodes_t(d["ls"])
    d_on_m = interp.interpolate_points(m["forest"].node_xyz(), d["phi"], G.interpolation.quadratic_non_oscillatory_continuous_v2)
    band = np.abs(d_on_m) < 3 * dmin
    band_err = float(np.max(np.abs(m["phi"][band] - d_on_m[band]))) if band.any() else 0.0
    ms_step = 1e3 * m["wall_s"] / args.steps
    out = {
        "metric": "level-set transport time per step (semi-Lagrangian + regrid + 5 reinit iterations)",
        "value": ms_step, "unit": "ms/step", "n_gpus": 1, "steps": args.steps, "warmup": 0, "ms_per_step": ms_step,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64 interpolation, f32 mixed reinit",
        "data": "synthetic",
        "config": {"workload": f"3D transport: octree levels {lmin}-{lmax} on [0,1]^3, sphere R=0.15 at (0.35,0.35,0.35), "
                               f"single vortex T=3, dt=dx_min={dmin}, {args.steps} steps, 5 reinit iterations per step",
                   "nodes_mean": m["nodes_mean"], "nodes_last": m["nodes_last"], "t_final": m["t_final"],
                   "velocity_time": "cos(pi t/T) at the step midpoint"},
        "mixed": {"ms_per_step": ms_step, "breakdown_s": m["times_s"], "volume_loss_rel": (m["vol"] - m["vol0"]) / m["vol0"],
                  "regrid_iterations": m["regrid_iterations"]},
        "fp64": {"ms_per_step": 1e3 * d["wall_s"] / args.steps, "breakdown_s": d["times_s"],
                 "volume_loss_rel": (d["vol"] - d["vol0"]) / d["vol0"], "regrid_iterations": d["regrid_iterations"]},
        "band_linf_mixed_vs_fp64": band_err, "band_linf_over_dx_min": band_err / dmin,
        "same_final_grid": bool(m["forest"].num_leaves == d["forest"].num_leaves
                                and np.array_equal(m["forest"].leaves()[2], d["forest"].leaves()[2])),
    }
    # CPU baseline: a bounded sample of the same steps on the host cores, and the FP64 GPU path over the same
    # steps for comparison (the GPU evaluates the vortex velocity with its own sin/cos, so the two agree to
    # rounding, not bit for bit)
    k = min(args.steps, 10)
    cores = os.cpu_count() or 1
    f_cpu, phi_cpu, cpu_s = cpu_loop(k, cores)
    ref = results["fp64"] if k == args.steps else gpu_loop("fp64", k)
    same_grid = bool(f_cpu.num_leaves == ref["forest"].num_leaves and np.array_equal(f_cpu.leaves()[2], ref["forest"].leaves()[2]))
    out["cpu_baseline"] = {"value": 1e3 * cpu_s / k, "unit": "ms/step", "cores": cores, "kind": "port",
                           "sample": f"the first {k} steps of the same run on the host: the CPU restatement (oracle/) of the "
                                     "semi-Lagrangian step, the node-neighbour construction and 5 reinitialisation iterations on "
                                     f"{cores} threads, the regrid and node numbering by the host forest code"}
    out["cpu_vs_gpu_fp64"] = {"steps": k, "same_grid": same_grid,
                              "max_abs_diff": float(np.max(np.abs(phi_cpu - ref["phi"]))) if same_grid else None,
                              "gpu_fp64_ms_per_step": 1e3 * ref["wall_s"] / k}
    print(json.dumps(out), flush=True)


BATCH_LIP = 14.4  # refinement band |d| <= 7.2 diag: node counts from 4.2k (level 6) to about 420k (level 11)


def batch_grids(count, seed=2024):
    """256 independent quadtrees on [-1,1]^2: levels 6..lmax with lmax uniform in 6..11, refined where
    |d| <= 7.2 diag (lip 14.4, so that the node counts span the configuration's 5k-400k) for d the
    distance to the ellipses; phi0 the min signed distance to 1-8 random ellipses (centres U[-0.6,0.6],
    semi-axes U[0.05,0.4], random rotation) times 0.1 + U[0.5,1.5]*|x-(a,b)|^2 with (a,b) U[-0.5,0.5]."""
    import casl_p4est_gb300 as G
    from casl_p4est_gb300 import shapes
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        lmax = int(rng.integers(6, 12))
        items = [(rng.uniform(-0.6, 0.6), rng.uniform(-0.6, 0.6), rng.uniform(0.05, 0.4), rng.uniform(0.05, 0.4),
                  rng.uniform(0, np.pi)) for _ in range(int(rng.integers(1, 9)))]
        scale = (0.1, (rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5)), rng.uniform(0.5, 1.5))
        f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
        f.refine_levelset(shapes.ellipses(items), 6, lmax, lip=BATCH_LIP)
        f.build_nodes()
        out.append((f, f.sample(shapes.ellipses(items, scale=scale)), lmax))
    return out


def run_batch(args):
    """Batched 2D reinitialisation: all grids' tables concatenated, 30 iterations of every grid in one
    CUDA graph of batched launches, launch shape from the autotuner; against the same grids
    reinitialised one call per grid."""
    import torch
    import casl_p4est_gb300 as G
    torch.cuda.set_device(0)
    iters = 30
    t0 = time.perf_counter()
    grids = batch_grids(args.batch)
    t1 = time.perf_counter()
    b = G.my_p4est_level_set_batch_t([g[0] for g in grids], device_build=True)
    torch.cuda.synchronize()
    setup_s = {"grids": t1 - t0, "tables": time.perf_counter() - t1, "note": "host refinement and node numbering; tables on the GPU"}
    N = b.num_nodes
    stream = torch.cuda.current_stream()
    b.set_stream(stream.cuda_stream)
    phi0 = torch.from_numpy(b.concat([g[1] for g in grids])).cuda()
    cfg = b.autotune(phi0.cpu().numpy(), trials=3)
    phi = torch.empty_like(phi0)

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            phi.copy_(phi0)
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(steps):
            phi.copy_(phi0)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        return total / steps

    ms_graph = timed(lambda: b.reinitialize_2nd_order(phi, iters, use_graph=True), args.steps, args.warmup)
    batched = phi.cpu().numpy().copy()
    ms_nograph = timed(lambda: b.reinitialize_2nd_order(phi, iters, use_graph=False), args.steps, args.warmup)
    # the same grids one call per grid (each its own level-set object, same stream)
    singles = []
    for f, p0, _ in grids:
        ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), precision="mixed")
        ls.set_stream(stream.cuda_stream)
        singles.append(ls)
    views = [phi[int(b.offsets[k]):int(b.offsets[k + 1])] for k in range(b.count)]

    def one_by_one():
        for ls, v in zip(singles, views):
            ls.reinitialize_2nd_order(v, iters)

    ms_single = timed(one_by_one, max(1, args.steps // 2), 1)
    same = bool(np.array_equal(phi.cpu().numpy(), batched))
    # accuracy of every grid against its own FP64 reinitialisation: band L-infinity and interface location
    dmin_err = 0.0
    iface_err = 0.0
    mismatched = 0
    parts = b.split(batched)
    for k in range(b.count):
        f, p0, lmax = grids[k]
        ls64 = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
        ref = p0.copy()
        ls64.reinitialize_2nd_order(ref, iters, precision="fp64")
        dx = 2.0 / (1 << lmax)
        got = parts[k]
        band = np.abs(ref) < 3 * dx
        if band.any():
            dmin_err = max(dmin_err, float(np.max(np.abs(got[band] - ref[band]))) / dx)
        loc, _, mis = ls64.interface_location_error(torch.from_numpy(got).cuda(), torch.from_numpy(ref).cuda())
        iface_err = max(iface_err, loc / dx)
        mismatched += mis
    node_iters = N * iters
    out = {
        "metric": f"batched reinit node-iters/s ({b.count} quadtrees, one CUDA graph)", "value": node_iters / (ms_graph / 1e3),
        "unit": "node-iters/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_graph,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{b.count} quadtrees on [-1,1]^2, max level U{{6..11}}, union of 1-8 random ellipses, refined where "
                               f"|d| <= 7.2 diag, reinitialize_2nd_order {iters} iterations each, mixed", "nodes_total": N,
                   "nodes_min": int(np.min(np.diff(b.offsets))), "nodes_max": int(np.max(np.diff(b.offsets))),
                   "l2": "working set > L2 (no flush needed)"},
        "autotuned_stage_config": cfg,
        "batched_no_graph": {"ms": ms_nograph, "value": node_iters / (ms_nograph / 1e3)},
        "one_call_per_grid": {"ms": ms_single, "value": node_iters / (ms_single / 1e3)},
        "speedup_graph_vs_one_call_per_grid": ms_single / ms_graph,
        "one_call_per_grid_equals_batched": same,
        "band_linf_vs_fp64_over_dx_min": dmin_err, "interface_location_err_over_dx_min": iface_err,
        "interface_sign_mismatches": mismatched, "accuracy_checked_grids": b.count, "setup_s": setup_s,
        "box_copy_GBps": box_copy_bandwidth(stream),
    }
    print(json.dumps(out), flush=True)


def run_large(args):
    """Large 3D: octree on [-1,1]^3 around 64 random spheres (centres U[-0.8,0.8]^3, radii U[0.05,0.15],
    seed 5), refined where |d| <= 1.2 diag; phi0 = min signed distance x (0.1 + |x - c0|^2);
    reinitialize_2nd_order 50 iterations and advect_in_normal_direction with vn = 1 for 20 steps,
    mixed and FP64, on one GPU."""
    import torch
    import casl_p4est_gb300 as G
    from casl_p4est_gb300 import shapes
    torch.cuda.set_device(0)
    lmin, lmax = args.large_levels
    rng = np.random.default_rng(5)
    centres = rng.uniform(-0.8, 0.8, (64, 3))
    radii = rng.uniform(0.05, 0.15, 64)
    t0 = time.perf_counter()
    f = G.my_p4est_brick_new([1, 1, 1], [-1, -1, -1], [1, 1, 1])
    f.refine_levelset(shapes.spheres(centres, radii), lmin, lmax, lip=LIP)
    f.build_nodes(device=True)
    torch.cuda.synchronize()
    t_grid = time.perf_counter() - t0
    phi0 = f.sample(shapes.spheres(centres, radii, scale=(0.1, centres[0])))
    N = f.num_nodes
    t0 = time.perf_counter()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), precision="mixed", device_build=True)
    torch.cuda.synchronize()
    t_tables = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    ls.set_stream(stream.cuda_stream)
    _, dmin, _ = f.dxyz_min(lmax)
    if args.stage_config:
        ls.stage_config = parse_stage_config(args.stage_config)
        cfg = dict(ls.stage_config, fixed=True)
    else:
        cfg = ls.autotune(phi0, trials=2)
    phi0_d = torch.from_numpy(phi0).cuda()
    del phi0
    phi_d = torch.empty_like(phi0_d)
    iters = 50

    def timed(fn, steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(steps):
            phi_d.copy_(phi0_d)
            torch.cuda.synchronize()
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        return total / steps

    reinit = lambda prec: ls.reinitialize_2nd_order(phi_d, iters, precision=prec)
    phi_d.copy_(phi0_d)
    reinit("mixed")  # warm-up
    ms_mixed = timed(lambda: reinit("mixed"), args.steps)
    mixed_d = phi_d.clone()
    ms_fp64 = timed(lambda: reinit("fp64"), 1)
    band_err, band_nodes = ls.band_linf(mixed_d, phi_d, 3 * dmin)
    near_err, _ = ls.band_linf(mixed_d, phi_d, dmin)
    iface_loc, iface_edges, iface_mismatch = ls.interface_location_error(mixed_d, phi_d)
    del mixed_d
    # normal advection, vn = 1, 20 steps from the reinitialised field
    vn = torch.ones_like(phi0_d)
    dt = 0.8 * dmin  # CFL 0.8 on the finest cells (vn = 1)
    adv_ms = {}
    adv_out = {}
    for prec in ("mixed", "fp64"):
        start = phi_d.clone()

        def adv():
            for _ in range(20):
                ls.advect_in_normal_direction(vn, phi_d, dt, precision=prec)

        phi_d.copy_(start)
        adv()  # warm-up
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        phi_d.copy_(start)
        e0.record(stream)
        adv()
        e1.record(stream)
        torch.cuda.synchronize()
        adv_ms[prec] = e0.elapsed_time(e1)
        adv_out[prec] = phi_d.clone()
        phi_d.copy_(start)
    adv_err, _ = ls.band_linf(adv_out["mixed"], adv_out["fp64"], 3 * dmin)
    peak, peak_kind = measured_peak()
    value = N * iters / (ms_mixed / 1e3)
    gbs = 284 * value / 1e9
    out = {
        "metric": "large-grid reinit node-iters/s on 1 GB300 (mixed vs FP64) + normal advection", "value": value,
        "unit": "node-iters/s", "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": ms_mixed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"3D octree [-1,1]^3 levels {lmin}-{lmax} (lip 2.4) around 64 random spheres, {N} nodes, "
                               f"reinitialize_2nd_order {iters} iterations + advect_in_normal_direction vn=1 x 20",
                   "nodes": N, "leaves": f.num_leaves, "l2": "working set > L2 (no flush needed)"},
        "fp64": {"ms_per_step": ms_fp64, "value": N * iters / (ms_fp64 / 1e3)},
        "speedup_mixed_vs_fp64": ms_fp64 / ms_mixed,
        "band_linf_vs_fp64": band_err, "band_linf_over_dx_min": band_err / dmin, "band_linf_near_interface_vs_fp64": near_err,
        "interface_location_err_vs_fp64": iface_loc, "interface_location_err_over_dx_min": iface_loc / dmin,
        "interface_cut_edges": iface_edges, "interface_sign_mismatches": iface_mismatch,
        "band_nodes": band_nodes, "dx_min": dmin,
        "roofline_per_iteration": {"alg_bytes_per_node_iter": 284, "achieved_GBps": gbs, "peak": peak, "frac": gbs / peak,
                                   "peak_source": peak_kind},
        "advect_20_steps": {"mixed_ms": adv_ms["mixed"], "fp64_ms": adv_ms["fp64"],
                            "mixed_node_steps_per_s": N * 20 / (adv_ms["mixed"] / 1e3),
                            "fp64_node_steps_per_s": N * 20 / (adv_ms["fp64"] / 1e3),
                            "band_linf_mixed_vs_fp64": adv_err, "dt": dt},
        "autotuned_stage_config": cfg, "box_copy_GBps": box_copy_bandwidth(stream),
        "setup_s": {"grid": t_grid, "tables": t_tables, "note": "host refinement, node numbering and tables on the GPU"},
        "device_memory_used_gb": (lambda fr: (fr[1] - fr[0]) / 1e9)(torch.cuda.mem_get_info()),
    }
    print(json.dumps(out), flush=True)


def run_reinit2d(args):
    """The 2D configuration: quadtree on [-1,1]^2, levels 4-9, refined where |r - 0.5| <= 1.2 diag (lip 2.4);
    phi0 = (r - 0.5)(0.1 + (x-0.2)^2 + (y-0.3)^2); reinitialize_2nd_order, 20 iterations, FP64. Error
    max |phi - (r - 0.5)| over |phi| < 3 dx_min (and over |phi| < 3 diag_min, the example's band). The FP64
    GPU path, the mixed path and the CPU restatement (all host cores and one core) on the same grid; the FP64
    GPU result must equal the CPU result bit for bit."""
    import torch
    import casl_p4est_gb300 as G
    from casl_p4est_gb300 import shapes
    torch.cuda.set_device(0)
    iters, lmin, lmax = 20, 4, 9
    f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
    f.refine_levelset(shapes.sphere([0, 0], 0.5), lmin, lmax, lip=LIP)
    f.build_nodes()
    phi0 = f.sample(shapes.sphere_scaled([0, 0], 0.5, 0.1, [0.2, 0.3]))
    N = f.num_nodes
    x = f.node_xyz()
    exact = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2) - 0.5
    _, dmin, diag = f.dxyz_min(lmax)
    stream = torch.cuda.current_stream()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    ls.set_stream(stream.cuda_stream)
    phi0_d = torch.from_numpy(phi0).cuda()
    phi_d = torch.empty_like(phi0_d)

    def gpu(prec, steps):
        for _ in range(args.warmup):
            phi_d.copy_(phi0_d)
            ls.reinitialize_2nd_order(phi_d, iters, precision=prec)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(steps):
            phi_d.copy_(phi0_d)
            e0.record(stream)
            ls.reinitialize_2nd_order(phi_d, iters, precision=prec)
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        return total / steps, phi_d.cpu().numpy()

    ms64, p64 = gpu("fp64", args.steps)
    ms32, p32 = gpu("mixed", args.steps)
    cores = os.cpu_count() or 1
    cpu = {}
    for nt in (cores, 1):
        reps = 5 if nt > 1 else 2
        best = None
        for _ in range(reps):
            s, pc = cpu_reinit_sample(f, phi0, iters, nt)
            best = s if best is None else min(best, s)
        cpu[nt] = (best, pc)

    def err(p, band):
        m = np.abs(p) < band
        return float(np.max(np.abs(p[m] - exact[m])))

    band = np.abs(p64) < 3 * dmin
    out = {
        "metric": "reinit node-iters/s, 2D quadtree L4-9, 20 iterations (FP64 GPU vs CPU restatement) and error vs r-0.5",
        "value": N * iters / (ms64 / 1e3), "unit": "node-iters/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"2D quadtree [-1,1]^2 levels {lmin}-{lmax} (lip 2.4), {N} nodes, phi0 = (r-0.5)(0.1+(x-0.2)^2+(y-0.3)^2), "
                               f"reinitialize_2nd_order {iters} iterations", "nodes": N, "iterations": iters,
                   "l2": "working set inside L2 (a 2D grid of this size; no flush, each step restarts from phi0)"},
        "fp64_gpu": {"ms": ms64, "value": N * iters / (ms64 / 1e3), "err_3dx_min": err(p64, 3 * dmin), "err_3diag_min": err(p64, 3 * diag)},
        "mixed_gpu": {"ms": ms32, "value": N * iters / (ms32 / 1e3), "err_3dx_min": err(p32, 3 * dmin),
                      "band_linf_vs_fp64_over_dx_min": float(np.max(np.abs(p32[band] - p64[band]))) / dmin},
        "cpu_restatement": {str(nt): {"ms": 1e3 * s, "value": N * iters / s} for nt, (s, _) in cpu.items()},
        "cpu_err_3dx_min": err(cpu[cores][1], 3 * dmin),
        "fp64_gpu_equals_cpu": bool(np.array_equal(p64, cpu[cores][1]) and np.array_equal(p64, cpu[1][1])),
        "dx_min": dmin, "diag_min": diag,
        "cpu_baseline": {"value": N * iters / cpu[cores][0], "unit": "node-iters/s", "cores": cores, "kind": "port",
                         "sample": f"the whole workload ({iters} iterations x {N} nodes), best of 5, oracle/ (CPU restatement of the reference loops)"},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "transport3d":
        if rank == 0:
            run_transport(args)
        return
    if args.workload == "batch2d":
        if rank == 0:
            run_batch(args)
        return
    if args.workload == "large3d":
        if rank == 0:
            run_large(args)
        return
    if args.workload == "reinit2d":
        if rank == 0:
            run_reinit2d(args)
        return

    import torch
    import casl_p4est_gb300 as G
    from casl_p4est_gb300 import _lib as L

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    t0 = time.perf_counter()
    f, phi0 = build_grid(args.levels)
    N = f.num_nodes
    ngbd = G.my_p4est_node_neighbors_t(f)
    # node-neighbour tables built on the GPU (the same tables as the host build)
    ls = G.my_p4est_level_set_t(ngbd, precision="mixed", device_build=True)
    stream = torch.cuda.current_stream()
    ls.set_stream(stream.cuda_stream)
    if args.stage_config:
        ls.stage_config = parse_stage_config(args.stage_config)
        stage_cfg = dict(ls.stage_config, fixed=True)
    else:
        stage_cfg = ls.autotune(phi0, trials=8)
    setup_s = time.perf_counter() - t0
    _, dmin, _ = f.dxyz_min(args.levels[1])

    phi0_d = torch.from_numpy(phi0).cuda()
    phi_d = torch.empty_like(phi0_d)

    def step(prec):
        phi_d.copy_(phi0_d)
        ls.reinitialize_2nd_order(phi_d, args.iters, precision=prec)

    # accuracy of mixed vs FP64 (untimed): band L-infinity and near-interface error, checked in FP64
    # on the device
    step("fp64")
    ref64_d = phi_d.clone()
    step("mixed")
    band_err, band_nodes = ls.band_linf(phi_d, ref64_d, 3 * dmin)
    near_err, _ = ls.band_linf(phi_d, ref64_d, dmin)
    iface_loc, iface_edges, iface_mismatch = ls.interface_location_error(phi_d, ref64_d)
    del ref64_d

    # warm-up and timed region (mixed)
    for _ in range(args.warmup):
        step("mixed")
    lib = L.load()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lib.lsg_level_set_launch_count(ls.handle)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        step("mixed")
    ev1.record(stream)
    barrier()
    launches = lib.lsg_level_set_launch_count(ls.handle) - launches0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    ms_t = torch.tensor([ms], device="cuda")
    if dist is not None:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms = float(ms_t.item())
    node_iters = N * args.iters * args.steps * world
    value = node_iters / (ms / 1e3)

    # FP64 GPU path, same workload (fewer steps: it is compute-bound on GB300's FP64 units)
    step("fp64")
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.fp64_steps):
        step("fp64")
    e1.record(stream)
    barrier()
    ms64 = e0.elapsed_time(e1)
    value64 = N * args.iters * args.fp64_steps * world / (ms64 / 1e3)

    # per-kernel timing pass (events around each launch) for the roofline
    import ctypes as C
    kms = np.zeros(10)
    kcnt = np.zeros(10, np.int64)
    lib.lsg_level_set_kernel_times(ls.handle, kms.ctypes.data_as(L._DP), kcnt.ctypes.data_as(C.POINTER(C.c_int64)), 10, 1)
    lib.lsg_level_set_enable_kernel_timing(ls.handle, 1)
    step("mixed")
    lib.lsg_level_set_kernel_times(ls.handle, kms.ctypes.data_as(L._DP), kcnt.ctypes.data_as(C.POINTER(C.c_int64)), 10, 1)
    kinds = L.KERNEL_KINDS
    per_kernel = {kinds[k]: {"ms_total": float(kms[k]), "launches": int(kcnt[k]),
                             "ms_per_launch": float(kms[k] / kcnt[k]) if kcnt[k] else None} for k in range(10) if kcnt[k]}
    step("fp64")
    lib.lsg_level_set_kernel_times(ls.handle, kms.ctypes.data_as(L._DP), kcnt.ctypes.data_as(C.POINTER(C.c_int64)), 10, 1)
    lib.lsg_level_set_enable_kernel_timing(ls.handle, 0)
    per_kernel_fp64 = {kinds[k]: {"ms_total": float(kms[k]), "launches": int(kcnt[k]),
                                  "ms_per_launch": float(kms[k] / kcnt[k]) if kcnt[k] else None} for k in range(10) if kcnt[k]}
    # Algorithmic bytes per node (mixed 3D, w_f = w_d = 4 B), fixed by the reference's data flow: a
    # table-reading sweep costs 2D*(4+w_d) = 48 B of stencil table; the second-derivative sweep reads
    # 1 value and writes D; the stage sweep reads phi_0, phi_k and D second derivatives and writes 1;
    # the RK average moves 3 values per iteration. The fused stage kernel performs the second-derivative
    # sweep and the stage sweep of one RK stage (and, every second launch, the average).
    table = 6 * (4 + 4)
    dd_sweep = table + (1 + 3) * 4
    stage_sweep = table + (3 + 3) * 4
    alg = {"stage32": dd_sweep + stage_sweep + 3 * 4 / 2}
    peak, peak_kind = measured_peak()
    dom = "stage32"
    dom_ms = per_kernel[dom]["ms_per_launch"]
    achieved = alg[dom] * N / (dom_ms / 1e3) / 1e9
    tpn = profile_traffic_per_node(dom)
    traffic = tpn * N if tpn is not None else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "kernel": "one mixed RK stage: k_dd_x32 then k_reinit_fused32 (side stream) alongside k_reinit_uniform32 then "
                          "k_reinit_fused_reg32 (higher-priority stream); second-derivative and stage sweeps of every node",
                "peak_source": peak_kind, "alg_bytes_per_node": alg[dom],
                "dram_GBps": (traffic / (dom_ms / 1e3) / 1e9 if traffic is not None else None),
                "dram_frac": (traffic / (dom_ms / 1e3) / 1e9 / peak if traffic is not None else None)}
    iter_bytes = 2 * (dd_sweep + stage_sweep) + 3 * 4  # 284 B per node-iteration
    roofline["per_iteration"] = {"alg_bytes_per_node_iter": iter_bytes, "achieved_GBps": iter_bytes * value / world / 1e9,
                                 "frac": iter_bytes * value / world / 1e9 / peak}
    box_bw = box_copy_bandwidth(stream)
    roofline["frac_of_box_copy"] = achieved / box_bw

    # end to end through the public host API: pinned host phi, H2D + reinit + D2H per step
    host = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(2):
        host[:] = phi0
        ls.reinitialize_2nd_order(host, args.iters, precision="mixed")
    barrier()
    te = 0.0
    for _ in range(args.steps):
        host[:] = phi0
        t = time.perf_counter()
        ls.reinitialize_2nd_order(host, args.iters, precision="mixed")
        te += time.perf_counter() - t
    te_t = torch.tensor([te], device="cuda")
    if dist is not None:
        dist.all_reduce(te_t, op=dist.ReduceOp.MAX)
    e2e = {"value": N * args.iters * args.steps * world / float(te_t.item()), "unit": "node-iters/s",
           "h2d_bytes_per_step": N * 8, "d2h_bytes_per_step": N * 8}

    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        secs, cpu_phi = cpu_reinit_sample(f, phi0, CPU_SAMPLE_ITERS, cores)
        cpu = {"value": N * CPU_SAMPLE_ITERS / secs, "unit": "node-iters/s", "cores": cores, "kind": "port",
               "sample": f"{CPU_SAMPLE_ITERS} reinitialize_2nd_order iterations of the same {N}-node grid on {cores} host threads "
                         f"({secs:.1f} s; oracle/, CPU restatement of the reference loops, bit-identical to the reference's own "
                         "code built from its sources)"}
        # the FP64 GPU path on the full grid for the same iterations, against the oracle's result
        gpu_phi = phi0.copy()
        ls.reinitialize_2nd_order(gpu_phi, CPU_SAMPLE_ITERS, precision="fp64")
        diff = float(np.max(np.abs(gpu_phi - cpu_phi)))
        parity = {"fp64_equals_oracle": bool(np.array_equal(gpu_phi, cpu_phi)), "max_abs_diff": diff,
                  "iterations": CPU_SAMPLE_ITERS, "nodes": N}

    if rank == 0:
        out = {
            "metric": METRIC,
            "value": value, "unit": "node-iters/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "precision": "mixed: FP32 stencil/RK, FP64 subcell step and checks",
            "config": workload_config(args, N, world),
            "fp64": {"value": value64, "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps},
            "speedup_mixed_vs_fp64": value / value64,
            "band_linf_vs_fp64": band_err, "band_linf_over_dx_min": band_err / dmin, "band_nodes": band_nodes,
            "band_linf_near_interface_vs_fp64": near_err,
            "interface_location_err_vs_fp64": iface_loc, "interface_location_err_over_dx_min": iface_loc / dmin,
            "interface_cut_edges": iface_edges, "interface_sign_mismatches": iface_mismatch,
            "dx_min": dmin,
            "fp64_vs_oracle_full_grid": parity,
            "fp64_vs_cpu_same_precision": (value64 / cpu["value"] if cpu else None),
            "roofline": roofline, "kernels": per_kernel, "kernels_fp64": per_kernel_fp64,
            "e2e": e2e, "gpu_launches": int(launches), "cpu_baseline": cpu, "clocks": clk, "box_copy_GBps": box_bw,
            "gpu": gpu_info(local), "setup_s": setup_s,
            "autotuned_stage_config": stage_cfg, "mixed_tables": ls.table_stats(),
        }
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
