"""Benchmark of the fused LBM stream–collide step on GB300.

Default workload: D3Q19 SRT lid-driven cube 256^3, float32 storage and arithmetic, Re = 100,
lid u = 0.1 (tau = 3*0.1*255/100 + 0.5 = 1.265), two-lattice pull streaming (double buffer),
six bounce-back walls with a moving lid — the D3Q19 configuration the headline metric (D3Q19
MLUPs, % HBM roofline) is quoted on.  A step is one lattice update of every cell.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One JSON line on rank 0.  `value` = MLUPs of all ranks with the lattices already resident in
HBM (2 x 1.27 GB, larger than the 129 MB L2, so no flush is needed between steps); `e2e` = the
same job through the public API (Solver.run) from pinned host buffers, the upload of f/bc/flags
and the download of f inside the timed region.  Multi-GPU runs are independent replicas (the
step has no exchange on one domain per GPU): value = cells x steps of all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_UPDATE = {("D2Q9", False): 72, ("D3Q19", False): 152, ("D3Q19", True): 76, ("D3Q27", False): 216,
                    ("D3Q27", True): 108}

WORKLOADS = {
    # name: (lattice, n, method, collision, LES, float16c+DDF, Re, lid u, tile)
    "ldc3d_d3q19_256_fp32": dict(lattice="D3Q19", n=256, method="db", coll="SRT", les=False, f16=False, Re=100.0,
                                 U=0.1, tile=(8, 8, 4),
                                 desc="D3Q19 SRT lid-driven cube 256^3, FP32/FP32, Re=100, lid u=0.1, "
                                      "two-lattice pull streaming (double buffer)"),
    "ldc3d_d3q19_256_f16c": dict(lattice="D3Q19", n=256, method="db", coll="SRT", les=False, f16=True, Re=100.0,
                                 U=0.1, tile=(8, 8, 4), arith="fast",
                                 desc="D3Q19 SRT lid-driven cube 256^3, Float16C storage + DDF shift, FP32 math, "
                                      "Re=100, lid u=0.1, pull streaming"),
    "ldc3d_d3q27_256_kbc_f16c_eso": dict(lattice="D3Q27", n=256, method="eso", coll="KBC", les=True, f16=True,
                                         Re=10000.0, U=0.1, tile=(8, 8, 4), arith="fast",
                                         desc="D3Q27 KBC + Smagorinsky Cs=0.1 lid-driven cube 256^3, Re=10000, "
                                              "Float16C + DDF shift, FP32 math, esoteric-pull in place"),
    # the reference's CPU-runnable configuration (its 2D cavity examples, examples/LDC.mojo)
    "ldc2d_d2q9_256_fp32": dict(lattice="D2Q9", n=256, method="db", coll="SRT", les=False, f16=False, Re=100.0,
                                U=0.1, tile=(16, 16, 1), full_steps=20000,
                                desc="D2Q9 SRT lid-driven cavity 256x256, FP32, Re=100, lid u=0.1, rest equilibrium "
                                     "init, bounce-back walls + moving-wall lid, pull streaming (20k-step run)"),
    "batch2d_cylinders_512": dict(lattice="D2Q9", n=0, method="db", coll="SRT", les=False, f16=False, batch=512,
                                  tile=(16, 16, 1), autotune=True,
                                  desc="512 D2Q9 SRT cylinder channels, nx ~ U[200,800], ny = 0.41 nx (sizes on a 32-cell granule, tile autotuned), "
                                       "Re ~ U[20,200], parabolic moving-wall inlet u_max=0.05, equilibrium outlet, "
                                       "Bouzidi links on the cylinder, FP32, one persistent launch per step"),
}
# The reference's published benchmark (README of JohnCSu/mojo_lbm): D3Q19 256^3, fully periodic, all
# fluid, at rest, tau = 0.884 (benchmarks/D3.mojo:39-46), FP32 and Float16C + DDF shift; the MLUPs it
# publishes for this configuration (on an RTX 2070 SUPER, one step per timed iteration) are the
# vs_baseline denominators.
for _f16, _pub in ((False, 2212.0), (True, 2776.0)):
    WORKLOADS[f"periodic256_d3q19_{'f16c' if _f16 else 'fp32'}_rest"] = dict(
        kind="rest", lattice="D3Q19", n=256, method="db", coll="SRT", les=False, f16=_f16, tau=0.884,
        tile=(8, 8, 4), published_mlups=_pub, **({"arith": "fast"} if _f16 else {}),
        desc="D3Q19 SRT periodic 256^3 at rest, tau=0.884, " + ("Float16C storage + DDF shift, FP32 math"
                                                                if _f16 else "FP32/FP32")
             + ", pull streaming (double buffer): the reference's published benchmark configuration")
for _les in ("learned", "smagorinsky"):
    WORKLOADS[f"tgv256_d3q19_les_{_les}"] = dict(
        kind="tgv", lattice="D3Q19", n=256, method="db", coll="SRT", les=True, closure=_les, f16=False,
        Re=1600.0, U=0.05, tile=(8, 8, 4),
        desc=f"D3Q19 SRT LES decaying Taylor-Green vortex, periodic 256^3, Re=1600, u0=0.05, FP32, "
             + ("learned closure (MLP 8->32->32->1, BF16 tensor-core inference, FP32 accumulate; trained on "
                "box-filtered 512^3 runs; Smagorinsky fallback outside the training range)" if _les == "learned"
                else "Smagorinsky Cs=0.1"))
CLOSURE_FILE = ROOT / "mojo_lbm_gb300" / "data" / "tgv_re1600_512to256_closure.npz"
DEFAULT_WORKLOAD = "ldc3d_d3q19_256_fp32"


# ---------------------------------------------------------------------------------------------
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def aggregate(local_ms: float, local_units: float, world: int, backend_device=None):
    """Max of the per-rank times and sum of the per-rank units (replicas).  With world == 1 no
    process group is needed."""
    if world == 1:
        return local_ms, local_units
    import torch
    import torch.distributed as dist
    t = torch.tensor([local_ms, -local_units], dtype=torch.float64, device=backend_device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([local_units], dtype=torch.float64, device=backend_device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t[0]), float(u[0])


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


L2_FLUSH_BYTES = 256 << 20  # twice the 129 MB L2


def profiled_traffic(workload: str):
    """DRAM bytes per launch of the step kernel from the committed ncu summary, if present."""
    p = ROOT / "profiles" / f"{workload}.txt"
    if not p.exists():
        return None, None
    m = re.search(r"^dram_bytes_per_launch_full:\s*([0-9.eE+]+)", p.read_text(), re.M)
    return (float(m.group(1)) if m else None), str(p.relative_to(ROOT))


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running (200 ms period)."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.out = None
        try:
            self.out = open(os.devnull if not os.access(".", os.W_OK) else "/tmp/_lbm_clocks.csv", "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        rows = []
        for ln in Path("/tmp/_lbm_clocks.csv").read_text().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def timed_repeats(run_k, stream, dev, world: int, min_seconds: float, max_repeats: int = 100000, flush=None):
    """Times run_k() (K steps) between CUDA events on the launching stream, with a barrier and a
    synchronize on both sides of every repeat, until min_seconds of timed work have passed (at
    least one repeat).  Returns the per-repeat times in ms.  All ranks run the same number of
    repeats (rank 0's count is broadcast after the first repeat).  flush(), when given, runs before
    every repeat, outside the timed region (the L2 flush of workloads smaller than the L2)."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times: list[float] = []
    n_target = None
    while True:
        if flush is not None:
            flush()
        barrier(world)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        run_k()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier(world)
        times.append(e0.elapsed_time(e1))
        if n_target is None:
            n = max(1, min(max_repeats, math.ceil(min_seconds * 1e3 / max(times[0], 1e-3))))
            if world > 1:
                import torch.distributed as dist
                t = torch.tensor([n], dtype=torch.int64, device=dev)
                dist.broadcast(t, 0)
                n = int(t.item())
            n_target = n
        if len(times) >= n_target:
            return times


# ---------------------------------------------------------------------------------------------
def build_case(wl: dict):
    """Grid, config, host flags/bc and tau of a workload (host numpy, tiled layout)."""
    from mojo_lbm_gb300 import Flags, LBM_Config, LBM_Grid, LBM_method, preprocess
    from mojo_lbm_gb300.lattice import get_lattice
    lat_id = {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}[wl["lattice"]]
    n = wl["n"]
    grid = LBM_Grid(get_lattice(lat_id), n, n, 1 if lat_id == 0 else n, wl["tile"])
    method = LBM_method.DOUBLE_BUFFER if wl["method"] == "db" else LBM_method.ESOTERIC_PULL
    N, D = grid.num_points, grid.D
    flags = np.zeros(N, np.uint8)
    bc = np.zeros(N * (D + 1), np.float32)
    ar = wl.get("arith", "exact")
    if wl.get("kind") == "tgv":  # periodic, all fluid; tau from Re = u0 L / nu with L = n / (2 pi)
        cfg = LBM_Config(method, collision_op=wl["coll"], LES=True, include_moving_boundary=False, arithmetic=ar)
        return grid, cfg, flags, bc, 3.0 * wl["U"] * (n / (2 * math.pi)) / wl["Re"] + 0.5
    if wl.get("kind") == "rest":  # periodic, all fluid, rest equilibrium, fixed tau
        cfg = LBM_Config(method, collision_op=wl["coll"], LES=wl["les"], DDF_shift=wl["f16"], use_float16c=wl["f16"],
                         include_moving_boundary=False, arithmetic=ar)
        return grid, cfg, flags, bc, wl["tau"]
    if wl.get("periodic"):  # diagnostic: the workload's kernel on a periodic box, no walls
        cfg = LBM_Config(method, collision_op=wl["coll"], LES=wl["les"], DDF_shift=wl["f16"], use_float16c=wl["f16"],
                         include_moving_boundary=False, arithmetic=ar)
        return grid, cfg, flags, bc, 3.0 * wl["U"] * (n - 1) / wl["Re"] + 0.5
    cfg = LBM_Config(method, collision_op=wl["coll"], LES=wl["les"], DDF_shift=wl["f16"], use_float16c=wl["f16"],
                     arithmetic=ar)
    for s in ("-Y", "+X", "-X") + (("+Z", "-Z") if D == 3 else ()):
        preprocess.set_exterior_walls(grid, cfg, flags, bc, s, Flags.SOLID, [0.0] * D, 1.0)
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "+Y", Flags.SOLID, [wl["U"]] + [0.0] * (D - 1), 1.0)
    tau = 3.0 * wl["U"] * (n - 1) / wl["Re"] + 0.5
    return grid, cfg, flags, bc, tau


def oracle_closure(wl: dict):
    """The learned closure as the oracle's struct (None for other workloads)."""
    if wl.get("closure") != "learned":
        return None
    import oracle
    d = np.load(CLOSURE_FILE)
    return oracle.closure_struct(d["theta"], float(d["nu_scale"]), d["mean"], d["scale"], d["lo"], d["hi"])


def cpu_sample(wl: dict, grid, cfg, flags, bc, tau, budget_s: float, max_steps: int | None = None):
    """Times the float32 CPU oracle (OpenMP over all host threads) on slabs of the same workload
    (whole-grid steps for grids of at most 2^20 cells).  Returns (MLUPs, cores, description)."""
    import oracle
    N, Q = grid.num_points, grid.Q
    f = np.zeros(N * Q, oracle.f_dtype(cfg, 32))
    oracle.init(cfg, grid, 32, f)
    oracle.set_closure(oracle_closure(wl))
    f2 = f.copy() if wl["method"] == "db" else f
    cores = oracle.max_threads()
    slab = N if N <= (1 << 20) else max(1, N // 16)
    done_cells, t_total, k = 0, 0.0, 0
    while (t_total < budget_s or k < 2) and (max_steps is None or k < max_steps):
        b = (k * slab) % N
        t0 = time.perf_counter()
        oracle.step_range(cfg, grid, 32, f2, f, bc, flags, tau, k % 2 == 0, b, min(N, b + slab), cores)
        t_total += time.perf_counter() - t0
        done_cells += min(N, b + slab) - b
        k += 1
    oracle.set_closure(None)
    if max_steps is not None and slab == N and k == max_steps:
        return done_cells / t_total / 1e6, cores, f"the full {k}-step run of the whole grid, {t_total:.1f} s"
    part = "the whole grid" if slab == N else "1/16 of the grid"
    return done_cells / t_total / 1e6, cores, f"{k} slab-steps of {slab} cells ({part}) each, {t_total:.1f} s"


# ---------------------------------------------------------------------------------------------
def run_ours(args, wl: dict):
    import torch
    from mojo_lbm_gb300.solver import Solver

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    grid, cfg, flags, bc, tau = build_case(wl)
    N, Q = grid.num_points, grid.Q
    solver = Solver(grid, cfg)
    if args.threads:
        solver.set_block_threads(args.threads)
    kernel = args.kernel or wl.get("kernel", "auto")
    if kernel != "auto":
        solver.set_kernel_path({"generic": 1, "tile": 2, "pair": 3, "staged": 4}[kernel])
    f_dtype = torch.int16 if cfg.use_float16c else torch.float32
    fa = torch.empty(N * Q, dtype=f_dtype, device=dev)
    fb = torch.empty_like(fa) if wl["method"] == "db" else fa
    bct = torch.from_numpy(bc).to(dev)
    flt = torch.from_numpy(flags).to(dev)
    closure = None
    if wl.get("kind") == "tgv" or wl.get("periodic"):
        from mojo_lbm_gb300 import tgv
        from mojo_lbm_gb300.closure import LearnedClosure, set_closure
        u0, g0 = tgv.tgv_fields(grid.nx, wl["U"], seed=0, device=dev)
        solver.init_equilibrium(fa, 1.0, tau, u0, g0)
        del u0, g0
        if wl.get("closure") == "learned":
            closure = LearnedClosure.load(CLOSURE_FILE, device=dev)
            set_closure(solver, closure)
    else:
        solver.init_equilibrium(fa)
    if wl["method"] == "db":
        fb.copy_(fa)
    stream = torch.cuda.current_stream(dev)

    # warm-up: W steps, then one graph replay so the 64-step graph is captured before timing
    solver.run(fa, fb, bct, flt, tau, args.warmup, 0, stream)
    solver.run(fa, fb, bct, flt, tau, 64, 0, stream)
    torch.cuda.synchronize(dev)

    # the single-step API (each call also checks the flags against the warp masks' summary): 8 calls
    # back to back between two CUDA events on the launching stream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    for i in range(8):
        if wl["method"] == "db":
            if i % 2 == 0:
                solver.double_buffer_step(fb, fa, bct, flt, tau, stream)
            else:
                solver.double_buffer_step(fa, fb, bct, flt, tau, stream)
        else:
            solver.esoteric_pull_step(fa, bct, flt, tau, i % 2 == 0, stream)
    ev[1].record(stream)
    torch.cuda.synchronize(dev)
    single_ms = ev[0].elapsed_time(ev[1]) / 8

    # timed region: K steps from the graph, barrier + synchronize on both sides, repeated until
    # --repeat-seconds have passed so the clock sampler sees the GPU under load
    clocks = ClockSampler(local) if rank == 0 else None
    K = args.steps
    # lattices that fit in the L2 (the 256^2 D2Q9 cavity): the L2 is flushed by a 256 MB write before
    # every timed replay, so each replay starts from DRAM; within a replay they stay in the L2 from
    # step to step, as in a long run
    lattice_bytes = N * Q * (2 if wl["f16"] else 4) * (2 if wl["method"] == "db" else 1)
    flush = None
    if lattice_bytes < L2_FLUSH_BYTES:
        scratch = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
        flush = scratch.zero_
    reps = timed_repeats(lambda: solver.run(fa, fb, bct, flt, tau, K, 0, stream), stream, dev, world,
                         args.repeat_seconds, flush=flush)
    clk = clocks.stop() if clocks else None
    local_ms = statistics.median(reps)
    t_ms, units = aggregate(local_ms, float(N) * K, world, dev)
    mlups = units / (t_ms * 1e-3) / 1e6

    # end to end through the public API from pinned host buffers
    f_host = torch.empty(N * Q, dtype=f_dtype).pin_memory()
    f_host.copy_(fa)
    bc_host = torch.from_numpy(bc).pin_memory()
    fl_host = torch.from_numpy(flags).pin_memory()
    out_host = torch.empty_like(f_host).pin_memory()

    def e2e_pass(steps):
        fa.copy_(f_host, non_blocking=True)
        bct.copy_(bc_host, non_blocking=True)
        flt.copy_(fl_host, non_blocking=True)
        if wl["method"] == "db":
            fb.copy_(fa)
        solver.run(fa, fb, bct, flt, tau, steps, 0, stream)
        out_host.copy_(fa if (steps % 2 == 0 or wl["method"] != "db") else fb, non_blocking=True)

    # one untimed pass first: the first transfers from and to a freshly pinned buffer are slower
    # (its pages are mapped for the copy engines then), which is set-up, not a step's cost
    e2e_pass(64)
    barrier(world)
    torch.cuda.synchronize(dev)
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    e2e_pass(K)
    h1.record(stream)
    torch.cuda.synchronize(dev)
    barrier(world)
    e2e_ms, e2e_units = aggregate(h0.elapsed_time(h1), float(N) * K, world, dev)
    e2e_mlups = e2e_units / (e2e_ms * 1e-3) / 1e6
    h2d = f_host.numel() * f_host.element_size() + bc_host.numel() * 4 + fl_host.numel()
    d2h = out_host.numel() * out_host.element_size()

    if rank != 0:
        return None
    key = (wl["lattice"], wl["f16"])
    b_alg = BYTES_PER_UPDATE[key]
    # the step kernel's average launch duration over the timed region: the region holds the K step
    # kernels of the graph replays and, once, the two kernels that check the flags' summary
    launch_ms = t_ms / K
    achieved = b_alg * N / (launch_ms * 1e-3) / 1e9
    extra = {}
    if closure is not None:
        # the Smagorinsky step on the same fields, timed the same way, for the per-step time ratio
        from mojo_lbm_gb300 import tgv
        smag = Solver(grid, cfg)  # the same LES configuration without the closure
        u0, g0 = tgv.tgv_fields(grid.nx, wl["U"], seed=0, device=dev)
        smag.init_equilibrium(fa, 1.0, tau, u0, g0)
        del u0, g0
        fb.copy_(fa)
        smag.run(fa, fb, bct, flt, tau, 64, 0, stream)
        torch.cuda.synchronize(dev)
        s_reps = timed_repeats(lambda: smag.run(fa, fb, bct, flt, tau, K, 0, stream), stream, dev, 1,
                               args.repeat_seconds)
        smag_mlups = float(N) * K / (statistics.median(s_reps) * 1e-3) / 1e6
        smag.close()
        m = closure.meta
        extra = {"smagorinsky_mlups": round(smag_mlups, 2), "time_ratio_vs_smagorinsky": round(smag_mlups / mlups, 4),
                 "tensor_tflops": round(2624.0 * N / (launch_ms * 1e-3) / 1e12, 2),
                 "closure_study": {k: m.get(k) for k in ("N_fine", "N_coarse", "Re", "eval_times", "spectrum_error",
                                                         "energy_error", "time_ratio", "command")},
                 "closure_study_note": "errors vs the box-filtered 512^3 run, recorded when the committed network "
                                       "was trained (not re-run by this benchmark)"}
    peak, peak_kind = measured_peaks()
    # the committed capture is of the workload as defined (size, tile, automatic kernel)
    traffic, traffic_src = (profiled_traffic(args.workload) if not (args.n or args.tile or args.kernel)
                            else (None, None))
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        if wl.get("full_steps") and grid.num_points <= (1 << 20):
            # the reference's CPU-runnable configuration: its whole run on the host cores
            v, cores, desc = cpu_sample(wl, grid, cfg, flags, bc, tau, float("inf"), wl["full_steps"])
        else:
            v, cores, desc = cpu_sample(wl, grid, cfg, flags, bc, tau, args.cpu_seconds)
        cpu = {"value": round(v, 3), "unit": "MLUPs", "cores": cores, "kind": "port",
               "sample": f"float32 CPU oracle on {desc} of the same workload"}
    line = {
        "metric": "D3Q19 MLUPs" if wl["lattice"] == "D3Q19" else f"{wl['lattice']} MLUPs",
        "value": round(mlups, 2), "unit": "MLUPs", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": round(t_ms / K, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": round(mlups / wl["published_mlups"], 3) if wl.get("published_mlups") else None,
        "dtype": "f16c" if wl["f16"] else "f32",
        "data": "synthetic (Taylor-Green vortex + seeded perturbation)" if wl.get("kind") == "tgv" or wl.get("periodic")
                else "synthetic (periodic box at rest)" if wl.get("kind") == "rest"
                else "synthetic (lid-driven cavity from rest)",
        "config": {"workload": wl["desc"], "grid": [grid.nx, grid.ny, grid.nz], "tile": list(grid.tile_shape),
                   "tile_source": wl.get("tile_source", "default of the workload"),
                   "layout": "reference tiled layout (col-major tile, col-major tiler)", "tau": round(tau, 6),
                   "arithmetic": cfg.arithmetic,
                   "kernel": {1: "generic", 2: "block-per-tile", 3: "cell-pair block-per-tile",
                              4: "staged block-per-tile (bulk async copies into shared memory)"}[solver.kernel_path],
                   "timing": f"CUDA events around each of {len(reps)} replays of the K-step graph on the launching "
                             f"stream (at least {args.repeat_seconds:g} s in all); value from the median replay "
                             f"(min {min(reps) / K:.5f}, max {max(reps) / K:.5f} ms/step)",
                   "repeats": len(reps),
                   "l2": ("L2 flushed before each timed replay by a %d MB write: the lattices (%.1f MB) fit in the "
                          "129 MB L2 and stay there from step to step within a replay, as in a long run"
                          % (L2_FLUSH_BYTES >> 20, lattice_bytes / 1e6)) if flush is not None else
                         ("no flush: the lattices (%.2f GB) exceed the 129 MB L2" % (lattice_bytes / 1e9)),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "note": f"{b_alg} B/update x {N} cells / average step-kernel duration over the timed region "
                             f"{launch_ms:.4f} ms (CUDA events around the K graph-replayed launches; one step "
                             f"through the single-step API, summary check included: {single_ms:.4f} ms); "
                             f"peak {peak_kind} (MEASURED_PEAKS.json hbm_gbs); traffic = ncu dram bytes per launch "
                             f"({traffic_src or 'no capture committed'})"},
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_mlups, 2), "unit": "MLUPs", "h2d_bytes_per_step": int(h2d / K),
                "d2h_bytes_per_step": int(d2h / K),
                "note": "Solver.run from pinned host buffers: upload of f, bc, flags and download of f inside the "
                        f"timed region, amortised over the {K} steps (after one untimed pass of 64 steps)"},
        "gpu_launches": K + 3,  # per timed K-step replay
        "clocks": clk,
    }
    line.update(extra)
    print(json.dumps(line), flush=True)
    solver.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return line


def run_batch(args, wl: dict):
    """512 uneven D2Q9 cylinder channels, one persistent launch per step."""
    import torch
    from mojo_lbm_gb300.batch import BatchSolver
    from mojo_lbm_gb300.solver import Solver
    from mojo_lbm_gb300.workloads import cylinder_channels, links_of

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    tile_source = "default of the workload"
    if args.autotune or (wl.get("autotune") and not args.no_autotune):
        # sizes on a 32 x 32 granule, so every candidate tile divides every channel
        from mojo_lbm_gb300 import autotune
        from mojo_lbm_gb300.workloads import Channel, channel_specs
        specs = channel_specs(wl["batch"], seed=rank, granule=(32, 32))
        by_shape = {(nx, ny): (nx, ny, Re, off) for nx, ny, Re, off in specs}

        def build(shape, tile):
            nx, ny, Re, off = by_shape[(shape[0], shape[1])]
            ch = Channel(nx, ny, Re, 0.05, off, tuple(tile))
            links = (ch.body.fluid_boundaries_list, ch.body.lattice_links_list, ch.body.link_distances_list)
            return ch.grid, ch.cfg, ch.flags, ch.bc, ch.tau, links

        tile, timing = autotune.batch_tile([(nx, ny, 1) for nx, ny, _, _ in specs], build)
        wl["tile"] = tile
        chans = cylinder_channels(tile=tile, specs=specs)
        tile_source = ("autotuned on a batch of replicas of 4 channels at evenly spaced size quantiles, each "
                       "replica with its own flags and boundary values (" +
                       ", ".join(f"{t[0]}x{t[1]}: {v:.0f}" for t, v in sorted(timing.items())) + " MLUPs)")
    else:
        # the same channels as the autotuned run (32 x 32 granule), in the given tile
        from mojo_lbm_gb300.workloads import channel_specs
        chans = cylinder_channels(tile=wl["tile"], specs=channel_specs(wl["batch"], seed=rank, granule=(32, 32)))
    cfg = chans[0].cfg
    batch = BatchSolver([c.grid for c in chans], cfg)
    # every domain's arrays are slices of one device allocation per kind (the library takes any
    # device pointers per domain), so the end-to-end transfers below are one copy per kind
    cells = [ch.grid.num_points for ch in chans]
    off = np.concatenate([[0], np.cumsum(cells)]).astype(np.int64)
    fa_all = torch.empty(int(off[-1]) * 9, device=dev)
    fb_all = torch.empty_like(fa_all)
    bc_all = torch.from_numpy(np.concatenate([ch.bc for ch in chans])).to(dev)
    fl_all = torch.from_numpy(np.concatenate([ch.flags for ch in chans])).to(dev)
    keep = []
    for i, ch in enumerate(chans):
        a, b = int(off[i]), int(off[i + 1])
        fa, fb = fa_all[9 * a:9 * b], fb_all[9 * a:9 * b]
        bc, fl = bc_all[3 * a:3 * b], fl_all[a:b]
        Solver(ch.grid, cfg).init_equilibrium(fa)
        keep.append((fa, fb, bc, fl))
        batch.set_domain(i, fa, fb, bc, fl, ch.tau)
    fb_all.copy_(fa_all)
    dom, ids, dirs, dists, method = links_of(chans, dev)
    force = torch.zeros(ids.numel() * 2, device=dev)
    batch.set_links(dom, ids, dirs, dists, method, 0.0, force)
    links_mode = args.links or wl.get("links", "separate")
    batch.set_link_mode(links_mode == "fused")
    N = batch.num_cells
    stream = torch.cuda.current_stream(dev)
    batch.run(args.warmup, 0, stream)
    batch.run(64, 0, stream)
    torch.cuda.synchronize(dev)
    K = args.steps
    clocks = ClockSampler(local) if rank == 0 else None
    reps = timed_repeats(lambda: batch.run(K, 0, stream), stream, dev, world, args.repeat_seconds)
    clk = clocks.stop() if clocks else None
    t_ms, units = aggregate(statistics.median(reps), float(N) * K, world, dev)
    mlups = units / (t_ms * 1e-3) / 1e6
    launch_ms = t_ms / K  # per step: the persistent step launch (+ the link launch when separate), averaged

    # end to end through the public API: every domain's f, bc and flags uploaded from pinned host
    # memory, K batched steps, every f downloaded, inside the timed region
    f_host = torch.empty_like(fa_all, device="cpu").pin_memory().copy_(fa_all)
    bc_host = torch.empty_like(bc_all, device="cpu").pin_memory().copy_(bc_all)
    fl_host = torch.empty_like(fl_all, device="cpu").pin_memory().copy_(fl_all)
    out_host = torch.empty_like(f_host).pin_memory()

    def e2e_pass(steps):
        fa_all.copy_(f_host, non_blocking=True)
        fb_all.copy_(fa_all)
        bc_all.copy_(bc_host, non_blocking=True)
        fl_all.copy_(fl_host, non_blocking=True)
        batch.run(steps, 0, stream)
        out_host.copy_(fa_all if steps % 2 == 0 else fb_all, non_blocking=True)

    e2e_pass(64)  # untimed: maps the freshly pinned buffers for the copy engines
    barrier(world)
    torch.cuda.synchronize(dev)
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    e2e_pass(K)
    h1.record(stream)
    torch.cuda.synchronize(dev)
    barrier(world)
    e2e_ms, e2e_units = aggregate(h0.elapsed_time(h1), float(N) * K, world, dev)
    h2d = f_host.numel() * 4 + bc_host.numel() * 4 + fl_host.numel()
    d2h = out_host.numel() * 4
    if rank != 0:
        return None
    peak, peak_kind = measured_peaks()
    achieved = 72 * N / (launch_ms * 1e-3) / 1e9
    traffic, traffic_src = profiled_traffic(args.workload) if wl["batch"] == 512 else (None, None)
    line = {
        "metric": "D2Q9 MLUPs (batched domains)", "value": round(mlups, 2), "unit": "MLUPs", "n_gpus": world,
        "steps": K, "warmup": args.warmup, "ms_per_step": round(t_ms / K, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded channels from rest)",
        "config": {"workload": wl["desc"], "domains": len(chans), "cells": N, "links": int(ids.numel()),
                   "tile": list(wl["tile"]), "tile_source": tile_source,
                   "link_mode": "fused into the step kernel" if links_mode == "fused"
                            else "link-wise kernel after every step",
                   "timing": f"CUDA events around each of {len(reps)} replays of the K-step graph on the launching "
                             f"stream (at least {args.repeat_seconds:g} s in all); value from the median replay",
                   "repeats": len(reps),
                   "l2": "no flush: 2 x %.2f GB of lattices exceed L2" % (N * 36 / 1e9)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "note": f"72 B/update x {N} cells / average per-step time over the timed region {launch_ms:.4f} "
                             f"ms (persistent step{'' if links_mode == 'fused' else ' + link kernel'}); peak {peak_kind}; traffic = ncu dram bytes per "
                             f"launch ({traffic_src or 'no capture committed'}, scaled by cells)"},
        "cpu_baseline": None,
        "e2e": {"value": round(e2e_units / (e2e_ms * 1e-3) / 1e6, 2), "unit": "MLUPs",
                "h2d_bytes_per_step": int(h2d / K), "d2h_bytes_per_step": int(d2h / K),
                "note": "BatchSolver.run with every domain's f, bc and flags uploaded from pinned host buffers and "
                        f"every f downloaded inside the timed region, amortised over the {K} steps (after one "
                        "untimed pass of 64 steps); the domains' arrays are slices of one allocation per kind, "
                        "so each transfer is one copy"},
        "gpu_launches": (K if links_mode == "fused" else 2 * K) + 3, "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    return line


def run_reference_batch(args, wl: dict):
    """The reference arm of the batched workload.  The reference has no batched step: it steps a
    domain at a time.  Its restatement (the float32 CPU oracle, OpenMP over all host threads) takes
    one full step of one channel (stream-collide, then the Bouzidi links) per timed step, cycling
    through the first 16 channels of the workload's seeded set."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    import oracle
    from mojo_lbm_gb300 import Bounceback_method
    from mojo_lbm_gb300.workloads import channel_specs, cylinder_channels
    specs = channel_specs(wl["batch"], seed=0, granule=(32, 32))
    chans = cylinder_channels(tile=tuple(wl["tile"]), specs=specs[:16])
    state = []
    for ch in chans:
        f = np.zeros(ch.grid.num_points * 9, np.float32)
        oracle.init(ch.cfg, ch.grid, 32, f)
        state.append([f, f.copy()])
    cores = oracle.max_threads()
    cells, times = 0, []
    for k in range(args.warmup + args.steps):
        i = k % len(chans)
        ch, (fi, fo) = chans[i], state[i]
        b = ch.body
        t0 = time.perf_counter()
        oracle.step(ch.cfg, ch.grid, 32, fo, fi, ch.bc, ch.flags, ch.tau, True, cores)
        oracle.links(ch.cfg, ch.grid, 32, fo, None, b.fluid_boundaries_list.astype(np.int32),
                     b.lattice_links_list.astype(np.int32), b.link_distances_list.astype(np.float32),
                     int(Bounceback_method.BOUZIDI), False, 0.0)
        dt = time.perf_counter() - t0
        state[i] = [fo, fi]
        if k >= args.warmup:
            times.append(dt)
            cells += ch.grid.num_points
    t = sum(times)
    v = cells / t / 1e6
    sample = (f"float32 CPU oracle (restatement of the reference step and link-wise bounce-back), "
              f"{len(times)} channel steps cycling through {len(chans)} of the {wl['batch']} channels "
              f"({sum(c.grid.num_points for c in chans)} cells); the reference itself is Mojo and not runnable")
    line = {"impl": "reference", "metric": "D2Q9 MLUPs (batched domains)", "value": round(v, 3), "unit": "MLUPs",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * t / len(times), 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded channels from rest)",
            "config": {"workload": wl["desc"], "domains": wl["batch"], "tile": list(wl["tile"]),
                       "step_sample": "each step is one full step of one channel, domains one at a time"},
            "cpu_baseline": {"value": round(v, 3), "unit": "MLUPs", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": round(v, 3), "unit": "MLUPs", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return line


def run_reference(args, wl: dict):
    """The reference arm: the reference's CPU path is not runnable here (Mojo), so its restatement
    (the float32 CPU oracle, OpenMP over all host threads) runs on bounded slabs of the workload."""
    if wl.get("batch"):
        return run_reference_batch(args, wl)
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    grid, cfg, flags, bc, tau = build_case(wl)
    import oracle
    N, Q = grid.num_points, grid.Q
    f = np.zeros(N * Q, oracle.f_dtype(cfg, 32))
    oracle.init(cfg, grid, 32, f)
    f2 = f.copy() if wl["method"] == "db" else f
    # the reference's LES is Smagorinsky (it has no learned closure): its path for LES workloads
    cores = oracle.max_threads()
    slab = max(1, N // 64)
    times = []
    for k in range(args.warmup + args.steps):
        b = (k * slab) % N
        t0 = time.perf_counter()
        oracle.step_range(cfg, grid, 32, f2, f, bc, flags, tau, k % 2 == 0, b, min(N, b + slab), cores)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    t = sum(times)
    v = slab * len(times) / t / 1e6
    line = {"impl": "reference", "metric": "D3Q19 MLUPs" if wl["lattice"] == "D3Q19" else f"{wl['lattice']} MLUPs",
            "value": round(v, 3), "unit": "MLUPs", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * t / len(times), 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16c" if wl["f16"] else "f32",
            "data": "synthetic (periodic box at rest)" if wl.get("kind") in ("tgv", "rest")
                    else "synthetic (lid-driven cavity from rest)",
            "config": {"workload": wl["desc"], "grid": [grid.nx, grid.ny, grid.nz], "tile": list(grid.tile_shape),
                       "step_sample": f"each step updates one slab of {slab} cells (1/64 of the grid)",
                       **({"reference_path": "Smagorinsky LES: the reference has no learned closure"}
                          if wl.get("closure") == "learned" else {})},
            "cpu_baseline": {"value": round(v, 3), "unit": "MLUPs", "cores": cores, "kind": "port",
                             "sample": f"float32 CPU oracle (restatement of the reference step), {len(times)} "
                                       f"slab-steps of {slab} cells; the reference itself is Mojo and not runnable"},
            "e2e": {"value": round(v, 3), "unit": "MLUPs", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return line


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=64)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--threads", type=int, default=0, help="threads per block (0 = built-in)")
    ap.add_argument("--tile", type=str, default="", help="tile shape tx,ty,tz of the layout (default per workload)")
    ap.add_argument("--n", type=int, default=0, help="cube edge override (profiling on a smaller case)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--arithmetic", choices=["exact", "fast"], default=None,
                    help="the step's arithmetic: exact (the reference's operation order, bit-identical to the "
                         "float32 oracle) or fast (FMA rearranged, held to a float32 tolerance); default per workload")
    ap.add_argument("--kernel", choices=["auto", "generic", "tile", "pair", "staged"], default=None,
                    help="step kernel: generic, block-per-tile, cell-pair block-per-tile (two cells per thread "
                         "along x) or staged block-per-tile (bulk async copies of each tile's neighbourhood into "
                         "shared memory); the last two double buffer only; default per workload")
    ap.add_argument("--links", choices=["separate", "fused"], default=None,
                    help="batched workload: Bouzidi links by the link-wise kernel after every step, or fused into "
                         "the step kernel; default per workload")
    ap.add_argument("--repeat-seconds", type=float, default=2.0,
                    help="replay the timed K steps until this much timed work has passed (median replay reported)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--autotune", action="store_true",
                    help="choose the layout's tile with the library's autotuner before the run")
    ap.add_argument("--no-autotune", action="store_true", help="keep the workload's default tile")
    ap.add_argument("--domains", type=int, default=0, help="domain count override of the batched workload")
    ap.add_argument("--periodic", action="store_true",
                    help="diagnostic: the cavity workload's kernel on a periodic box without walls, started from a "
                         "perturbed Taylor-Green vortex (every warp on the block-per-tile kernel's fast branch)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    wl = dict(WORKLOADS[args.workload])
    if args.arithmetic:
        wl["arith"] = args.arithmetic
    if args.tile:
        wl["tile"] = tuple(int(v) for v in args.tile.split(","))
    if args.domains and wl.get("batch"):
        wl["batch"] = args.domains
        wl["desc"] = wl["desc"].replace("512 D2Q9", f"{args.domains} D2Q9")
    if args.n:
        wl["n"] = args.n
        wl["desc"] = wl["desc"].replace("256^3", f"{args.n}^3")
    if args.periodic:
        if wl.get("kind") == "tgv" or wl.get("batch"):
            ap.error("--periodic applies to the cavity workloads")
        wl["periodic"] = True
        wl["desc"] = "periodic-box diagnostic (no walls, perturbed Taylor-Green vortex) of: " + wl["desc"]
    if args.autotune and args.impl == "ours" and not wl.get("batch"):
        import torch
        from mojo_lbm_gb300 import autotune
        untiled = dict(wl, tile=(wl["n"],) * 3)
        grid, cfg, flags, bc, _ = build_case(untiled)  # the workload's flags in the untiled layout
        tile, _, tuned = autotune.best_tile(cfg, grid.lattice, grid.nx, grid.ny, grid.nz,
                                            flags=torch.from_numpy(flags).cuda(), bc=torch.from_numpy(bc).cuda())
        wl["tile"] = tile
        wl["tile_source"] = f"autotuned ({len(autotune.candidates(grid.lattice, grid.nx, grid.ny, grid.nz))} " \
                            f"candidate tiles timed on the workload's own flags: {tuned:.0f} MLUPs)"
    if args.impl == "reference":
        return run_reference(args, wl)
    if wl.get("batch"):
        return run_batch(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    main()
