"""Benchmark: the landscape-evolution timestep on GB300.

Default workload (--workload ensemble): a batched parameter-sweep ensemble
of 256 independent LEM runs on one GPU. Member grids have sides drawn
uniformly from 128-1024 cells (rows and columns independently), dx = 30 m,
bc "nnon"; K log-uniform 1e-6..1e-4, m uniform 0.35..0.6, n from {1, 1.5,
2}, D log-uniform 1e-3..1e-1 m^2/yr, U log-uniform 1e-4..1e-2 m/yr, dt =
1000 yr; initial surfaces seeded uniform noise 0-1 m plus a 0.001 tilt
toward the open south edge. One step advances every member by one LEM step:
fill_pits(1e-4, in the reference's FIFO order, bit for bit) -> D8 receivers
-> s-vector / contributing counts -> implicit
stream power (per-node Newton for n != 1) -> linear implicit hillslope by
Jacobi-PCG to a 1e-8 relative residual -> uplift and boundary restore. The
metric is member cells advanced per second (cell-steps/s).

The same line reports:
  * plain_gpu: the members stepped one at a time through the single-grid
    LEM (lsdtt_gpu_lem_step), all of them -- the plain GPU form;
  * e2e: the ensemble stepped through the C ABI with the packed surfaces
    uploaded from and downloaded to pinned host memory every step;
  * kernels / roofline: every kernel (and the exact fill's stages) of a
    profiled (eager) step of the same ensemble, and the dominant single
    kernel's algorithmic bytes over its CUDA-event time;
  * cpu_baseline: the C++/numpy restatement of the reference (oracle/) on a
    bounded sample of members, on the host cores.

--workload routing keeps the single-grid routing pass (8192^2 fractal +
100k pits: fill + D8 + s-vector + Kahn order).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload ensemble|routing]

N > 1 runs under torchrun as independent replicas (each rank its own
ensemble; members are independent and the path has no exchange step), so
the aggregate is weak scaling. `--impl reference` times the CPU
restatement of the same step on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LEM cell-steps/s on 1 GB300: learned-precond+batched vs plain GPU at equal residual"
WORKLOAD = ("routing pass on an 8192x8192 fractal (k^-2, 1000 m relief) + 100k pits, dx=10 m, bc oooo: "
            "fill(eps=1e-4) + D8 receivers + donors/outlets + s-vector/int64 counts + Kahn order")
ENS_WORKLOAD = ("batched ensemble of 256 LEM runs, sides U{128..1024} (non-square), dx=30 m, bc nnon, dt=1000 yr, "
                "K logU[1e-6,1e-4], m U[0.35,0.6], n in {1,1.5,2}, D logU[1e-3,1e-1], U logU[1e-4,1e-2], "
                "noise 0-1 m + 0.001 tilt; step = fill(1e-4) + D8 + s-vector + stream power + linear implicit "
                "hillslope (Jacobi-PCG, 1e-8 relative residual) + uplift/boundary restore")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def surface(n: int, seed: int = 7):
    from tests import surfaces
    return surfaces.fractal_pits(n, relief=1000.0, seed=seed)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.p = None
        self.path = os.path.join(tempfile.gettempdir(), f"lsdtt_gb300_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
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
            self.f.close()

    def summary(self):
        if self.p is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def traffic_per_cell(kernel: str):
    """DRAM bytes per cell of one launch of `kernel`, from its committed ncu
    summary (profiles/<kernel>_ncu.md, the line 'traffic_bytes_per_cell: X':
    dram__bytes_read.sum + dram__bytes_write.sum of a captured launch over
    the cells it covered); None when no summary exists."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_ncu.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("traffic_bytes_per_cell:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except (ValueError, IndexError):
                return None
    return None


def profile_table(L):
    """Every profile record of the library (name -> ms, launches, bytes)."""
    need = ctypes.c_int64()
    L.lsdtt_gpu_profile_names.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    L.lsdtt_gpu_profile_names(None, 0, ctypes.byref(need))
    buf = ctypes.create_string_buffer(int(need.value) + 1)
    L.lsdtt_gpu_profile_names(buf, len(buf), ctypes.byref(need))
    out = {}
    for name in buf.value.decode().split():
        t, k, b = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
        L.lsdtt_gpu_profile_read(name.encode(), ctypes.byref(t), ctypes.byref(k), ctypes.byref(b))
        if k.value:
            out[name] = {"ms": t.value, "launches": k.value, "bytes": b.value}
    return out


def cpu_baseline(n_sample: int, reps: int = 1):
    """The oracle (C++ restatement of the reference path) on the host cores:
    fill + lsdtt_flowinfo (receivers OpenMP-parallel, the rest serial, as in
    the reference) on an n_sample^2 sample of the same surface."""
    import oracle
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    P = oracle.port()
    z = surface(n_sample)
    m = np.ones_like(z, np.uint8)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        f = P.fill_pits(z, m, 10.0, "oooo", 1e-4)
        P.flowinfo(f, m, 10.0, "oooo", allow_pits_as_outlets=True, want_accum=False)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return z.size / best, best


def routing_reference(args, rank, world):
    if rank != 0:
        return 0
    n_sample = args.cpu_sample
    times = []
    import oracle
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    P = oracle.port()
    z = surface(n_sample)
    m = np.ones_like(z, np.uint8)
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        f = P.fill_pits(z, m, 10.0, "oooo", 1e-4)
        P.flowinfo(f, m, 10.0, "oooo", allow_pits_as_outlets=True, want_accum=False)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    per = statistics.median(times)
    value = z.size / per
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": f"{n_sample}x{n_sample} sample of the same surface per step",
                       "cells_per_step": int(z.size)},
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{n_sample}x{n_sample} fractal+pits, fill+D8+s-vector+topo, "
                                       f"median of {args.steps}"},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def rank_max(t: float, dist=None, device: str = "cuda") -> float:
    """The largest of the ranks' values (a job's time is its slowest rank's);
    t itself without a process group. FP64, so a time keeps its digits."""
    if dist is None:
        return t
    import torch
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_rate(units_per_rank: float, steps: int, t_max: float, world: int) -> float:
    """Whole-job throughput of independent replicas (weak scaling): every
    rank processed units_per_rank units a step for `steps` steps, and the job
    took its slowest rank's time t_max."""
    return world * units_per_rank * steps / t_max


def routing_gpu(args, rank, world):
    import torch
    import lsdtt_gb300 as G
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = G.lib()
    L.lsdtt_gpu_launch_count.restype = ctypes.c_ulonglong
    L.lsdtt_gpu_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]
    n = args.size
    z = surface(n, seed=7 + rank)
    m = np.ones_like(z, np.uint8)
    zt = torch.from_numpy(z).cuda()
    mt = torch.from_numpy(m).cuda()
    ft = torch.empty_like(zt)
    stream = torch.cuda.current_stream()
    grid = G.make_grid(n, n, 10.0, "oooo")
    opts = G.FlowOptions(1, 1, 1, 1, 1)
    h = ctypes.c_void_p()
    G._check(L.lsdtt_gpu_flow_create(ctypes.byref(grid), ctypes.byref(h)))
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        G._check(L.lsdtt_gpu_fill_pits(ctypes.byref(grid), ctypes.c_void_p(zt.data_ptr()),
                                       ctypes.c_void_p(mt.data_ptr()), ctypes.c_float(1e-4),
                                       ctypes.c_void_p(ft.data_ptr()), sp))
        G._check(L.lsdtt_gpu_flow_build(h, ctypes.c_void_p(ft.data_ptr()), ctypes.c_void_p(mt.data_ptr()),
                                        ctypes.byref(opts), None, ctypes.c_int64(0), sp))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    launches0 = L.lsdtt_gpu_launch_count()
    L.lsdtt_gpu_profile_enable(1)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    launches = L.lsdtt_gpu_launch_count() - launches0
    # Kernel table from the live event pairs (every record of the timed steps).
    kernels = profile_table(L)
    L.lsdtt_gpu_profile_enable(0)
    t_max = rank_max(elapsed, dist)
    value = job_rate(n * n, args.steps, t_max, world)

    # End to end through the public host-buffer call.
    zh = torch.from_numpy(z).pin_memory()
    mh = torch.from_numpy(m).pin_memory()
    fh = torch.empty(n * n, dtype=torch.float32).pin_memory()
    rh = torch.empty(n * n, dtype=torch.int64).pin_memory()
    th = torch.empty(n * n, dtype=torch.int64).pin_memory()
    ch = torch.empty(n * n, dtype=torch.int64).pin_memory()

    def e2e_step():
        G._check(L.lsdtt_gpu_route_host(ctypes.byref(grid), ctypes.c_void_p(zh.data_ptr()),
                                        ctypes.c_void_p(mh.data_ptr()), ctypes.c_float(1e-4), ctypes.byref(opts),
                                        ctypes.c_void_p(fh.data_ptr()), ctypes.c_void_p(rh.data_ptr()),
                                        ctypes.c_void_p(th.data_ptr()), ctypes.c_void_p(ch.data_ptr()), sp))

    e2e_step()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2e_steps = max(1, min(args.steps, 3))
    e0.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_t = rank_max(e0.elapsed_time(e1) / 1e3, dist)
    e2e_value = job_rate(n * n, e2e_steps, e2e_t, world)

    if rank == 0:
        peak, peak_kind = peaks()
        # the exact fill's sort and scan stages are several kernels each
        one = {k: v for k, v in kernels.items()
               if k not in ("fill_exact_levels", "fill_exact_candidates", "fill_exact_cell_sort")}
        dom = max(one.items(), key=lambda kv: kv[1]["ms"]) if one else None
        roof = None
        if dom:
            name, d = dom
            avg_s = d["ms"] / d["launches"] / 1e3
            achieved = d["bytes"] / d["launches"] / avg_s / 1e9
            tpc = traffic_per_cell(name)
            roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)"
                    if peak_kind == "measured" else "fallback 6.8 TB/s",
                    "traffic": (tpc * n * n) if tpc is not None else None,
                    "algorithmic_bytes_per_launch": d["bytes"] / d["launches"],
                    "avg_launch_ms": d["ms"] / d["launches"], "launches": d["launches"],
                    "share_of_step": d["ms"] / (elapsed * 1e3)}
        cpu_v, cpu_t = (None, None)
        if world == 1 and not args.skip_cpu:
            cpu_v, cpu_t = cpu_baseline(args.cpu_sample)
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells_per_step": n * n, "parallelism": f"replicas x{world}",
                       "l2": "inputs (z 268 MB + mask 67 MB) larger than the 129 MB L2; no flush"},
            "roofline": roof,
            "kernels": {k: {"ms_per_launch": v["ms"] / v["launches"], "launches": v["launches"],
                            "share": v["ms"] / (elapsed * 1e3),
                            "GBps": (v["bytes"] / (v["ms"] / 1e3) / 1e9) if v["bytes"] > 0 else None}
                        for k, v in sorted(kernels.items(), key=lambda kv: -kv[1]["ms"])},
            "cpu_baseline": None if cpu_v is None else {
                "value": cpu_v, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
                "sample": f"{args.cpu_sample}x{args.cpu_sample} sample of the same surface: fill + D8 + s-vector + "
                          f"topo in the C++ restatement of the reference ({cpu_t:.1f} s)"},
            "e2e": {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": 5 * n * n,
                    "d2h_bytes_per_step": 28 * n * n,
                    "call": "lsdtt_gpu_route_host: z,mask in; filled,int64 receivers,topo,counts out"},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    L.lsdtt_gpu_flow_destroy(h)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# ensemble workload
# ---------------------------------------------------------------------------
def ensemble_specs(n_members: int, rank: int = 0, seed: int = 4):
    from tests import surfaces
    rng = np.random.default_rng(seed + 7919 * rank)
    specs = []
    for _ in range(n_members):
        nr, nc = (int(v) for v in rng.integers(128, 1025, 2))
        K = float(10.0 ** rng.uniform(-6.0, -4.0))
        mm = float(rng.uniform(0.35, 0.6))
        nn = float(rng.choice([1.0, 1.5, 2.0]))
        D = float(10.0 ** rng.uniform(-3.0, -1.0))
        U = float(10.0 ** rng.uniform(-4.0, -2.0))
        z = surfaces.noise_tilt(nr, nc, 30.0, int(rng.integers(1 << 30)), "nnon", 0.001)
        specs.append(dict(z=z, cell_size=30.0, boundary_conditions="nnon", timestep=1000.0, erodibility=K,
                          m_exponent=mm, n_exponent=nn, uplift_rate=U, hillslope_diffusivity=D, fill_min_slope=1e-4,
                          hillslope_rel_tol=1e-8, hillslope_max_iter=2000))
    return specs


def ensemble_cpu_step(P, H, lem_finish, spec):
    """One LEM step of one member in the restatement of the reference:
    fill_pits -> lsdtt_flowinfo + compute_d8_stream_power_incision (C++) ->
    the implicit linear hillslope step (FP64 Jacobi-PCG to the member's
    relative residual, scipy) -> uplift and boundary restore."""
    z = spec["z"]
    m = np.ones_like(z, np.uint8)
    cell, bc = spec["cell_size"], spec["boundary_conditions"]
    dt = spec["timestep"]
    bf = P.boundary_flats(m, bc)
    zf = P.fill_pits(z, m, cell, bc, spec["fill_min_slope"])
    zsp = P.stream_power(zf, m, cell, bc, spec["erodibility"], spec["m_exponent"], spec["n_exponent"], dt)
    zh, _, _ = H.linear_step(zsp, m, cell, bc, spec["hillslope_diffusivity"], dt, solver="pcg",
                             rel_tol=spec["hillslope_rel_tol"])
    zn, _ = lem_finish(zh, zf, m, spec["uplift_rate"], dt, bf)
    return zn


def ensemble_cpu_sample(specs, budget_s: float):
    """Members in order, one step each, until budget_s of CPU work."""
    import oracle
    from oracle import hillslope as H
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    P = oracle.port()
    cells, t, used = 0, 0.0, 0
    for spec in specs:
        t0 = time.perf_counter()
        ensemble_cpu_step(P, H, oracle.lem_finish, spec)
        t += time.perf_counter() - t0
        cells += spec["z"].size
        used += 1
        if t >= budget_s:
            break
    return cells / t, cells, used, t


def ensemble_reference(args, rank, world):
    if rank != 0:
        return 0
    specs = ensemble_specs(args.members)
    times, cells_done = [], []
    for i in range(args.warmup + args.steps):
        # each step: a bounded sample of the ensemble's members (rotating)
        rot = specs[(i * 3) % len(specs):] + specs[:(i * 3) % len(specs)]
        v, cells, used, t = ensemble_cpu_sample(rot, 3.0)
        if i >= args.warmup:
            times.append(t)
            cells_done.append(cells)
    value = sum(cells_done) / sum(times)
    line = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": ENS_WORKLOAD,
                       "sample": "each step: members in order until ~3 s of CPU work, one LEM step each"},
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "members of the same ensemble, one LEM step each, ~3 s per step: C++ "
                                       "restatement (fill, flowinfo with OpenMP receivers, stream power) + FP64 "
                                       "Jacobi-PCG hillslope solve (scipy, 1e-8 relative residual)"},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# Records that time a stage whose kernels are also timed one by one (the
# s-vector stage): listed, but left out of the step's total and shares.
ENS_STAGES = ("ens_stack_counts",)
# Records of several kernels (those stages, and the exact fill's sorts and
# scans): never the roofline's dominant kernel.
ENS_MULTI = ENS_STAGES + ("ens_fill_exact_levels", "ens_fill_exact_candidates", "ens_fill_exact_cell_sort")


def ensemble_gpu(args, rank, world):
    import torch
    import lsdtt_gb300 as G
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = G.lib()
    L.lsdtt_gpu_launch_count.restype = ctypes.c_ulonglong
    L.lsdtt_gpu_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]
    specs = ensemble_specs(args.members, rank=rank)
    cells = int(sum(sp["z"].size for sp in specs))
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(t):
        return rank_max(t, dist)

    ens = G.Ensemble(specs, use_graph=True)
    ens.set_member_groups(bool(args.member_groups))
    if args.sweep_mode >= 0:
        # pin the stream-power sweep schedule (a profiler distorts the
        # autotuner's own timings)
        ens.override_schedule(sweep_mode=args.sweep_mode)
    t_warm0 = time.perf_counter()
    for _ in range(args.warmup):
        ens.step()
    barrier()
    t_warm = time.perf_counter() - t_warm0
    launches0 = L.lsdtt_gpu_launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier()
        torch.cuda.nvtx.range_push("timed_steps")  # lets an ncu launch list select the timed steps
        ev0.record(stream)
        for _ in range(args.steps):
            ens.step()
        ev1.record(stream)
        torch.cuda.nvtx.range_pop()
        barrier()
    elapsed = max_over_ranks(ev0.elapsed_time(ev1) / 1e3)
    launches = L.lsdtt_gpu_launch_count() - launches0
    info = ens.info()
    value = job_rate(cells, args.steps, elapsed, world)

    # Kernel table: one profiled step (profiling keeps the ensemble eager).
    # Its NVTX range lets an ncu launch list select it: ncu does not profile
    # the kernel nodes of a graph with conditional (device-side loop) nodes.
    L.lsdtt_gpu_profile_enable(1)
    torch.cuda.nvtx.range_push("profiled_step")
    ens.step()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    kernels = profile_table(L)
    L.lsdtt_gpu_profile_enable(0)

    # End to end: the packed surfaces to and from pinned host memory every step.
    npk = int(ens.offsets()[-1])
    zh = torch.empty(npk, dtype=torch.float32).pin_memory()
    G._check(L.lsdtt_gpu_ensemble_download(ens._h, ctypes.c_void_p(zh.data_ptr()), G._stream(stream)))
    barrier()
    e2e_steps = max(1, min(args.steps, 3))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        G._check(L.lsdtt_gpu_ensemble_upload(ens._h, ctypes.c_void_p(zh.data_ptr()), G._stream(stream)))
        ens.step()
        G._check(L.lsdtt_gpu_ensemble_download(ens._h, ctypes.c_void_p(zh.data_ptr()), G._stream(stream)))
    e1.record(stream)
    barrier()
    e2e_t = max_over_ranks(e0.elapsed_time(e1) / 1e3)
    e2e_value = job_rate(cells, e2e_steps, e2e_t, world)
    ens.close()

    # The plain GPU form: members one at a time through the single-grid LEM.
    plain = None
    if args.plain_members != 0:
        sub = specs if args.plain_members < 0 else specs[:args.plain_members]
        models = []
        for sp in sub:
            o = {k: v for k, v in sp.items() if k not in ("z", "cell_size", "boundary_conditions")}
            models.append(G.LandscapeModel(sp["z"], np.ones_like(sp["z"], np.uint8), sp["cell_size"],
                                           sp["boundary_conditions"], **o))
        for mdl in models:
            mdl.step(want_stats=False)
        barrier()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for mdl in models:
            mdl.step(want_stats=False)
        p1.record(stream)
        barrier()
        pt = p0.elapsed_time(p1) / 1e3
        pc = int(sum(sp["z"].size for sp in sub))
        plain = {"value": pc / pt, "unit": "cell-steps/s", "members": len(sub), "cells": pc, "ms_per_step": pt * 1e3,
                 "call": "lsdtt_gpu_lem_step per member (fill, D8 engine, stream power, Jacobi-PCG hillslope), the "
                         "same members one grid at a time"}
        for mdl in models:
            mdl.close()

    if rank == 0:
        peak, peak_kind = peaks()
        single = {k: v for k, v in kernels.items() if k not in ENS_STAGES}
        one = {k: v for k, v in kernels.items() if k not in ENS_MULTI}
        dom = max(one.items(), key=lambda kv: kv[1]["ms"]) if one else None
        step_ms = sum(v["ms"] for v in single.values())
        roof = None
        if dom:
            name, d = dom
            avg_s = d["ms"] / d["launches"] / 1e3
            achieved = d["bytes"] / d["launches"] / avg_s / 1e9
            tpc = traffic_per_cell(name)
            roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak,
                    "peak_source": "measured hbm_gbs (MEASURED_PEAKS.json), of measured"
                    if peak_kind == "measured" else "fallback 6.8 TB/s, of fallback",
                    "traffic": (tpc * cells) if tpc is not None else None,
                    "traffic_source": f"profiles/{name}_ncu.md (dram bytes of a captured launch, scaled by cells)"
                    if tpc is not None else None,
                    "algorithmic_bytes_per_launch": d["bytes"] / d["launches"],
                    "avg_launch_ms": d["ms"] / d["launches"], "launches": d["launches"],
                    "share_of_step": d["ms"] / step_ms if step_ms > 0 else None,
                    "source": "CUDA events around every kernel launch of one profiled (eager) step of the same "
                              "ensemble, run right after the timed region; the dominant kernel is the one with the "
                              "largest total"}
        # The >= 60% of HBM bar for the D8 receivers and the
        # contributing counts (algorithmic bytes per cell: receivers 6 + the
        # exported int64 receiver 8; counts 10).
        bars = {}
        rd = kernels.get("ens_d8_receivers")
        if rd:
            t = rd["ms"] + kernels.get("ens_d8_receivers_fixup", {}).get("ms", 0.0)
            bars["d8_receivers"] = {"bytes_per_cell": 14.0, "ms": t, "achieved": 14.0 * cells / (t / 1e3) / 1e9,
                                    "frac": 14.0 * cells / (t / 1e3) / 1e9 / peak, "bar": 0.6,
                                    "kernels": "ens_d8_receivers + ens_d8_receivers_fixup"}
        sc = kernels.get("ens_stack_counts")
        if sc:
            bars["contributing_counts"] = {"bytes_per_cell": 10.0, "ms": sc["ms"],
                                           "achieved": 10.0 * cells / (sc["ms"] / 1e3) / 1e9,
                                           "frac": 10.0 * cells / (sc["ms"] / 1e3) / 1e9 / peak, "bar": 0.6,
                                           "kernels": "the s-vector stage (Euler tour links, ruling-set list "
                                                      "ranking, count/depth outputs)"}
        cpu = None
        if world == 1 and not args.skip_cpu:
            v, cc, used, t = ensemble_cpu_sample(specs, 20.0)
            cpu = {"value": v, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"the first {used} members of the same ensemble, one LEM step each ({cc} cells, "
                             f"{t:.1f} s): C++ restatement (fill, flowinfo with OpenMP receivers, stream power) + "
                             f"FP64 Jacobi-PCG hillslope solve (scipy, 1e-8 relative residual)"}
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": ENS_WORKLOAD, "members": len(specs), "cells_per_step": cells,
                       "packed_cells": int(info["packed_cells"]), "parallelism": f"replicas x{world}",
                       "preconditioner": "Jacobi (the learned FPCG is not selected: the members' D dt/dx^2 <= 0.11 "
                                         "converge in <= 20 Jacobi-PCG iterations, cheaper than one network "
                                         "application)",
                       "l2": f"inputs ({cells * 4 / 1e9:.2f} GB of surfaces alone) larger than the 129 MB L2; "
                             f"no flush", "warmup_s": t_warm},
            "schedule": info,
            "plain_gpu": plain,
            "batched_over_plain": (value / plain["value"]) if plain else None,
            "roofline": roof,
            "hbm_bars": bars,
            "kernels": {k: {"ms": v["ms"], "launches": v["launches"],
                            "share": (v["ms"] / step_ms) if (step_ms > 0 and k not in ENS_STAGES) else None,
                            "GBps": (v["bytes"] / (v["ms"] / 1e3) / 1e9) if v["bytes"] > 0 else None}
                        for k, v in sorted(kernels.items(), key=lambda kv: -kv[1]["ms"])},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": 4 * npk,
                    "d2h_bytes_per_step": 4 * npk,
                    "call": "lsdtt_gpu_ensemble_upload -> lsdtt_gpu_ensemble_step -> lsdtt_gpu_ensemble_download "
                            "(packed float32 surfaces, pinned host memory)"},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# learned-preconditioner workloads (large single-grid LEM, hillslope solve)
# ---------------------------------------------------------------------------
def train_preconditioner(G, size, cell, D, Sc, dt, nonlinear, n_surfaces, pairs_per, steps, capacity, seed=100):
    """A U-Net trained on the GPU on residual/correction pairs captured from
    plain Jacobi-PCG solves on seeded fractal surfaces of side `size` (with
    the same slope statistics as the target surface)."""
    import torch
    from tests import surfaces
    rs, es = [], []
    for k in range(n_surfaces):
        z, _ = surfaces.fractal_subcritical(size, size, cell, Sc, seed + k)
        r, e = G.capture_pairs(z, np.ones_like(z, np.uint8), cell, "oooo", D, Sc, dt, pairs_per, nonlinear=nonlinear)
        rs.append(r)
        es.append(e)
    r = torch.cat(rs)
    e = torch.cat(es)
    net = G.UNet(size, size, seed=seed)
    order = np.random.default_rng(seed).integers(0, r.shape[0], steps)
    t0 = time.perf_counter()
    # Adam, one pair a step, learning rate 2e-3 cosine-decayed to 2e-4
    lrs = 2e-4 + 0.5 * (2e-3 - 2e-4) * (1.0 + np.cos(np.pi * np.arange(steps) / max(1, steps)))
    losses = [net.train_step(r[k], e[k], lr=float(lr)) for k, lr in zip(order, lrs)]
    torch.cuda.synchronize()
    if capacity > size:
        # an inference-only copy sized for the target grid (no training buffers)
        big = G.UNet(capacity, capacity, seed=seed)
        big.set_params(net.get_params())
        net.close()
        net = big
    conv = getattr(train_preconditioner, "conv_kernel", "")
    if conv:
        net.set_conv_kernel(conv)
    n_pairs = int(r.shape[0])
    del r, e, rs, es
    torch.cuda.empty_cache()
    return net, {"pairs": n_pairs, "surfaces": n_surfaces, "steps": steps,
                 "loss_first50": float(np.mean(losses[:50])), "loss_last50": float(np.mean(losses[-50:])),
                 "train_s": time.perf_counter() - t0}


def large_gpu(args, rank, world):
    """Config 5: a single-grid LEM with the Roering hillslope, plain
    Jacobi-PCG against the learned preconditioner, cell-steps/s each."""
    import torch
    import lsdtt_gb300 as G
    from tests import surfaces
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    n = args.size if args.size != 8192 else 16384
    # The k^-2 fractal at 2000 m relief is steeper than Sc = 1.2 on most
    # cells at this cell size; the relief is scaled to a well-posed Roering
    # problem (steepest slope 0.8 Sc) and reported.
    z0, relief = surfaces.fractal_subcritical(n, n, 30.0, 1.2, 5 + rank)
    m0 = np.ones_like(z0, np.uint8)
    opts = dict(timestep=500.0, erodibility=2e-5, m_exponent=0.45, n_exponent=1.5, uplift_rate=1e-3,
                hillslope_diffusivity=0.02, hillslope_nonlinear=True, critical_slope=1.2, fill_min_slope=1e-4,
                hillslope_rel_tol=1e-8, hillslope_max_iter=4000)
    stream = torch.cuda.current_stream()
    net, tinfo = train_preconditioner(G, 512, 30.0, 0.02, 1.2, 500.0, True, args.train_surfaces, 8,
                                      args.train_steps, n)
    out = {}
    for form in ("plain", "learned"):
        model = G.LandscapeModel(z0, m0, 30.0, "oooo", **opts)
        if form == "learned":
            model.set_preconditioner(net)
        its = []
        for _ in range(args.warmup):
            its.append(model.step()["hillslope_iterations"])
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            its.append(model.step()["hillslope_iterations"])
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        out[form] = {"value": n * n * args.steps / t, "unit": "cell-steps/s", "ms_per_step": t / args.steps * 1e3,
                     "hillslope_pcg_iterations": its}
        out[form + "_z"] = model.z
        model.close()
    zp, zl = out.pop("plain_z"), out.pop("learned_z")
    diff = float(((zl - zp).abs().max() / max(float((zp.max() - zp.min()).item()), 1.0)).item())
    line = {"metric": METRIC, "value": out["learned"]["value"], "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["learned"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"large LEM {n}x{n}, dx=30 m, fractal k^-2 scaled to {relief:.0f} m relief "
                                   f"(steepest slope 0.8 Sc), dt=500 yr, K=2e-5, m=0.45, n=1.5, U=1e-3, "
                                   f"fill 1e-4, Roering Sc=1.2 D=0.02, PCG 1e-8"},
            "learned": out["learned"], "plain_gpu": out["plain"], "training": tinfo,
            "learned_vs_plain_surface_max_rel_diff": diff}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def hillslope_gpu(args, rank, world):
    """Config 3: the Roering implicit hillslope step on a 4096^2 fractal
    (dx = 5 m, 300 m relief, D = 0.01, Sc = 1.0, D dt / dx^2 = 10), plain
    Jacobi-PCG against the learned preconditioner, both to 1e-8."""
    import torch
    import lsdtt_gb300 as G
    from tests import surfaces
    n = args.size if args.size != 8192 else 4096
    dt = 25000.0
    net, tinfo = train_preconditioner(G, 512, 5.0, 0.01, 1.0, dt, True, args.train_surfaces, 8, args.train_steps, n)
    res = {}
    reliefs = []
    for k in range(max(1, args.steps)):
        # 300 m relief at dx = 5 m is steeper than Sc = 1 almost everywhere:
        # scaled to a well-posed Roering problem, relief reported
        z, relief = surfaces.fractal_subcritical(n, n, 5.0, 1.0, 900 + k)
        reliefs.append(relief)
        m = np.ones_like(z, np.uint8)
        for form in ("plain", "learned"):
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push("hillslope_" + form)  # lets an ncu capture select one solve
            t0 = time.perf_counter()
            zo, rep = G.hillslope_implicit(z, m, 5.0, "oooo", 0.01, 1.0, dt, nonlinear=True, rel_tol=1e-8,
                                           max_pcg_iter=20000, net=net if form == "learned" else None)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
            res.setdefault(form, []).append({"s": time.perf_counter() - t0, **rep.as_dict()})
            res.setdefault(form + "_z", []).append(zo)
    diffs = [float(((a - b).abs().max()).item()) for a, b in zip(res.pop("plain_z"), res.pop("learned_z"))]
    # kernel table of one more learned solve (CUDA events per launch)
    L = G.lib()
    L.lsdtt_gpu_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]
    L.lsdtt_gpu_profile_enable(1)
    G.hillslope_implicit(z, m, 5.0, "oooo", 0.01, 1.0, dt, nonlinear=True, rel_tol=1e-8, max_pcg_iter=20000, net=net)
    torch.cuda.synchronize()
    kernels = {}
    for name in ["unet_prep", "unet_conv_in", "unet_pool"] + [f"unet_layer{l}" for l in range(1, 7)] + \
            ["unet_conv_out", "hillslope_apply"]:
        t, k, b = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
        G._check(L.lsdtt_gpu_profile_read(name.encode(), ctypes.byref(t), ctypes.byref(k), ctypes.byref(b)))
        if k.value:
            kernels[name] = {"total_ms": t.value, "launches": k.value, "GBps": b.value / (t.value / 1e3) / 1e9}
    L.lsdtt_gpu_profile_enable(0)
    line = {"workload": f"Roering implicit hillslope step {n}x{n}, dx=5 m, k^-2 fractal scaled to a steepest "
                        f"slope of 0.8 Sc, D=0.01, Sc=1.0, dt={dt} (D dt/dx^2 = 10), PCG 1e-8", "reliefs_m": reliefs,
            "training": tinfo,
            "plain": res["plain"], "learned": res["learned"], "max_abs_surface_diff_m": diffs,
            "learned_solve_kernels": kernels}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def unet_gpu(args, rank, world):
    """Network applications on one residual image (--size, default 2048):
    the U-Net forward pass alone, CUDA-event time per application and the
    tensor-core convolution share."""
    import torch
    import lsdtt_gb300 as G
    n = args.size if args.size != 8192 else 2048
    net = G.UNet(n, n, seed=3)
    if args.conv_kernel:
        net.set_conv_kernel(args.conv_kernel)
    r = torch.randn(n, n, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    for _ in range(args.warmup):
        net.apply(r)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        net.apply(r)
    e1.record()
    torch.cuda.synchronize()
    net.status()
    ms = e0.elapsed_time(e1) / args.steps
    # useful FLOPs of one application (2 * 9 * Cin * Cout per output pixel per layer)
    flops = 0.0
    for (name, ci, co), px in zip(G.UNET_LAYERS, [n * n, n * n / 4, n * n / 16, n * n / 64, n * n / 16, n * n / 4,
                                                   n * n, n * n]):
        flops += 2.0 * 9 * ci * co * px
    # per-layer table of one more application (CUDA events per launch)
    L = G.lib()
    L.lsdtt_gpu_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]
    L.lsdtt_gpu_profile_enable(1)
    net.apply(r)
    torch.cuda.synchronize()
    kernels = {}
    for name in ["unet_prep", "unet_conv_in", "unet_pool"] + [f"unet_layer{l}" for l in range(1, 7)] + ["unet_conv_out"]:
        t, k, b = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
        G._check(L.lsdtt_gpu_profile_read(name.encode(), ctypes.byref(t), ctypes.byref(k), ctypes.byref(b)))
        if k.value:
            kernels[name] = {"ms": round(t.value, 4), "GBps": round(b.value / (t.value / 1e3) / 1e9, 1)}
    L.lsdtt_gpu_profile_enable(0)
    if rank == 0:
        print(json.dumps({"workload": f"U-Net forward on a {n}x{n} residual", "conv_kernel": args.conv_kernel or "default",
                          "ms_per_application": ms,
                          "tflops": flops / (ms / 1e3) / 1e12, "steps": args.steps, "kernels": kernels}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--workload", default="ensemble", choices=["ensemble", "routing", "large", "hillslope", "unet"])
    ap.add_argument("--train-surfaces", type=int, default=64)
    ap.add_argument("--train-steps", type=int, default=4000)
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--sweep-mode", type=int, default=-1, help="ensemble sweep: -1 autotuned, 0 levels, 1 dataflow, 2 cooperative levels, 3 member clusters")
    ap.add_argument("--plain-members", type=int, default=-1,
                    help="members stepped one at a time for the plain GPU form (-1: all of them, 0: skip)")
    ap.add_argument("--member-groups", type=int, default=0, choices=[0, 1],
                    help="ensemble: the deep members' sweep beside the others' sweep and hillslope solve (1) or not")
    ap.add_argument("--conv-kernel", default="", choices=["", "mma", "tcgen05", "tcgen05_rows", "tcgen05_ws"],
                    help="U-Net convolution kernels (default: the library's)")
    args = ap.parse_args()
    train_preconditioner.conv_kernel = args.conv_kernel  # the inference network's convolutions
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.workload == "large":
        return large_gpu(args, rank, world)
    if args.workload == "hillslope":
        return hillslope_gpu(args, rank, world)
    if args.workload == "unet":
        return unet_gpu(args, rank, world)
    if args.workload == "routing":
        if args.impl == "reference":
            return routing_reference(args, rank, world)
        return routing_gpu(args, rank, world)
    if args.impl == "reference":
        return ensemble_reference(args, rank, world)
    return ensemble_gpu(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
