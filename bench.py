"""Benchmark: one routing pass of the landscape-evolution hot path on GB300.

Workload (the single-GPU routing configuration): an 8192 x 8192 float32 DEM,
dx = 10 m, seeded spectral-synthesis fractal (power spectrum ~ k^-2, relief
1000 m) plus 100,000 seeded pits (depth U[0,5] m, radius U[1,4] cells),
boundary "oooo". One step = fill_pits(min_slope 1e-4) -> D8 receivers (int64
receivers exported) -> donor counts and outlets -> s-vector (contributing
counts, int64) -> Kahn topological order. The metric is cells routed per
second ("cell-steps/s": one step routes every cell once).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs under torchrun as independent replicas (one grid per GPU; the path
does not shard), so the aggregate is weak scaling. `--impl reference` times
the CPU implementation of the same pass (the C++ restatement of the
reference, oracle/liblsdtt_oracle.so) on the host cores with a 4096 x 4096
sample of the same surface per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LEM cell-steps/s on 1 GB300: learned-precond+batched vs plain GPU at equal residual"
WORKLOAD = ("routing pass on an 8192x8192 fractal (k^-2, 1000 m relief) + 100k pits, dx=10 m, bc oooo: "
            "fill(eps=1e-4) + D8 receivers + donors/outlets + s-vector/int64 counts + Kahn order")


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
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

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
    """DRAM bytes per cell for a kernel from the committed ncu summary
    (profiles/ncu_traffic.txt: '<kernel> <bytes_per_cell> <note>')."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


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


def run_reference(args, rank, world):
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


def run_gpu(args, rank, world):
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
    # Kernel table from the live event pairs.
    kernels = {}
    for name in ("fill_relax", "d8_receivers", "d8_donors", "stack_ruler_walk"):
        t, k, b = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
        G._check(L.lsdtt_gpu_profile_read(name.encode(), ctypes.byref(t), ctypes.byref(k), ctypes.byref(b)))
        if k.value:
            kernels[name] = {"ms": t.value, "launches": k.value, "bytes": b.value}
    L.lsdtt_gpu_profile_enable(0)
    t_max = elapsed
    if dist is not None:
        tt = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    value = world * n * n * args.steps / t_max

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
    e2e_t = e0.elapsed_time(e1) / 1e3
    if dist is not None:
        tt = torch.tensor([e2e_t], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_t = float(tt.item())
    e2e_value = world * n * n * e2e_steps / e2e_t

    if rank == 0:
        peak, peak_kind = peaks()
        dom = max(kernels.items(), key=lambda kv: kv[1]["ms"]) if kernels else None
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
                            "GBps": v["bytes"] / (v["ms"] / 1e3) / 1e9} for k, v in kernels.items()},
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--skip-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gpu(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
