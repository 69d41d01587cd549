"""Benchmark of the projector-DQMC hot path: sweeps/s at 14x14, Lt=1000.

A step is one sweep (src/Main_PQMC.f90:99-154: Lt slices of local updates,
two-way wraps, stabilised recompute every ngroup slices and the
equal-time measurement) of every chain of the workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload c2_fp64|c4_mixed]

Prints one JSON line (rank 0).  Under torchrun each rank runs its own
independent replica chains (the path does not shard: chains are
independent Markov processes), timing is max over ranks.
"""
from __future__ import annotations

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

FP64_PEAK_GFLOPS = 1010.8   # measured DFMA rate on this GB300 pool (profiles/fp64_peak_probe.md)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="c2_fp64", choices=["c2_fp64", "c4_mixed", "small"])
    p.add_argument("--cpu-slices", type=int, default=0, help="slices per chain in the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


# ---------------------------------------------------------------------------
def workload_model(name: str):
    from pqmc_allinone_gb300 import model as M
    if name == "small":
        spec = M.epsocz_spec(6, lam=0.8, alpha=0.3, ntime=100, ngroup=10, filling=0.5, jump_distance=0.5)
    else:
        # 14x14 spin-orbit lattice (Ns=392, 392 bonds), Nup=196, Lt=1000,
        # dtau=0.1, lambda=0.8, omega=1, static SOC alpha=0.3, ngroup=10
        spec = M.epsocz_spec(14, lam=0.8, alpha=0.3, ntime=1000, ngroup=10, filling=0.5,
                             jump_distance=0.5)
    m = M.build_model(spec, twist_seed=11, twist=1e-3)
    return m


def config_of(name: str, m, n_gpus: int, chains: int) -> dict:
    return {
        "workload": {"c2_fp64": "14x14 SOC EPSOCZ, Lt=1000, plain FP64, 1 chain per GPU",
                     "c4_mixed": "14x14 SOC EPSOCZ, Lt=1000, batched mixed precision",
                     "small": "6x6 SOC EPSOCZ, Lt=100, plain FP64"}[name],
        "L": int(m.lat.dlength[0]), "ns": m.ns, "nelec": m.nelec, "ntime": m.ntime,
        "ngroup": m.ngroup, "dtau": m.spec.delt, "lambda": m.spec.ep_parameter, "alpha": 0.3,
        "omega": m.spec.omega, "chains_per_gpu": chains, "parallelism": f"replicas x{n_gpus}",
        "field_init": "x ~ N(0, 0.5^2), numpy PCG64 seed 2+rank",
        "proposal": "uniform, half-width 0.5",
        "l2": "working set per chain 0.33 GB (expKV 0.2 GB + Q string 0.125 GB) > 129 MB L2; no flush",
    }


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
def cpu_baseline(m, field, words, slices: int) -> dict:
    """The oracle (FP64 restatement of the reference CPU path) on all host
    cores, one independent chain per core, for a bounded sample of slices."""
    from oracle.oracle import OracleChain
    cores = os.cpu_count() or 1
    o = OracleChain(m, field=field, seed_words=words, meas=False)
    o.init_expkv()
    o.init_g(1)
    secs = o.time_parallel(cores, cores, 1, slices)
    sweeps = cores * slices / m.ntime
    return {"value": sweeps / secs, "unit": "sweeps/s", "cores": cores, "kind": "port",
            "sample": f"{cores} chains x {slices} slices of one backward sweep ({slices}/{m.ntime} sweep each), "
                      f"{secs:.1f} s wall", "per_core": sweeps / secs / cores}


def run_reference(args, world, rank):
    if rank != 0:
        return
    m = workload_model(args.workload if args.workload != "c4_mixed" else "c2_fp64")
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.rng import seed_words
    f = M.field_gaussian(m, 2)
    slices = args.cpu_slices or (2 if m.ntime >= 1000 else 20)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(m, f, seed_words(42), max(1, slices // 2))
    for _ in range(args.steps):
        vals.append(cpu_baseline(m, f, seed_words(42), slices))
    v = float(np.mean([x["value"] for x in vals]))
    cb = dict(vals[-1])
    cb["value"] = v
    out = {"metric": "sweeps/s @14x14 Lt=1000", "value": v, "unit": "sweeps/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v if v else None,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic", "config": config_of("c2_fp64", m, args.gpus, 1), "impl": "reference",
           "cpu_baseline": cb, "e2e": {"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0,
                                       "d2h_bytes_per_step": 0},
           "note": "reference Fortran cannot be built here (no Fortran compiler); this is the oracle's "
                   "line-cited C++ FP64 restatement of the same path"}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
def algorithmic_update_flops(m, n_acc: int, n_prop: int) -> float:
    """FP64 flops of update_phonon_field: per proposal the 4x4 ratio
    (G_SS Delta, Delta, det: ~3*dim^3 CMAC), per accepted move the rank-dim
    update Ns*dim*dim + Ns*Ns*dim CMAC (src/mod_update.f90:146-187);
    1 CMAC = 8 flop."""
    d = m.pdim
    return 8.0 * (n_prop * 3.0 * d ** 3 + n_acc * (m.ns * d * d + m.ns * m.ns * d))


def run_gpu(args, world, rank, local):
    import ctypes
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.engine import PqmcChain, kernel_launches
    from pqmc_allinone_gb300.rng import seed_words
    import torch

    torch.cuda.set_device(local)
    m = workload_model(args.workload)
    field = M.field_gaussian(m, 2 + rank)
    words = seed_words(1000 + rank)
    ch = PqmcChain(m, field=field, rng_words=words)
    ch.init_expkv()
    ch.init_g(1)
    loop = 1
    for _ in range(args.warmup):
        ch.sweep(loop, 1)
        loop += 1
    torch.cuda.synchronize()
    s0 = ch.state()
    n0 = kernel_launches()
    clk = ClockSampler(local)
    barrier(world)
    clk.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ch.sweep(loop, 1)
        loop += 1
    torch.cuda.synchronize()
    ev1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    barrier(world)
    launches = kernel_launches() - n0
    s1 = ch.state()
    # the library runs on its own stream; host wall time bracketed by device
    # synchronisation is the step time (the torch events only bracket it)
    t_step = max_over_ranks(world, wall) / args.steps
    value = world * 1.0 / t_step
    n_acc = s1["positive_accept"] - s0["positive_accept"]
    n_rej = s1["negative_accept"] - s0["negative_accept"]

    # dominant kernel: update_phonon_field, timed alone per family launch
    upd = time_update_kernel(ch, m)
    flops_per_launch = algorithmic_update_flops(m, upd["acc"], upd["prop"]) / upd["launches"]
    achieved = flops_per_launch / (upd["ms_per_launch"] * 1e-3) / 1e9

    # end to end through the C-ABI with host buffers: set_field (H2D) +
    # sweep with the measurement record + read back field and record (D2H)
    e2e = run_e2e(ch, m, field, loop + 10, args.steps)

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(m, field, words, args.cpu_slices or (2 if m.ntime >= 1000 else 20))
    if rank != 0:
        return
    out = {"metric": "sweeps/s @14x14 Lt=1000", "value": value, "unit": "sweeps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1000.0,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic", "config": config_of(args.workload, m, world, 1),
           "e2e": e2e, "gpu_launches": int(launches),
           "roofline": {"bound": "fp64", "achieved": achieved, "peak": FP64_PEAK_GFLOPS, "unit": "GFLOP/s",
                        "frac": achieved / FP64_PEAK_GFLOPS, "traffic": None,
                        "kernel": "k_update (update_phonon_field, one family)",
                        "peak_source": "measured DFMA throughput of this GB300 (not in MEASURED_PEAKS.json)"},
           "clocks": clocks, "cpu_baseline": cb,
           "accept_ratio": n_acc / max(1, n_acc + n_rej),
           "event_ms_per_step": ev0.elapsed_time(ev1) / args.steps}
    print(json.dumps(out))


def time_update_kernel(ch, m) -> dict:
    """CUDA-event timing of update_phonon_field launches on the library's
    stream (per-family calls through the C-ABI)."""
    import torch
    lib = ch.lib
    st0 = ch.state()
    t = m.ntime // 2
    reps = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for pf in range(1, len(m.pf) + 1):
        for tt in range(t, t + 5):
            ch.update_phonon_field(pf, tt)
            reps += 1
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    st1 = ch.state()
    acc = st1["positive_accept"] - st0["positive_accept"]
    rej = st1["negative_accept"] - st0["negative_accept"]
    return {"launches": reps, "ms_per_launch": el * 1000.0 / reps, "acc": acc, "prop": acc + rej}


def run_e2e(ch, m, field, loop, steps) -> dict:
    import torch
    from pqmc_allinone_gb300.model import record_width
    hf = np.asfortranarray(field)
    w = record_width(m)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        ch.set_field(hf)
        rec = ch.sweep(loop + 2 * k, 1, warmup=0, meas_number=0, cap=1)
        hf = ch.field()
        _ = rec.sum()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    return {"value": 1.0 / dt, "unit": "sweeps/s", "h2d_bytes_per_step": int(hf.nbytes),
            "d2h_bytes_per_step": int(hf.nbytes + 16 * w)}


def main():
    args = parse()
    world, rank, local = dist_setup() if args.impl == "gb300" else (
        int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()
