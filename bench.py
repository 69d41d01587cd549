"""Benchmark of the projector-DQMC hot path at 14x14 (Ns=392), Lt=1000.

Headline (default ``--workload c4_mixed``): chain-sweeps/s of 64 chains
advanced together by the batched mixed-precision form (FP32 delayed-update
panels, split-BF16 tensor-core flush into an FP64 G, FP64-class recompute
every ngroup slices), next to the plain single-chain FP64 form on the same
GPU (``plain_fp64``) and the CPU oracle on the host cores.

A step is one stabilisation block: ngroup=10 consecutive slices of the
sweep loop (src/Main_PQMC.f90:99-154: per slice the four families' local
updates and two-way wraps, then one stabilised recompute) for every chain.
100 steps make one sweep at Lt=1000; a sweep of 64 chains takes tens of
seconds, so a block is the unit that keeps the run within minutes.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload c4_mixed|c2_fp64|small] [--chains C]

Prints one JSON line (rank 0).  Under torchrun each rank advances its own
independent chains (chains are independent Markov processes: replicas, no
collective on the data path); the step time is the max over ranks.
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

METRIC = "sweeps/s @14x14 Lt=1000: batched mixed-prec vs plain FP64 on GB300"

# DFMA throughput of this GB300 pool measured with a dependent-free FP64 FMA
# loop over all SMs (MEASURED_PEAKS.json holds no FP64 figure)
FP64_PEAK_GFLOPS = 1010.8


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="c4_mixed", choices=["c4_mixed", "c2_fp64", "small", "c5_adjoint", "c3_uneven"])
    p.add_argument("--chains", type=int, default=0, help="chains per GPU of the mixed batch (default 64)")
    p.add_argument("--delay", type=int, default=0,
                   help="delay depth of the mixed batch (0: chosen by the autotuner during warm-up)")
    p.add_argument("--flush", type=int, default=2, choices=[0, 1, 2],
                   help="round update: 2 exact (double-float Woodbury update of the round from G, Ozaki-split "
                        "tcgen05 products, double-float wraps), 1 tcgen05 flush of the FP32 panels, 0 mma.sync "
                        "flush of them")
    p.add_argument("--plain-steps", type=int, default=3, help="timed blocks of the plain FP64 chain")
    p.add_argument("--cpu-slices", type=int, default=0, help="slices per chain in the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--graphs", type=int, default=1, choices=[0, 1],
                   help="replay each slice's family steps from a captured CUDA graph (mixed batches)")
    p.add_argument("--gemm-engine", type=int, default=1, choices=[0, 1],
                   help="engine of the recompute's GEMMs (mixed batches): 0 double-float on the FP32 pipe, "
                        "1 Ozaki-split BF16 on the tensor cores")
    p.add_argument("--flush-tile", type=int, default=0, choices=[0, 64, 32, 2, 1],
                   help="flush of the exact round update in --profile-block runs (0: the library default)")
    p.add_argument("--profile-block", type=int, default=0, metavar="C",
                   help="profiling run instead of the benchmark: C chains of the workload's model in one "
                        "group (delay depth 64, no graphs, the --flush round update), one warm-up block of "
                        "ngroup slices, then one block inside an NVTX range named 'block' (for ncu "
                        "--nvtx-include block/); prints the chains' largest drift")
    return p.parse_args()


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d["bf16_tflops_sustained"], "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


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
    return M.build_model(spec, twist_seed=11, twist=1e-3)


def config_of(name: str, m, n_gpus: int, chains: int, extra: dict | None = None) -> dict:
    d = {
        "workload": {"c2_fp64": "14x14 SOC EPSOCZ, Lt=1000, plain FP64, 1 chain per GPU",
                     "c4_mixed": f"14x14 SOC EPSOCZ, Lt=1000, batched mixed precision, {chains} chains per GPU",
                     "small": f"6x6 SOC EPSOCZ, Lt=100, batched mixed precision, {chains} chains per GPU"}[name],
        "L": int(m.lat.dlength[0]), "ns": m.ns, "nelec": m.nelec, "ntime": m.ntime,
        "ngroup": m.ngroup, "dtau": m.spec.delt, "lambda": m.spec.ep_parameter, "alpha": 0.3,
        "omega": m.spec.omega, "chains_per_gpu": chains, "parallelism": f"replicas x{n_gpus}",
        "step": f"{m.ngroup} slices (one stabilisation block) of every chain; {m.ntime // m.ngroup} steps = 1 sweep",
        "proposal": "uniform, half-width 0.5 (mod_update.f90:84)",
        "measurement": "not in the timed region (equal-time measurement runs once per sweep)",
        "l2": "no flush: G alone is 2.46 MB per chain (x2 buffers) and expKV 0.2 GB per chain, "
              "well above the 129 MB L2",
    }
    if extra:
        d.update(extra)
    return d


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap,utilization.gpu,utilization.memory")

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
        sm, smax, pw, reasons, ug, um = [], [], [], set(), [], []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                pw.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
            try:   # percent of the sample period with a kernel running / with device memory read or written
                ug.append(float(parts[8]))
                um.append(float(parts[9]))
            except (IndexError, ValueError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_median": float(np.median(pw)) if pw else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "gpu_util_pct_median": float(np.median(ug)) if ug else None,
                "mem_util_pct_median": float(np.median(um)) if um else None}


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
    """The oracle (line-cited FP64 restatement of the reference CPU path) on
    all host cores, one independent chain per core, for a bounded sample of
    slices of one backward sweep."""
    from oracle.oracle import OracleChain
    cores = os.cpu_count() or 1
    o = OracleChain(m, field=field, seed_words=words, meas=False)
    o.init_expkv()
    o.init_g(1)
    secs = o.time_parallel(cores, cores, 1, slices)
    sweeps = cores * slices / m.ntime
    return {"value": sweeps / secs, "unit": "chain-sweeps/s", "cores": cores, "kind": "port",
            "sample": f"{cores} chains x {slices} slices of one backward sweep ({slices}/{m.ntime} sweep each, "
                      f"incl. {slices // m.ngroup} recomputes), {secs:.1f} s wall",
            "per_core": sweeps / secs / cores}


def run_reference(args, world, rank):
    if rank != 0:
        return
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.rng import seed_words
    name = "small" if args.workload == "small" else "c2_fp64"
    m = workload_model(name)
    f = M.field_gaussian(m, 2)
    slices = args.cpu_slices or (10 if m.ntime >= 1000 else 20)
    for _ in range(min(args.warmup, 1)):
        cpu_baseline(m, f, seed_words(42), max(1, slices // 5))
    vals = [cpu_baseline(m, f, seed_words(42), slices) for _ in range(args.steps)]
    v = float(np.mean([x["value"] for x in vals]))
    cb = dict(vals[-1])
    cb["value"] = v
    ref_config = config_of(name, m, args.gpus, cb["cores"])
    ref_config["workload"] = (f"{int(m.lat.dlength[0])}x{int(m.lat.dlength[0])} SOC EPSOCZ, Lt={m.ntime}: the "
                              "reference's CPU path (the line-cited C++ FP64 restatement), one chain per host core, "
                              f"{cb['cores']} cores")
    out = {"metric": METRIC, "value": v, "unit": "chain-sweeps/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * (m.ngroup / m.ntime) / v,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic", "config": ref_config, "impl": "reference",
           "cpu_baseline": cb, "e2e": {"value": v, "unit": "chain-sweeps/s", "h2d_bytes_per_step": 0,
                                       "d2h_bytes_per_step": 0},
           "note": "the reference Fortran cannot be built on these machines (no Fortran compiler, no "
                   "LAPACK); this arm times the oracle, the line-cited C++ FP64 restatement of the same path, "
                   "one chain per host core"}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
class Cursor:
    """(loop, first slice) of the next block in the sweep order."""

    def __init__(self, m):
        self.m = m
        self.loop, self.tc = 1, 1

    def next(self):
        out = (self.loop, self.tc)
        self.tc += self.m.ngroup
        if self.tc > self.m.ntime:
            self.loop += 1
            self.tc = 1
        return out


def g_error_full_size(m, rank: int, flush: int) -> dict:
    """Green's-function and observable error of the mixed form at full size
    on identical phonon fields: the benchmark's first two chains (seeds 3000,
    3001) run the first block of sweep 1 (slices Lt..Lt-9, the stabilised
    recompute at its end) in a mixed batch; the plain FP64 chain then
    recomputes G at the same slice from the mixed chain's own field
    (init_g_T0 + get_g_scratch_T0) and the two G are compared (relative
    Frobenius), with ln_cw beside, and one equal-time measurement record
    (every observable of ms_take_measurement with its k-space part) taken
    from each G at slice Lt/2 of that field."""
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.engine import PqmcBatch, PqmcChain
    from pqmc_allinone_gb300.rng import seed_words
    seeds = [3000 + i + 1000 * rank for i in range(2)]
    b = PqmcBatch([m] * 2, [M.field_gaussian(m, s) for s in seeds], [seed_words(s) for s in seeds], precision=1,
                  meas=True)
    b.set_flush(flush)
    b.init()
    b.sweep_slices(1, 1, m.ngroup)
    t = m.ntime - m.ngroup + 1
    errs, dl, obs, obs_max = [], [], [], []
    for c in b.chains:
        p = PqmcChain(m, field=c.field(), rng_words=seed_words(1), meas=True)
        p.init_expkv()
        p.init_g(1)
        p.get_g_scratch(t, False, 1)
        g0, g1 = p.g(), c.g()
        errs.append(float(np.linalg.norm(g1 - g0) / np.linalg.norm(g0)))
        dl.append(abs(c.state()["ln_cw"].real - p.state()["ln_cw"].real))
        r0 = p.begin_measure(False, m.ntime // 2, 0)
        r1 = c.begin_measure(False, m.ntime // 2, 0)
        obs.append(float(np.linalg.norm(r1 - r0) / np.linalg.norm(r0)))
        big = np.abs(r0) > 1e-6 * np.abs(r0).max()
        obs_max.append(float(np.max(np.abs(r1 - r0)[big] / np.abs(r0)[big])))
        p.close()
    drift = max(c.state()["err_g_rel_max"] for c in b.chains)
    b.close()
    return {"recompute_vs_fp64_rel_max": max(errs), "re_ln_cw_abs_diff_max": max(dl),
            "observables_rel_fro_max": max(obs), "observables_componentwise_rel_max": max(obs_max),
            "fast_path_drift_in_block_rel_max": drift, "seeds": seeds,
            "definition": "||G_mixed - G_fp64||_F / ||G_fp64||_F at the recompute closing the first block of "
                          f"sweep 1 (slice {t}), same phonon field, the benchmark's chains 0 and 1; the FP64 G from "
                          "the plain single-chain path (parity-tested against the oracle at this size); observables: "
                          "one measurement record (all observables and their k-space parts) from each G at slice "
                          "Lt/2, relative Frobenius and the largest relative error of components above 1e-6 of "
                          "the largest"}


def run_profile_block(args) -> None:
    """A short, self-contained run for kernel captures: one chain group, no
    CUDA graphs (each kernel is its own launch), a warm-up block and one
    block inside the NVTX range 'block'."""
    import torch
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.engine import PqmcBatch
    from pqmc_allinone_gb300.rng import seed_words
    m = workload_model("small" if args.workload == "small" else "c4_mixed")
    c = args.profile_block
    seeds = [3000 + i for i in range(c)]
    b = PqmcBatch([m] * c, [M.field_gaussian(m, s) for s in seeds], [seed_words(s) for s in seeds], precision=1)
    b.set_graphs(False)
    b.set_flush(args.flush)
    b.set_delay(args.delay or 64)
    b.set_gemm_engine(args.gemm_engine)
    if args.flush_tile:
        b.set_flush_tile(args.flush_tile)
    b.init()
    b.sweep_slices(1, 1, m.ngroup)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("block")
    b.sweep_slices(1, 1 + m.ngroup, m.ngroup)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    drift = max(ch.state()["err_g_rel_max"] for ch in b.chains)
    free, total = torch.cuda.mem_get_info()
    b.close()
    print(json.dumps({"profile_block": c, "flush": args.flush, "ns": m.ns, "ntime": m.ntime,
                      "drift_rel_max": drift, "device_gb_in_use": (total - free) / 1e9}))


def flush_standalone(m, depth: int, flush: int) -> dict:
    """The round update's products timed alone: one chain group of 8 chains
    (nothing else on the GPU), phase timers over one block of 10 slices."""
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.engine import PqmcBatch
    from pqmc_allinone_gb300.rng import seed_words
    seeds = [3000 + i for i in range(8)]
    b = PqmcBatch([m] * 8, [M.field_gaussian(m, s) for s in seeds], [seed_words(s) for s in seeds], precision=1)
    b.set_flush(flush)
    b.set_delay(depth)
    b.init()
    b.sweep_slices(1, 1, m.ngroup)   # warm-up block
    b.set_timing(True)
    b.sweep_slices(1, 1 + m.ngroup, m.ngroup)
    ph = b.timing()
    rounds = sum(b.flush_rounds())
    b.set_timing(False)
    b.close()
    ms, n = ph["flush"]
    bytes_alg = 32.0 * m.ns * m.ns * rounds
    return {"chains": 8, "flush_ms_per_launch_pair": ms / max(1, n), "rounds_with_columns": rounds,
            "launches": n, "achieved_gbs": bytes_alg / (ms * 1e-3) / 1e9 if ms > 0 else 0.0,
            "algorithmic_bytes_per_round": 32.0 * m.ns * m.ns * 8}


def run_plain(m, steps: int, rank: int) -> dict:
    """Plain single-chain FP64 form on this GPU (bit-identical decisions to
    the oracle), same block definition; wall time between device syncs (every
    C-ABI call synchronises its stream)."""
    import torch
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.engine import PqmcChain
    from pqmc_allinone_gb300.rng import seed_words
    ch = PqmcChain(m, field=M.field_gaussian(m, 2 + rank), rng_words=seed_words(1000 + rank))
    ch.init_expkv()
    ch.init_g(1)
    cur = Cursor(m)
    loop, tc = cur.next()
    ch.sweep_slices(loop, tc, m.ngroup)          # warm-up block
    torch.cuda.synchronize()
    s0 = ch.state()
    t0 = time.perf_counter()
    for _ in range(steps):
        loop, tc = cur.next()
        ch.sweep_slices(loop, tc, m.ngroup)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    s1 = ch.state()
    acc = s1["positive_accept"] - s0["positive_accept"]
    prop = acc + s1["negative_accept"] - s0["negative_accept"]
    ch.close()
    return {"value": (m.ngroup / m.ntime) / dt, "unit": "sweeps/s", "ms_per_step": dt * 1000.0,
            "steps": steps, "accept_ratio": acc / max(1, prop), "err_g_rel_max": s1["err_g_rel_max"]}


def mixed_dtype(args) -> str:
    """The arithmetic of the mixed batch, as the dtype string of its lines."""
    rec = ("recompute GEMMs bf16 Ozaki slices x6 with exact level sums, summed in double-float; "
           "Cholesky, triangular inverse and Gauss-Jordan in double-float"
           if args.gemm_engine == 1 else "double-float recompute (compensated FP32-pipe GEMMs)")
    if args.flush == 2:
        return ("double-float (48-bit) G and wraps; fp32 scan ratios; round update from G: fp32 inverse + "
                "double-float Newton step, bf16 Ozaki slices x5 with exact level sums; " + rec)
    return "bf16x3 tensor products + fp32 (fast path) on a double-float G; " + rec


def run_mixed(args, world, rank, local):
    import torch
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.engine import PqmcBatch, kernel_launches
    from pqmc_allinone_gb300.rng import seed_words

    torch.cuda.set_device(local)
    m = workload_model(args.workload)
    C = args.chains or (64 if args.workload == "c4_mixed" else 8)
    seeds = [3000 + i + 1000 * rank for i in range(C)]
    fields = [M.field_gaussian(m, s) for s in seeds]
    b = PqmcBatch([m] * C, fields, [seed_words(s) for s in seeds], precision=1)
    b.set_graphs(bool(args.graphs))
    b.set_flush(args.flush)
    b.set_gemm_engine(args.gemm_engine)
    t0 = time.perf_counter()
    b.init()
    t_init = time.perf_counter() - t0
    cur = Cursor(m)
    tune = None
    if args.delay > 0:
        b.set_delay(args.delay)
        b.set_flush(args.flush)
        depth = args.delay
    else:
        # the autotuner runs one block per candidate depth (part of the warm-up);
        # the tensor-core round updates take at most 64 columns
        cands = (16, 32, 48, 64) if args.flush in (1, 2) else (32, 48, 64, 96, 128)
        depth, table = b.autotune(cur.loop, cur.tc, m.ngroup, cands)
        for _ in cands:
            cur.next()
        (tile, ftile, qc), ttable, ftable, qtable = b.autotune_tiles(cur.loop, cur.tc, m.ngroup)
        for _ in range(b.tiles_timed(ttable, ftable, qtable)):   # the blocks the timed tiles ran
            cur.next()
        tune = {"candidates_ms_per_slice": table, "chosen": depth,
                "wrap_tile_ms_per_slice": {b.WRAP_TILES[k]: v for k, v in ttable.items()},
                "wrap_tile_chosen": b.WRAP_TILES[tile],
                "flush_tile_ms_per_slice": {b.flush_tile_name(k): v for k, v in ftable.items()},
                "flush_tile_chosen": b.flush_tile_name(ftile),
                "scan_chunk_ms_per_slice": [[f"{k} panel columns", v] for k, v in qtable],
                "scan_chunk_chosen": f"{qc} panel columns"}
    for _ in range(args.warmup):
        b.sweep_slices(*cur.next(), m.ngroup)
    torch.cuda.synchronize()
    st0 = [c.state() for c in b.chains]
    n0 = kernel_launches()
    stream = torch.cuda.ExternalStream(b.stream())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local)
    barrier(world)
    clk.start()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        b.sweep_slices(*cur.next(), m.ngroup)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier(world)
    launches = kernel_launches() - n0
    binfo = b.info()
    binfo["slice_graphs"] = bool(args.graphs)
    binfo["recompute_gemm_engine"] = ("Ozaki-split BF16, tensor cores" if b.gemm_engine() == 1
                                      else "double-float, FP32 pipe")
    t_step = max_over_ranks(world, ev0.elapsed_time(ev1) / 1000.0 / args.steps)
    per_gpu = C * (m.ngroup / m.ntime) / t_step
    value = world * per_gpu
    st1 = [c.state() for c in b.chains]
    acc = sum(s1["positive_accept"] - s0["positive_accept"] for s0, s1 in zip(st0, st1))
    rej = sum(s1["negative_accept"] - s0["negative_accept"] for s0, s1 in zip(st0, st1))
    drift = max(s["err_g_rel_max"] for s in st1)
    # phase breakdown on two further blocks, outside the timed region (the
    # event timers between phases bypass the slice graphs)
    b.set_timing(True)
    for _ in range(2):
        b.sweep_slices(*cur.next(), m.ngroup)
    torch.cuda.synchronize()
    phases = b.timing()
    rounds = b.flush_rounds()
    scanprof = b.scan_profile()
    b.set_timing(False)
    st2 = [c.state() for c in b.chains]
    # the phase timers follow chain group 0 (the first C/groups chains)
    g0 = C // max(1, binfo["groups"])
    acc_ph = sum(s2["positive_accept"] - s1["positive_accept"] for s1, s2 in zip(st1[:g0], st2[:g0]))

    # The contraction the delayed update reduces to, per round with columns:
    # G += X Z (exact update, k_xgemm<1>; X = G(:,S) M by k_xgemm<0> first)
    # or G += A B (FP32 panels, k_bflush_um / k_bflush).  At delay depth K it
    # does 8*Ns^2*K flop (counted once, not the slice products) against
    # 32*Ns^2 bytes of the double-float G (read and write): 16 flop/B at
    # K = 64, under the HBM roof (x16 the measured copy bandwidth), far below
    # the tensor roof.  Algorithmic bytes: 32*Ns^2 per round with columns
    # (counted on the device per chain) over the flush phase's own event
    # time on chain group 0's stream (the other groups' kernels run beside
    # it); the same figure with nothing else on the GPU is reported apart.
    pk = peaks()
    dim = 4
    flush_ms, flush_n = phases["flush"]
    rounds_g0 = sum(rounds[:g0])
    bytes_alg = 32.0 * m.ns * m.ns * rounds_g0
    flops = 8.0 * m.ns * m.ns * dim * acc_ph
    secs = flush_ms * 1e-3
    achieved = bytes_alg / secs / 1e9 if secs > 0 else 0.0
    key = {2: "k_xgemm_flush", 1: "k_bflush_um"}.get(args.flush)
    traffic, traffic_note = None, None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tj = json.load(f).get(key) if key else None
            if tj and tj.get("ns") == m.ns:
                # DRAM bytes of one launch, scaled to group 0's chains
                traffic = tj["bytes_per_launch"] * g0 / tj["chains"]
                traffic_note = tj.get("note")
    except Exception:
        pass
    kname = {2: "k_xgemm<1> (round update G += X Z from G: Ozaki-split BF16 tcgen05 products, exact level sums "
                "in tensor memory, double-float epilogue; after k_xgemm<0>, X = G(:,S) M)",
             1: "k_bflush_um (rank-K flush G += A B, tcgen05 BF16x3 products, FP32 accumulator in tensor memory)",
             0: "k_bflush (rank-K flush G += A B, mma.sync BF16x3 products, FP32 accumulate)"}[args.flush]
    sc_cyc = sum(x[0] for x in scanprof)
    sc_acc = sum(x[1] for x in scanprof)
    sc_rej = sum(x[2] for x in scanprof)
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
            "per_launch_bytes_algorithmic": bytes_alg / max(1, flush_n),
            "per_launch_bytes_algorithmic_all_columns": 32.0 * m.ns * m.ns * g0,
            "traffic_note": traffic_note,
            "tensor_achieved_tflops": flops / secs / 1e12 if secs > 0 else 0.0,
            "tensor_peak_tflops": pk["bf16_tflops_sustained"],
            "kernel": kname,
            "algorithmic": "32*Ns^2 bytes (G read + write, double-float) per round with columns (device count, "
                           "chain group 0) and 8*Ns^2*dim flop per accepted move, over the flush phase's event time "
                           "during two blocks (the other groups' kernels share the GPU meanwhile; launches of empty "
                           "rounds included)",
            "flush_rounds_group0": rounds_g0,
            "peak_source": f"{pk['source']} HBM copy bandwidth; bf16 sustained for the tensor figure",
            "scan": {"kernel": "k_bscan (sequential ratio scan, one CTA per chain)",
                     "sm_cycles_per_accepted_move": sc_cyc / max(1, sc_acc),
                     "sm_cycles_per_proposal": sc_cyc / max(1, sc_acc + sc_rej),
                     "accepted": sc_acc, "rejected": sc_rej,
                     "definition": "device clock64 of every scan CTA from its start to its last bookkeeping, "
                                   "summed over the two phase-timed blocks of all chains, over the moves it "
                                   "accepted (the scan's cost model: ~17k cycles per accepted move, 11k of them the "
                                   "panel stream)"},
            "dominant_by_time": "k_bscan: the sequential ratio scan, one CTA per chain, latency-bound by the "
                                "Markov order, neither an HBM nor a tensor-pipe kernel (its cycles per accepted "
                                "move are under scan)"}
    total_ms = sum(v[0] for v in phases.values())
    phase_out = {k: {"ms_per_step": v[0] / 2, "share": v[0] / total_ms if total_ms else None,
                     "launch_groups": v[1]} for k, v in phases.items()}

    # end to end through the C-ABI with host buffers: every chain's field block
    # for the step goes host->device (the host copy, kept in step), the block
    # runs, the updated block and each chain's state come back
    e2e = run_e2e_mixed(b, m, cur, min(args.steps, 5))
    b.close()
    gerr = g_error_full_size(m, rank, args.flush)
    standalone = flush_standalone(m, depth, args.flush) if rank == 0 else None
    roof["standalone"] = standalone
    roof["standalone_frac"] = (standalone["achieved_gbs"] / pk["hbm_gbs"]) if standalone else None

    plain = None if args.no_plain else run_plain(m, args.plain_steps, rank)
    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from pqmc_allinone_gb300 import model as M2
        from pqmc_allinone_gb300.rng import seed_words as sw
        cb = cpu_baseline(m, M2.field_gaussian(m, 2), sw(42), args.cpu_slices or 10)
    if rank != 0:
        return
    out = {"metric": METRIC,
           "value": value, "unit": "chain-sweeps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": mixed_dtype(args),
           "data": "synthetic (x ~ N(0,0.5^2), seeds 3000+i)",
           "config": config_of(args.workload, m, world, C, {"autotune": tune, **binfo}),
           "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "clocks": clocks,
           "cpu_baseline": cb, "plain_fp64": plain,
           "speedup_vs_plain_fp64": (per_gpu / plain["value"]) if plain else None,
           "g_error": {"fast_path_drift_rel_max": drift,
                       "gate": 1e-8,
                       "meets_gate": bool(drift <= 1e-8 and gerr["recompute_vs_fp64_rel_max"] <= 1e-8),
                       "definition": "max over chains and recomputes in the timed region of "
                                     "||G_fast - G_recomputed||_F / ||G_recomputed||_F (drift of the fast "
                                     "path over one ngroup block; the recompute is FP64-class)",
                       "recompute_vs_fp64": gerr},
           "accept_ratio": acc / max(1, acc + rej), "phases": phase_out, "init_s": t_init}
    print(json.dumps(out))


def run_e2e_mixed(b, m, cur, steps: int) -> dict:
    import torch
    C = len(b.chains)
    nb, blk = m.n_bf, m.ngroup
    # the fields live on the host (pinned); every step the block of slices
    # it touches goes up for all chains in one call, the batch runs it, the
    # updated block and every chain's state come back
    field = torch.empty((C, m.ntime, nb), dtype=torch.float64, pin_memory=True)   # (n_bf, ntime) per chain
    io = torch.empty((C, blk, nb), dtype=torch.float64, pin_memory=True)          # chain after chain
    fv, iov = field.numpy(), io.numpy()
    for i, c in enumerate(b.chains):
        fv[i] = c.field().T
    state_bytes = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        loop, tc = cur.next()
        first_time = tc if loop % 2 == 0 else m.ntime - (tc + blk - 1) + 1
        iov[:] = fv[:, first_time - 1:first_time - 1 + blk]
        b.field_slices(first_time, blk, iov, True)
        b.sweep_slices(loop, tc, blk)
        b.field_slices(first_time, blk, iov, False)
        fv[:, first_time - 1:first_time - 1 + blk] = iov
        states = b.states()
        state_bytes = len(states) * 104
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    blk_bytes = C * nb * blk * 8
    return {"value": C * (blk / m.ntime) / dt, "unit": "chain-sweeps/s", "h2d_bytes_per_step": int(blk_bytes),
            "d2h_bytes_per_step": int(blk_bytes + state_bytes), "steps": steps,
            "path": "pqmc_batch_field_slices (pinned host, all chains) + pqmc_batch_sweep_slices + "
                    "pqmc_batch_field_slices back + pqmc_batch_states"}


def run_plain_headline(args, world, rank, local):
    """--workload c2_fp64: the plain FP64 single chain as the headline."""
    import torch
    from pqmc_allinone_gb300.engine import kernel_launches
    torch.cuda.set_device(local)
    m = workload_model("c2_fp64")
    n0 = kernel_launches()
    clk = ClockSampler(local)
    barrier(world)
    clk.start()
    p = run_plain(m, args.steps, rank)
    clocks = clk.stop()
    launches = kernel_launches() - n0
    t_step = max_over_ranks(world, p["ms_per_step"] / 1000.0)
    if rank != 0:
        return
    out = {"metric": "sweeps/s @14x14 Lt=1000 (plain FP64)", "value": world * (m.ngroup / m.ntime) / t_step,
           "unit": "sweeps/s", "n_gpus": world, "steps": args.steps, "warmup": 1, "ms_per_step": t_step * 1000,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
           "data": "synthetic", "config": config_of("c2_fp64", m, world, 1), "clocks": clocks,
           "gpu_launches": int(launches), "plain_fp64": p, "roofline": None, "cpu_baseline": None,
           "e2e": None}
    print(json.dumps(out))


def uneven_models(C: int, rank: int):
    """Chains of uneven size: per chain i a seed 1000+i draws L from {8,10,12},
    Lt from {200,400,600} and lambda ~ U(0.5,1.0); spin-orbit lattice with
    static alpha=0.3, dtau=0.1, half filling, omega=1, ngroup=10; the field is
    x ~ N(0,0.5^2) from the same seed."""
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.rng import seed_words
    out = []
    for i in range(C):
        seed = 1000 + i + 100000 * rank
        r = np.random.default_rng(seed)
        L = int(r.choice([8, 10, 12]))
        nt = int(r.choice([200, 400, 600]))
        lam = float(r.uniform(0.5, 1.0))
        spec = M.epsocz_spec(L, lam=lam, alpha=0.3, ntime=nt, ngroup=10, filling=0.5, jump_distance=0.5)
        m = M.build_model(spec, twist_seed=11, twist=1e-3)
        out.append((m, M.field_gaussian(m, seed), seed_words(seed)))
    return out


def run_uneven(args, world, rank, local):
    """--workload c3_uneven: 256 chains of uneven L and Lt in one mixed batch
    (geometry classes interleaved on their own streams, slice graphs, delay
    depth autotuned per class); a step is one sweep of every chain (each over
    its own Lt slices)."""
    import torch
    from pqmc_allinone_gb300.engine import PqmcBatch, PqmcChain, kernel_launches
    torch.cuda.set_device(local)
    C = args.chains or 256
    t0 = time.perf_counter()
    ms = uneven_models(C, rank)
    t_models = time.perf_counter() - t0
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.set_graphs(bool(args.graphs))
    b.set_gemm_engine(args.gemm_engine)
    t0 = time.perf_counter()
    b.init()
    t_init = time.perf_counter() - t0
    # autotune on the first blocks of sweep 1 (depth, then the wrap tile),
    # then finish sweep 1 from the slice the timed candidates reached (a
    # candidate the round update cannot take is skipped and runs no slices)
    if args.delay:
        cands = (args.delay,)
    else:
        cands = (16, 32, 48, 64) if args.flush in (1, 2) else (32, 64, 96)
    best, table = b.autotune(1, 1, 10, cands)
    tc = 1 + 10 * sum(1 for v in table.values() if v >= 0)
    (tile, ftile, qc), ttable, ftable, qtable = b.autotune_tiles(1, tc, 10)
    tc += 10 * b.tiles_timed(ttable, ftable, qtable)
    b.sweep_slices(1, tc, max(m.ntime for m, _, _ in ms))
    loop = 2
    for _ in range(args.warmup):
        b.sweep(loop)
        loop += 1
    torch.cuda.synchronize()
    st0 = [c.state() for c in b.chains]
    rounds0 = b.flush_rounds()
    n0 = kernel_launches()
    stream = torch.cuda.ExternalStream(b.stream())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local)
    barrier(world)
    clk.start()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        b.sweep(loop)
        loop += 1
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier(world)
    launches = kernel_launches() - n0
    t_step = max_over_ranks(world, ev0.elapsed_time(ev1) / 1000.0 / args.steps)
    st1 = [c.state() for c in b.chains]
    acc = sum(s1["positive_accept"] - s0["positive_accept"] for s0, s1 in zip(st0, st1))
    rej = sum(s1["negative_accept"] - s0["negative_accept"] for s0, s1 in zip(st0, st1))
    drift = max(s["err_g_rel_max"] for s in st1)
    rounds = [r1 - r0 for r0, r1 in zip(rounds0, b.flush_rounds())]
    classes = b.classes()
    n_graphs = b.graph_count()
    b.close()
    # step-level roofline: the round updates' and the wraps' algorithmic G
    # traffic (double-float G read + write, 32 Ns^2 bytes per pass) over the
    # step time; the scan and the recompute share the GPU meanwhile
    pk = peaks()
    g_bytes = sum(32.0 * m.ns * m.ns * (r + len(m.pf) * m.ntime * args.steps) for (m, _, _), r in zip(ms, rounds))
    achieved = g_bytes / (t_step * args.steps) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": None,
            "kernel": "whole step: k_xgemm<1> (round updates, one G pass per round with columns, device-counted) "
                      "and the wraps (one G pass per family and slice)",
            "algorithmic": "32*Ns^2 bytes per G pass (double-float read + write), summed over chains, over the "
                           "timed steps' event time; not a per-kernel figure (no phase timers in this mode)",
            "rounds_with_columns": int(sum(rounds)), "peak_source": f"{pk['source']} HBM copy bandwidth"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle on the host cores for one chain of each L of the mix
        # (20 slices each), scaled to the mix: core-seconds of one sweep of
        # every chain = sum_i Lt_i * (seconds per slice per core for L_i)
        per_slice, samples = {}, []
        for L in (8, 10, 12):
            x = next((x for x in ms if int(x[0].lat.dlength[0]) == L), None)
            if x is None:
                continue
            cb = cpu_baseline(x[0], x[1], x[2], 20)
            per_slice[L] = 1.0 / (cb["per_core"] * x[0].ntime)
            samples.append(f"L={L} (Lt={x[0].ntime}): {cb['sample']}")
        cores = os.cpu_count() or 1
        core_s = sum(m.ntime * per_slice[int(m.lat.dlength[0])] for m, _, _ in ms)
        cpu = {"value": C / (core_s / cores), "unit": "chain-sweeps/s", "cores": cores, "kind": "port",
               "sample": "; ".join(samples) + f"; scaled to the {C}-chain mix by Lt, {cores} chains at a time"}
    # plain FP64 single chains on a sample (one chain per L at Lt=200, one
    # sweep each), scaled to the batch's mix by Lt: the sequential FP64 form
    plain = None
    if not args.no_plain:
        secs = {}
        for L in (8, 10, 12):
            m, f, w = next((x for x in ms if int(x[0].lat.dlength[0]) == L), (None, None, None))
            if m is None:
                continue
            from pqmc_allinone_gb300 import model as M
            spec = M.epsocz_spec(L, lam=m.spec.ep_parameter, alpha=0.3, ntime=200, ngroup=10, filling=0.5,
                                 jump_distance=0.5)
            m2 = M.build_model(spec, twist_seed=11, twist=1e-3)
            ch = PqmcChain(m2, field=M.field_gaussian(m2, 7), rng_words=w)
            ch.init_expkv()
            ch.init_g(1)
            torch.cuda.synchronize()
            ta = time.perf_counter()
            ch.sweep(1, 1)
            torch.cuda.synchronize()
            secs[L] = time.perf_counter() - ta
            ch.close()
        est = sum(secs[int(m.lat.dlength[0])] * m.ntime / 200 for m, _, _ in ms)
        plain = {"value": C / est, "unit": "chain-sweeps/s", "sample_s_per_sweep_at_lt200": secs,
                 "method": "one plain FP64 chain per L at Lt=200 timed over one sweep; the batch's "
                           "sum of per-chain sweep times scaled by Lt (chains one after another)"}
        # the FP64 batch (single-chain kernels, chains driven concurrently
        # from host threads) on the first 24 chains of the mix, one sweep
        sub = ms[:24]
        fb = PqmcBatch([m for m, _, _ in sub], [f for _, f, _ in sub], [w for _, _, w in sub], precision=0)
        fb.init()
        torch.cuda.synchronize()
        ta = time.perf_counter()
        fb.sweep(1)
        torch.cuda.synchronize()
        tb = time.perf_counter() - ta
        fb.close()
        plain["fp64_batch_sample"] = {"chains": len(sub), "seconds": tb, "value": len(sub) / tb,
                                      "unit": "chain-sweeps/s",
                                      "note": "PQMC_PREC_FP64 batch of the first 24 chains, one sweep, wall time"}
    if rank != 0:
        return
    Ls = [int(m.lat.dlength[0]) for m, _, _ in ms]
    Lts = [m.ntime for m, _, _ in ms]
    out = {"metric": "chain-sweeps/s, 256 chains of uneven L in {8,10,12} and Lt in {200,400,600}",
           "value": world * C / t_step, "unit": "chain-sweeps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None,
           "dtype": mixed_dtype(args),
           "data": "synthetic (per chain i: seed 1000+i draws L, Lt, lambda~U(0.5,1); x ~ N(0,0.5^2))",
           "config": {"workload": f"{C} chains of uneven size, mixed precision, one batch per GPU",
                      "chains_by_L": {L: Ls.count(L) for L in (8, 10, 12)},
                      "chains_by_Lt": {t: Lts.count(t) for t in (200, 400, 600)},
                      "classes": classes, "graphs": bool(args.graphs), "slice_graphs_held": n_graphs,
                      "autotune": {"candidates_ms_per_slice_summed_over_classes": table, "class0_depth": best,
                                   "wrap_tile_ms_per_slice_summed_over_classes":
                                       {b.WRAP_TILES[k]: v for k, v in ttable.items()},
                                   "class0_wrap_tile": b.WRAP_TILES[tile],
                                   "flush_tile_ms_per_slice_summed_over_classes":
                                       {b.flush_tile_name(k): v for k, v in ftable.items()},
                                   "class0_flush_tile": b.flush_tile_name(ftile),
                                   "scan_chunk_ms_per_slice_summed_over_classes":
                                       [[f"{k} panel columns", v] for k, v in qtable],
                                   "class0_scan_chunk": f"{qc} panel columns"},
                      "step": "one sweep of every chain (its own Lt slices, one recompute per 10 slices)",
                      "l2": "no flush: the batch's G, expKV and Q strings (tens of GB) far exceed the 129 MB L2",
                      "parallelism": f"replicas x{world}"},
           "gpu_launches": int(launches), "clocks": clocks, "plain_fp64_sequential_estimate": plain,
           "speedup_vs_plain_fp64": (C / t_step / plain["value"]) if plain else None,
           "g_error": {"fast_path_drift_rel_max": drift},
           "accept_ratio": acc / max(1, acc + rej), "models_s": t_models, "init_s": t_init,
           "roofline": roof, "cpu_baseline": cpu, "e2e": None}
    print(json.dumps(out))


def run_adjoint(args, world, rank, local):
    """--workload c5_adjoint: forward and hand-written adjoint of the projector
    log-weight log det(P^H B(Lt..1) P) for 32 chains of 10x10 SOC (Ns=200),
    Lt=400, through the torch.autograd.Function; gradients/s."""
    import torch
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.autograd import log_weight
    from pqmc_allinone_gb300.engine import PqmcChain, kernel_launches
    from pqmc_allinone_gb300.rng import seed_words
    torch.cuda.set_device(local)
    spec = M.epsocz_spec(10, lam=0.8, alpha=0.3, ntime=400, ngroup=10, filling=0.5, jump_distance=0.5)
    m = M.build_model(spec, twist_seed=11, twist=1e-3)
    B = args.chains or 32
    fields = [M.field_gaussian(m, 5000 + i + 1000 * rank) for i in range(B)]
    chains = [PqmcChain(m, field=f, rng_words=seed_words(5000 + i)) for i, f in enumerate(fields)]
    x = torch.tensor(np.stack(fields), dtype=torch.float64, device="cuda", requires_grad=True)

    def step():
        x.grad = None
        w = log_weight(x, chains)
        w.sum().backward()
        return w

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    n0 = kernel_launches()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = max_over_ranks(world, (time.perf_counter() - t0) / args.steps)
    if rank != 0:
        return
    # FP64 roofline: complex multiply-adds per gradient, counted from the
    # algorithm (8 flop each): the right-to-left pass propagates P (Ns x
    # nelec) through every family of every slice (dim Ns nelec each); the
    # left-to-right pass propagates the running right factor the same way and
    # wraps G (Ns x Ns) through every family (2 dim Ns^2 each); the
    # Householder QR of each block and the G rebuild per block are ignored
    dims = [t.dim for t in m.pf]
    cmac = m.ntime * sum(2 * d * m.ns * m.nelec + 2 * d * m.ns * m.ns for d in dims)
    flops = 8.0 * cmac
    achieved = B * flops / dt / 1e9
    roof = {"bound": "fp64", "achieved": achieved, "peak": FP64_PEAK_GFLOPS, "unit": "GFLOP/s",
            "frac": achieved / FP64_PEAK_GFLOPS, "traffic": None,
            "algorithmic": f"{flops / 1e9:.2f} GFLOP per gradient: 8 flop x Lt x sum over families of "
                           "(2 dim Ns nelec + 2 dim Ns^2) complex multiply-adds (both passes' propagation and "
                           "the G wraps; QR and per-block G rebuilds not counted)",
            "peak_source": "FP64 FMA loop over all SMs measured on this GPU (1010.8 GFLOP/s)"}
    cpu = None
    if not args.no_cpu_baseline:
        # the reference has no gradient: its route is central differences of
        # cal_new_weight_T0, 2 n_bf Lt weight evaluations per gradient
        from oracle.oracle import OracleChain
        o = OracleChain(m, field=fields[0], seed_words=seed_words(5000), meas=False)
        o.init_expkv()
        o.init_g(1)
        ta = time.perf_counter()
        o.cal_new_weight()
        tw = time.perf_counter() - ta
        n_eval = 2 * m.n_bf * m.ntime
        cpu = {"value": 1.0 / (tw * n_eval), "unit": "chain-gradients/s", "cores": 1, "kind": "port",
               "sample": f"one oracle cal_new_weight_T0 at 10x10, Lt=400 ({tw:.3f} s on one core); a gradient by "
                         f"central differences needs 2 n_bf Lt = {n_eval} of them (the reference has no adjoint)"}
    out = {"metric": "log-weight gradients/s (forward + adjoint) @10x10 Lt=400", "value": world * B / dt,
           "unit": "chain-gradients/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": dt * 1000.0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "c128", "data": "synthetic (x ~ N(0,0.5^2), seeds 5000+i)",
           "config": {"workload": f"10x10 SOC EPSOCZ, Lt=400, {B} chains, checkpoint every ngroup=10 slices",
                      "ns": m.ns, "nelec": m.nelec, "ntime": m.ntime, "chains": B},
           "gpu_launches": int(kernel_launches() - n0), "roofline": roof, "cpu_baseline": cpu, "e2e": None}
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        world, rank = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))
        run_reference(args, world, rank)
        return
    if args.profile_block:
        run_profile_block(args)
        return
    world, rank, local = dist_setup()
    if args.workload == "c2_fp64":
        run_plain_headline(args, world, rank, local)
    elif args.workload == "c5_adjoint":
        run_adjoint(args, world, rank, local)
    elif args.workload == "c3_uneven":
        run_uneven(args, world, rank, local)
    else:
        run_mixed(args, world, rank, local)


if __name__ == "__main__":
    main()
