"""Throughput of batched monitored Haar trajectories at L=24 on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one batch of B trajectories of the L=24 periodic Haar brickwork
(48 layers, p cycled over linspace(0.05, 0.35, 16)), every layer followed by
Born-rule measurements with collapse, and the final half-chain Renyi-2
entropy of every trajectory. FP32 state vectors, FP64 probabilities and
entropies. Metric: trajectory-layers per second (whole job, all ranks).

value : device time of K steps with the inputs (gates, measured sites,
        uniforms) already resident in HBM, CUDA events on the launch stream.
e2e   : the same work through the C ABI's one-call entry point
        (host sampling, pinned host->device upload, device run, results back).
The reference arm times the CPU FP64 oracle on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "trajectory-layers/s at L=24 (batched FP32 vs plain FP64) at |dS|<=1e-5"
UNIT = "trajectory-layers/s"
N_QUBITS = 24
PERIODS = 24
PASS_TRAFFIC_PER_TRAJ = 237.9e6  # DRAM bytes per trajectory per pass launch (ncu)
P_GRID = np.linspace(0.05, 0.35, 16)


def workload_config(batch):
    return {
        "workload": "haar-brickwork-L24-monitored",
        "n_qubits": N_QUBITS,
        "layers_per_trajectory": 2 * PERIODS,
        "trajectories_per_gpu": batch,
        "boundary": "periodic",
        "p": "linspace(0.05,0.35,16) cycled over trajectories",
        "measurement": "joint Born sampling per layer, chunks of 16 sites",
        "observables": "final half-chain Renyi-2 entropy per trajectory",
        "state_dtype": "complex64; probabilities/entropies FP64",
        "l2": "inputs larger than L2 (one 128 MiB state per trajectory)",
    }


def seeds_for(rank, batch, step=0):
    import mipt_gb300 as mg
    base = (rank * 1_000_003 + step) * batch
    return np.array([mg.trajectory_seed(0, base + i) for i in range(batch)], np.uint64)


def p_for(batch):
    return np.array([P_GRID[i % len(P_GRID)] for i in range(batch)])


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
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
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_sample(steps=1):
    """Oracle (FP64, all host threads): a bounded sample of the same workload."""
    from oracle import pyoracle
    threads = pyoracle.max_threads()
    count = threads
    periods = 1
    t0 = time.perf_counter()
    for s in range(steps):
        pyoracle.run_batch(0, s * count, count, N_QUBITS, periods, 0.2, True, 16, obs_flags=0, threads=threads)
    dt = time.perf_counter() - t0
    value = steps * count * 2 * periods / dt
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{count} trajectories x {2 * periods} layers of the L=24 workload (p=0.2) per step, FP64, "
                      f"one trajectory per host thread; final-state entropy omitted (the GPU arm includes it)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import pyoracle
    pyoracle.lib()
    for _ in range(args.warmup):
        pass  # the oracle has no warm-up state; W is honoured by skipping nothing
    t0 = time.perf_counter()
    res = cpu_sample(args.steps)
    dt = time.perf_counter() - t0
    line = {
        "impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.batch), "cpu_baseline": res,
        "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import mipt_gb300 as mg

    B = args.batch
    T = 2 * PERIODS
    batch = mg.Batch(N_QUBITS, PERIODS, capacity=B, fp64=False, observables=mg.OBS_S2_HALF,
                     tile_qubits=args.tile)
    seeds = seeds_for(rank, B)
    ps = p_for(B)

    # ---------------------------------------------------------- value
    batch.prepare(seeds, ps)
    for _ in range(max(3, args.warmup)):
        batch.execute()
        batch.fetch()
    batch.set_profiling(True)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record()
        for _ in range(args.steps):
            batch.execute()
        stop.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    out = batch.fetch()
    stats = batch.kernel_stats()  # last step, per launch category
    launches = batch.launches * args.steps
    batch.set_profiling(False)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    units = B * T * world * args.steps
    value = units / (ms / 1000.0)

    # ------------------------------------------------------------ e2e
    for _ in range(1):
        batch.run(seeds, ps)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.steps):
        batch.run(seeds_for(rank, B, s + 1), ps)
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = B * T * world * args.steps / e2e_s
    h2d = B * T * (N_QUBITS // 2) * 16 * 8 + B * T * 136  # FP32 gates + measurement records
    d2h = B * T * 88 + B * 4 * 8

    line = None
    if rank == 0:
        # Roofline of the dominant kernel (the tiled layer pass): algorithmic
        # bytes = one read + one write of every state per layer.
        pass_ms, pass_n = stats["pass"]
        layer_bytes = 2 * (1 << N_QUBITS) * 8
        alg_bytes_step = B * T * layer_bytes
        passes_per_layer = pass_n / T
        achieved = alg_bytes_step / (pass_ms / 1000.0) / 1e9
        peak, peak_kind = measured_peak_hbm()
        # DRAM traffic per pass launch: ncu measured 237.9 MB per trajectory
        # (read 134.3 MB + write 103.7 MB, the rest of the writes still in L2)
        # on 2 trajectories; each launch streams every state once, so it
        # scales with the batch (profiles/k_pass_rounds_L24_batch2.md).
        traffic = PASS_TRAFFIC_PER_TRAJ * B
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": traffic, "traffic_source": "ncu dram bytes, 2-trajectory capture scaled to B",
                    "peak_source": peak_kind,
                    "kernel": "k_pass (tiled brickwork layer pass)",
                    "alg_bytes_per_launch": alg_bytes_step / pass_n, "launch_ms": pass_ms / pass_n,
                    "passes_per_layer": passes_per_layer,
                    "kernel_ms_per_step": {k: v[0] for k, v in stats.items()}}
        # Final half-chain S_2: tensor-core Gram, 4 d_A^2 d_B real flops per
        # trajectory for the Hermitian half (d_A = d_B = 2^12).
        obs_ms = stats["observables"][0]
        gram_flops = B * 4.0 * float(1 << (N_QUBITS // 2)) ** 3
        gram = {"kernel": "k_gram_tc (tcgen05 3xTF32)", "ms_per_step": obs_ms,
                "alg_tflops": gram_flops / (obs_ms / 1000.0) / 1e12 if obs_ms > 0 else None}

        # Plain FP64 per-trajectory path on the same GPU, one trajectory.
        plain = mg.Batch(N_QUBITS, PERIODS, capacity=1, fp64=True, observables=mg.OBS_S2_HALF)
        plain.run(seeds[:1], ps[:1])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pr = plain.run(seeds[:1], ps[:1])
        plain_s = time.perf_counter() - t0
        plain_value = T / plain_s
        same = bool(np.array_equal(pr["outcomes"][0], out["outcomes"][0]))
        ds = abs(float(pr["obs"][0, 0, 1]) - float(out["obs"][0, 0, 1]))
        plain.close()

        cpu = cpu_sample(1) if world == 1 else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(B), "roofline": roofline, "gram": gram, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clocks.summary(),
            "plain_fp64": {"value": plain_value, "unit": UNIT, "path": "FP64 state, one trajectory per launch sequence",
                           "speedup_batched_fp32": value / plain_value},
            "dS": {"max_abs": ds, "same_outcomes": same, "observable": "final half-chain S_2, trajectory 0"},
        }
        print(json.dumps(line), flush=True)
    batch.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tile", type=int, default=0, help="local qubits per pass tile (0 = library default)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
