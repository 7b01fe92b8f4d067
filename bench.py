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
dS    : the final half-chain S_2 of two trajectories of the batch against the
        CPU FP64 oracle running the same seeds free on host threads.
per_layer_observables: the same workload with the half-chain S_2 after
        every layer (one step, device time).
plain_fp64: the plain FP64 path, one trajectory per launch sequence,
        device time and end to end.
gram  : the final S_2 Gram's time and algorithmic flops. The entropies are
        taken with the last layer's collapse pending, so each trajectory's
        Gram covers only the rows and columns outside its measured sites
        (the state is a product on them), formed over the smaller side; the
        flops count that block.
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
PASS_TRAFFIC_PER_TRAJ = 191.0e6  # DRAM bytes per trajectory per pass launch, two layers averaged (ncu)
GRAM_TENSOR_PIPE_PCT = 66.5  # ncu sm__pipe_tensor_cycles_active of the final S_2 Gram
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


def max_over_ranks(value, dist, device):
    """The slowest rank's figure (the whole job ends with it); the value itself
    on one rank (dist None)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(batch, layers, world, steps, seconds):
    """Trajectory-layers per second over all ranks: every rank runs `batch`
    trajectories of `layers` layers per step (weak scaling)."""
    return batch * layers * world * steps / seconds


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


def cpu_model():
    """The host CPU's model name (for the baseline record)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_sample(steps=1):
    """Oracle (FP64, all host threads): a bounded sample of the same workload.
    One trajectory per host thread runs 4 layers (p = 0.2) of the L=24 chain,
    then each final state's half-chain S_2 comes from its 2^12 x 2^12 Gram
    partner (numpy, all cores). The two parts are timed separately and
    weighted as one 48-layer trajectory weights them: 12 samples of 4 layers
    plus one final entropy per trajectory."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import pyoracle
    threads = pyoracle.max_threads()
    count = threads
    periods = 2
    t_layers = t_entropy = 0.0
    for s in range(steps):
        seeds = [pyoracle.trajectory_seed(0, s * count + i) for i in range(count)]
        t0 = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            states = list(ex.map(lambda sd: pyoracle.run_trajectory(int(sd), N_QUBITS, periods, 0.2, True, 16,
                                                                     want_state=True)["psi"], seeds))
        t1 = time.perf_counter()
        for psi in states:
            m = psi.reshape(-1, 1 << (N_QUBITS // 2))
            -np.log2(float(np.sum(np.abs(m.conj().T @ m) ** 2)))
        t2 = time.perf_counter()
        del states
        t_layers += t1 - t0
        t_entropy += t2 - t1
    layers = 2 * PERIODS
    # Wall seconds per trajectory at full host throughput (the layer samples
    # run one per thread, the entropies one after another on all cores).
    per_traj = t_layers / (steps * count) * (layers / (2 * periods)) + t_entropy / (steps * count)
    value = layers / per_traj
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "sample": f"{count} trajectories x {2 * periods} layers of the L=24 workload (p=0.2) per step, FP64, "
                      f"one trajectory per host thread ({t_layers / steps:.2f} s), then each final half-chain "
                      f"S_2 from the 2^12 x 2^12 Gram (numpy, all cores, {t_entropy / steps:.2f} s); weighted as "
                      f"{layers} layers + one final entropy per trajectory"}


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
    # |dS| against the CPU FP64 oracle: trajectories 0 and 9 of the batch run
    # free (48 layers) on host threads while the GPU is timed.
    oracle_idx = [i for i in (0, 9) if i < B] if (rank == 0 and not args.kernels_only) else []
    oracle_res = {}

    def oracle_leg(i):
        from oracle import pyoracle as orc
        r = orc.run_trajectory(int(seeds[i]), N_QUBITS, PERIODS, float(ps[i]), True, 16, want_state=True)
        m = r["psi"].reshape(-1, 1 << (N_QUBITS // 2))
        g = m.conj().T @ m
        d = orc.haar_draw(int(seeds[i]), N_QUBITS, PERIODS, float(ps[i]), True, 16)
        oc = np.zeros(T, np.uint64)
        for t in range(T):
            for j, q in enumerate(d["sites"][t, : d["sites_per_layer"][t]]):
                if r["outcomes"][t, j]:
                    oc[t] |= np.uint64(1) << np.uint64(int(q))
        oracle_res[i] = (-np.log2(float(np.sum(np.abs(g) ** 2))), oc)

    oracle_threads = [threading.Thread(target=oracle_leg, args=(i,), daemon=True) for i in oracle_idx]
    for th in oracle_threads:
        th.start()

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
    ms = max_over_ranks(ms, dist, "cuda")
    value = whole_job_rate(B, T, world, args.steps, ms / 1000.0)
    if args.kernels_only:
        if rank == 0:
            print(json.dumps({"kernels_only": True, "value": value, "unit": UNIT, "ms_per_step": ms / args.steps,
                              "kernel_ms_per_step": {k: v[0] for k, v in stats.items()}}), flush=True)
        batch.close()
        return 0

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
    e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    e2e_value = whole_job_rate(B, T, world, args.steps, e2e_s)
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
        # DRAM traffic per pass launch: ncu dram bytes of four consecutive
        # launches (two layers: sparse, dense, sparse, dense) at 16
        # trajectories, 3.06 GB per launch on average = 191 MB per trajectory;
        # a launch streams each state it visits once, so it scales with the
        # batch (profiles/k_pass_rounds_L24_traffic_batch16.md).
        traffic = PASS_TRAFFIC_PER_TRAJ * B
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": traffic,
                    "traffic_source": "ncu dram bytes per launch, 16-trajectory capture of two layers scaled to B",
                    "peak_source": peak_kind,
                    "kernel": "k_pass (tiled brickwork layer pass)",
                    "alg_bytes_per_launch": alg_bytes_step / pass_n, "launch_ms": pass_ms / pass_n,
                    "passes_per_layer": passes_per_layer,
                    "kernel_ms_per_step": {k: v[0] for k, v in stats.items()}}
        # Final half-chain S_2: tensor-core Gram of each trajectory's block
        # without the sites its last layer measured (the state is a product
        # on them): d_A' = 2^(12 - measured sites among 0..11), d_B' likewise
        # for 12..23. The Gram runs over the smaller side (same purity), so
        # 4 min(d_A', d_B')^2 max(d_A', d_B') real flops for the Hermitian half.
        obs_ms = stats["observables"][0]
        half = N_QUBITS // 2
        last = np.asarray(out["measured"])[:, -1].astype(np.uint64)
        lo_meas = np.array([bin(int(m) & ((1 << half) - 1)).count("1") for m in last])
        hi_meas = np.array([bin(int(m) >> half).count("1") for m in last])
        small = np.minimum(half - lo_meas, half - hi_meas)
        large = np.maximum(half - lo_meas, half - hi_meas)
        gram_flops = float(np.sum(4.0 * 2.0 ** (2 * small) * 2.0 ** large))
        full_flops = B * 4.0 * float(1 << half) ** 3
        gram = {"kernel": "k_tf32_rows + k_gram_tc_pre (tcgen05 3xTF32, TMA-fed)", "ms_per_step": obs_ms,
                "alg_tflops": gram_flops / (obs_ms / 1000.0) / 1e12 if obs_ms > 0 else None,
                "alg_flops_per_step": gram_flops, "unreduced_flops_per_step": full_flops,
                "tensor_pipe_active_pct_unreduced": GRAM_TENSOR_PIPE_PCT,
                "tensor_pipe_source": "ncu sm__pipe_tensor_cycles_active, 2-trajectory capture of the unreduced "
                                      "half-chain Gram (profiles/k_gram_tc_L24_halfcut_batch2.md)"}

        # Plain FP64 per-trajectory path on the same GPU, one trajectory:
        # device time (CUDA events around the execute, as for `value`) and
        # end to end (host sampling, upload, run, fetch).
        plain = mg.Batch(N_QUBITS, PERIODS, capacity=1, fp64=True, observables=mg.OBS_S2_HALF)
        plain.run(seeds[:1], ps[:1])
        plain.prepare(seeds[:1], ps[:1])
        torch.cuda.synchronize()
        start.record()
        plain.execute()
        stop.record()
        torch.cuda.synchronize()
        plain_dev_s = start.elapsed_time(stop) / 1000.0
        pr = plain.fetch()
        t0 = time.perf_counter()
        plain.run(seeds[:1], ps[:1])
        plain_e2e_s = time.perf_counter() - t0
        plain_value = T / plain_dev_s
        plain.close()

        # Per-layer observables: the half-chain S_2 after every layer (one
        # step, device time), with the share of the Gram.
        per_layer = None
        if args.per_layer:
            pl = mg.Batch(N_QUBITS, PERIODS, capacity=B, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1,
                          tile_qubits=args.tile)
            pl.run(seeds, ps)
            pl.prepare(seeds, ps)
            pl.set_profiling(True)
            torch.cuda.synchronize()
            start.record()
            pl.execute()
            stop.record()
            torch.cuda.synchronize()
            pl_ms = start.elapsed_time(stop)
            pl_out = pl.fetch()
            pl_stats = pl.kernel_stats()
            pl.set_profiling(False)
            t0 = time.perf_counter()
            pl.run(seeds_for(rank, B, 99), ps)
            pl_e2e = time.perf_counter() - t0
            per_layer = {"value": whole_job_rate(B, T, world, 1, pl_ms / 1000.0), "unit": UNIT,
                         "observables": "half-chain Renyi-2 entropy after every layer",
                         "ms_per_step": pl_ms, "kernel_ms_per_step": {k: v[0] for k, v in pl_stats.items()},
                         "gram_share": pl_stats["observables"][0] / pl_ms,
                         "e2e": {"value": whole_job_rate(B, T, world, 1, pl_e2e), "unit": UNIT},
                         "same_final_S2_as_headline": bool(abs(pl_out["obs"][0, -1, 1] - out["obs"][0, 0, 1]) < 1e-9)}
            pl.close()

        for th in oracle_threads:
            th.join()
        ds_vals = [abs(oracle_res[i][0] - float(out["obs"][i, 0, 1])) for i in oracle_idx if i in oracle_res]
        same = all(np.array_equal(oracle_res[i][1], out["outcomes"][i]) for i in oracle_idx if i in oracle_res)

        cpu = cpu_sample(1) if world == 1 else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(B), "roofline": roofline, "gram": gram, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clocks.summary(),
            "plain_fp64": {"value": plain_value, "unit": UNIT,
                           "path": "FP64 state, one trajectory per launch sequence, device time",
                           "e2e": {"value": T / plain_e2e_s, "unit": UNIT},
                           "speedup_batched_fp32": value / plain_value,
                           "same_final_S2_as_batched": bool(abs(pr["obs"][0, 0, 1] - out["obs"][0, 0, 1]) < 1e-5)},
            "dS": {"max_abs": max(ds_vals) if ds_vals else None, "same_outcomes": bool(same),
                   "reference": "CPU FP64 oracle, free running",
                   "observable": f"final half-chain S_2 of trajectories {oracle_idx} (p = "
                                 f"{[round(float(ps[i]), 3) for i in oracle_idx]}), 48 layers"},
        }
        if per_layer is not None:
            line["per_layer_observables"] = per_layer
        print(json.dumps(line), flush=True)
    batch.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


# ------------------------------------------------- the other workload configurations
# `--config N` measures configuration N of the workload list (0: plain FP64
# chain, 1: free fermions, 2: mixed-length batch, 3: 2-D lattice, 4: GMN,
# 5: free-energy protocol, 6: RPPU / qRPPU gate sets) and
# prints one JSON line for it; the default run (no --config) is the headline
# L = 24 metric above.
def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def _oracle_pool(fn, items, threads):
    from concurrent.futures import ThreadPoolExecutor
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(fn, items))
    return res, time.perf_counter() - t0


def config0():
    """L = 12 open chain, FP64, p = 0.2, 24 layers, 200 trajectories from seed 0;
    per-layer half-chain S_vN, S_2 and TMI (A..D = 3 qubits)."""
    import mipt_gb300 as mg
    from oracle import pyoracle as orc
    n, periods, count = 12, 12, 200
    seeds = np.array([mg.trajectory_seed(0, i) for i in range(count)], np.uint64)
    b = mg.Batch(n, periods, capacity=count, closed=False, fp64=True, observables=15, observe_every=1)
    b.run(seeds, 0.2)
    out, dt = _timed(lambda: b.run(seeds, 0.2))
    units = count * 2 * periods
    ref = orc.run_trajectory(int(seeds[0]), n, periods, 0.2, False, 16, 15, 1)
    ds = float(np.nanmax(np.abs(out["obs"][0] - ref["obs"])))
    threads = orc.max_threads()
    sample = list(seeds[:threads])
    _, cdt = _oracle_pool(lambda sd: orc.run_trajectory(int(sd), n, periods, 0.2, False, 16, 15, 1), sample, threads)
    return {"config": "0: L=12 open chain, FP64, p=0.2, 24 layers, 200 trajectories, per-layer S_vN/S_2/TMI",
            "value": units / dt, "unit": UNIT, "e2e_includes": "host sampling, upload, all layers, fetch",
            "max_abs_dS_vs_oracle": ds,
            "cpu_baseline": {"value": len(sample) * 2 * periods / cdt, "unit": UNIT, "cores": threads,
                             "kind": "port", "sample": f"{len(sample)} trajectories, same observables"}}


def config1():
    """Free-fermion covariance, N = 128, depth 256, 500 trajectories per p in
    {0.1, 0.2, 0.3}; entropies of every block [0, l) and TMI of the quarters.
    The configuration's plain method is FP64 Gamma (`value`); the FP32
    evolution (FP64 denominators, re-purification, eigensolves) is reported
    beside it."""
    import mipt_gb300 as mg
    from oracle import pyoracle as orc
    N, depth, per_p = 128, 256, 500
    ps = np.repeat([0.1, 0.2, 0.3], per_p)
    seeds = np.array([mg.trajectory_seed(1, i) for i in range(len(ps))], np.uint64)
    blocks = list(range(1, N + 1))
    ref = orc.ff_trajectory(int(seeds[0]), N, depth, float(ps[0]), True, 64, blocks=blocks, want_gamma=False)
    res = {}
    for fp64 in (True, False):
        mg.ff_run(seeds[:8], ps[:8], N, depth, blocks=blocks, fp64=fp64)
        out, dt = _timed(lambda: mg.ff_run(seeds, ps, N, depth, blocks=blocks, fp64=fp64))
        res[fp64] = {"value": len(ps) * depth / dt, "seconds": dt,
                     "max_abs_dS_vs_oracle_traj0": float(np.max(np.abs(out["s_blocks"][0] - ref["s_blocks"]))),
                     "same_outcomes_traj0": bool(np.array_equal(out["outcomes"][0], ref["outcomes"]))}
    threads = orc.max_threads()
    sample = list(range(threads))
    _, cdt = _oracle_pool(lambda i: orc.ff_trajectory(int(seeds[i]), N, depth, float(ps[i]), True, 64,
                                                       blocks=blocks, want_gamma=False), sample, threads)
    return {"config": "1: free fermions N=128 (256 Majoranas), depth 256, 1500 trajectories, all prefix blocks + TMI",
            "value": res[True]["value"], "unit": UNIT, "dtype": "f64", "fp64": res[True], "fp32": res[False],
            "cpu_baseline": {"value": len(sample) * depth / cdt, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{len(sample)} trajectories, FP64 oracle"}}


def config2():
    """4096 trajectories, L uniform on {16, 18, 20, 22}, p from 16 values in
    [0.05, 0.35], periodic, depth 2L, FP32; per-layer half-chain S_2 and (L a
    multiple of 4) TMI of the quarters from S_2. The four lengths run as the
    branches of one CUDA graph (one launch per step). The configuration's
    per-layer half-chain S_vN (FP64 eigensolves of 256..2048-row spectra) is
    timed on a bounded sample beside it."""
    import mipt_gb300 as mg
    rng = np.random.default_rng(2)
    total = 4096
    Ls = rng.choice([16, 18, 20, 22], size=total)
    ps = P_GRID[rng.integers(0, 16, size=total)]
    seeds = np.array([mg.trajectory_seed(2, i) for i in range(total)], np.uint64)
    groups = []
    for L in (16, 18, 20, 22):
        idx = np.nonzero(Ls == L)[0]
        obs = mg.OBS_S2_HALF | (mg.OBS_TMI_S2 if L % 4 == 0 else 0)
        groups.append((L, idx, mg.Batch(L, L, capacity=len(idx), fp64=False, observables=obs, observe_every=1)))
    graph = mg.BatchGroup([b for _, _, b in groups])

    def step():
        for L, idx, b in groups:
            b.prepare(seeds[idx], ps[idx])
        graph.execute()
        return [b.fetch() for _, _, b in groups]

    step()  # normal execute + capture
    step()
    _, dt = _timed(step)
    units = int(sum(2 * L * len(idx) for L, idx, b in groups))
    graph.close()
    for _, _, b in groups:
        b.close()
    # Per-layer half-chain S_vN on a sample: the first 16 trajectories of the
    # two shorter lengths, one graph, FP64 eigensolves (256 and 512 rows; one
    # CTA per spectrum, so the 1024- and 2048-row spectra of L = 20 and 22 take
    # about 1 s and 8 s per layer at any batch size and are left out).
    svn_groups = []
    for L in (16, 18):
        idx = np.nonzero(Ls == L)[0][:16]
        svn_groups.append((L, idx, mg.Batch(L, L, capacity=len(idx), fp64=False, observables=mg.OBS_SVN_HALF,
                                            observe_every=1)))
    sg = mg.BatchGroup([b for _, _, b in svn_groups])

    def svn_step():
        for L, idx, b in svn_groups:
            b.prepare(seeds[idx], ps[idx])
        sg.execute()
        return [b.fetch() for _, _, b in svn_groups]

    svn_step()
    _, svn_dt = _timed(svn_step)
    svn_units = int(sum(2 * L * len(idx) for L, idx, b in svn_groups))
    sg.close()
    for _, _, b in svn_groups:
        b.close()
    # plain FP64 per-trajectory arm on a sample
    plain_units, plain_t = 0, 0.0
    for L in (16, 22):
        pb = mg.Batch(L, L, capacity=1, fp64=True, observables=mg.OBS_S2_HALF | (mg.OBS_TMI_S2 if L % 4 == 0 else 0),
                      observe_every=1)
        i = int(np.nonzero(Ls == L)[0][0])
        pb.run(seeds[i:i + 1], ps[i:i + 1])
        _, t = _timed(lambda: pb.run(seeds[i:i + 1], ps[i:i + 1]))
        plain_units += 2 * L
        plain_t += t
        pb.close()
    return {"config": "2: 4096 trajectories, L uniform on {16,18,20,22}, depth 2L, FP32, per-layer S_2 (+TMI_S2 for L%4==0)",
            "value": units / dt, "unit": UNIT, "trajectory_layers": units, "execution": "one CUDA graph, 4 branches",
            "per_layer_svn_sample": {"value": svn_units / svn_dt, "unit": UNIT, "trajectory_layers": svn_units,
                                     "sample": "16 trajectories each of L = 16 and 18, half-chain S_vN after every "
                                               "layer (FP64 eigensolver, 256 and 512 rows)"},
            "plain_fp64_per_trajectory": {"value": plain_units / plain_t, "unit": UNIT,
                                          "sample": "one L=16 and one L=22 trajectory"},
            "speedup_vs_plain_fp64": (units / dt) / (plain_units / plain_t)}


def config3():
    """4 x 7 lattice (L = 28, FP32, 2 GiB), p = 0.15, depth 56; per layer
    half-system S_2 (16384 x 16384 Gram on the tensor cores), S_vN of the first
    two rows (8 qubits) and three rho3 blocks."""
    import mipt_gb300 as mg
    X, Y, periods = 4, 7, 28
    # Warm-up on a 4 x 3 lattice with the same observable kinds: loads the
    # eigensolver and kernel modules outside the timed run.
    w = mg.Batch(12, 1, capacity=1, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1, rho3=True, lattice=(4, 3))
    w.add_region(list(range(8)), 1)
    w.set_rho3_subsystems([[0, 1, 2]])
    w.run(np.array([mg.trajectory_seed(3, 1)], np.uint64), 0.15)
    w.close()
    b = mg.Batch(X * Y, periods, capacity=1, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1, rho3=True,
                 lattice=(X, Y))
    b.add_region(list(range(8)), 1)
    b.set_rho3_subsystems([[0, 1, 2], [0, 4, 8], [5, 6, 9]])
    seed = np.array([mg.trajectory_seed(3, 0)], np.uint64)
    b.set_profiling(True)
    out, dt = _timed(lambda: b.run(seed, 0.15))
    stats = b.kernel_stats()
    return {"config": "3: 4x7 lattice L=28 FP32, p=0.15, depth 56, per-layer S_2(half)+S_vN(8 qubits)+3 rho3",
            "value": 2 * periods / dt, "unit": UNIT, "seconds_per_trajectory": dt,
            "kernel_ms": {k: v[0] for k, v in stats.items()}, "final_half_S2": float(out["obs"][0, -1, 1])}


def config4():
    """65,536 rho3 blocks: half from L = 16 trajectories (final ring triples,
    p in [0.05, 0.35]), half GHZ/W/product mixtures with white noise; batched
    GMN to a certified gap of 1e-6 (FP32 ADMM, FP64 certificates), cold and
    with the learned warm start."""
    import mipt_gb300 as mg
    from mipt_gb300 import gmn_warm
    from oracle import gmn as ogmn
    b = mg.Batch(16, 16, capacity=2048, fp64=False, rho3=True)
    rng = np.random.default_rng(4)
    seeds = np.array([mg.trajectory_seed(4, i) for i in range(2048)], np.uint64)
    r = b.run(seeds, rng.uniform(0.05, 0.35, size=2048))
    traj = (r["rho3"].reshape(-1, 128)[:, 0::2] + 1j * r["rho3"].reshape(-1, 128)[:, 1::2]).reshape(-1, 8, 8)
    rho = np.concatenate([traj, gmn_warm.mixtures(len(traj), 5)])
    cold, dt = _timed(lambda: mg.gmn_solve(rho, gap_tol=1e-6, max_iter=3000, check_every=10))
    ok = cold["iters"] > 0
    # The learned warm starts, at the penalty they are trained for, against a
    # cold start at that same penalty: training pairs from other trajectories
    # (65,536 rho3 blocks of 4,096 L = 16 trajectories) and 24,000 mixtures,
    # solved by the cold-start solver; the network's prediction and the
    # nearest solved training state, reported per class of the workload.
    ws = gmn_warm.WARM_SIGMA
    train = np.concatenate([gmn_warm.trajectory_states(4096, 41), gmn_warm.mixtures(24000, 6)])
    x, t, _ = gmn_warm.solve_pairs(train, gap_tol=1e-6, max_iter=3000, sigma=ws)
    model = gmn_warm.WarmStartModel(seed=0)
    (_, tdt) = _timed(lambda: model.fit(x, t))
    nearest = gmn_warm.NearestSolved(x, t)
    cold_ws, cwdt = _timed(lambda: mg.gmn_solve(rho, gap_tol=1e-6, max_iter=3000, check_every=10, sigma=ws))
    classes = {"trajectory": slice(0, len(traj)), "mixture": slice(len(traj), len(rho))}
    per_class = {}
    for name, guesser in (("network", model), ("nearest_solved", nearest)):
        guess = guesser.predict(rho)
        w, wt = _timed(lambda: mg.gmn_solve(rho, warm_start=guess, gap_tol=1e-6, max_iter=3000, check_every=10,
                                            sigma=ws))
        entry = {"value": len(rho) / wt}
        for cls, sl in classes.items():
            b2 = (cold_ws["iters"][sl] > 0) & (w["iters"][sl] > 0)
            entry[cls] = {"iterations_cold_warm": [float(cold_ws["iters"][sl][b2].mean()),
                                                   float(w["iters"][sl][b2].mean())],
                          "gain": float(cold_ws["iters"][sl][b2].mean() / w["iters"][sl][b2].mean()),
                          "certified_cold_warm": [float((cold_ws["iters"][sl] > 0).mean()),
                                                  float((w["iters"][sl] > 0).mean())],
                          "max_abs_dGMN": float(np.max(np.abs(w["gmn"][sl][b2] - cold_ws["gmn"][sl][b2])))}
        per_class[name] = entry
    warm, wdt = w, wt
    both = (cold_ws["iters"] > 0) & (warm["iters"] > 0)
    sample = list(range(0, len(rho), len(rho) // 16))
    _, cdt = _oracle_pool(lambda i: ogmn.solve(rho[i], gap_tol=1e-6, max_iter=3000), sample, 16)
    return {"config": "4: 65536 rho3 (half L=16 trajectories, half GHZ/W/product mixtures), GMN to gap 1e-6",
            "value": len(rho) / dt, "unit": "SDPs/s (cold start, incl. uncertified at 3000 iterations)",
            "certified_fraction": float(ok.mean()),
            "certified_fraction_trajectory_states": float(ok[:len(traj)].mean()),
            "certified_fraction_mixtures": float(ok[len(traj):].mean()),
            "mean_iterations_certified": float(cold["iters"][ok].mean()),
            "warm_start": {"sigma": ws, "cold_value_same_sigma": len(rho) / cwdt,
                           "cold_certified_fraction_same_sigma": float((cold_ws["iters"] > 0).mean()),
                           "per_method": per_class,
                           "nearest_solved_iterations_on_states_both_certify": [float(cold_ws["iters"][both].mean()),
                                                                                float(warm["iters"][both].mean())],
                           "train_pairs": int(len(x)), "train_seconds": tdt},
            "cpu_baseline": {"value": len(sample) / cdt, "unit": "SDPs/s", "cores": 16, "kind": "port",
                             "sample": f"{len(sample)} states, FP64 ADMM oracle (the reference uses MOSEK, absent)"}}


def config5():
    """The free-energy protocol (free_energy.exe's loop): N = 16 periodic Haar
    brickwork, p = 0.1, random Haar initial states, 28N = 448 timesteps per
    trajectory, half-chain S_vN at t = 0..2N; 512 trajectories in one batch,
    FP32 states. Timed end to end through the batch calls the executable makes
    (initial-state draw and upload, layer draw, all layers, fetch)."""
    import mipt_gb300 as mg
    from oracle import pyoracle as orc
    n, p, count = 16, 0.1, 512
    T = 28 * n
    steps = list(range(2 * n + 1))
    b = mg.Batch(n, T // 2, count, closed=True, fp64=False, observables=mg.OBS_SVN_HALF)
    b.set_observation_steps(steps)
    ts = [orc.fe_trajectory_seed(5, i) for i in range(count)]
    init = [orc.fe_initial_seed(t) for t in ts]
    ws = [orc.fe_workspace_seed(t) for t in ts]

    def step():
        b.set_initial_states(init, 1)
        b.prepare_workspace(ws, p)
        b.execute()
        return b.fetch()

    step()
    b.set_profiling(True)
    out, dt = _timed(step)
    stats = b.kernel_stats()
    want = orc.fe_trajectory(ts[0], n, p, 1, fp32_init=True, entropy_max_t=2 * n)
    threads = orc.max_threads()
    _, cdt = _timed(lambda: orc.fe_batch(5, 0, threads, n, p, 1, threads=threads))
    return {"config": "5: free-energy protocol N=16 periodic Haar, p=0.1, Haar initial states, 448 timesteps, "
                      "S_vN(half) at t=0..32, 512 trajectories, FP32",
            "value": count * T / dt, "unit": UNIT, "trajectories_per_s": count / dt,
            "kernel_ms": {k: v[0] for k, v in stats.items()},
            "max_abs_dF_vs_oracle_traj0": float(abs(out["surprisal"][0].sum() - want["surprisal"].sum())),
            "max_abs_dS_vs_oracle_traj0": float(np.max(np.abs(out["obs"][0, :, 0] - want["s_half"][steps]))),
            "cpu_baseline": {"value": threads * T / cdt, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{threads} trajectories, FP64 oracle, one per host thread, "
                                       "no entropies (the GPU arm includes them)"}}


def config6():
    """The headline's shape on the parity-preserving gate sets: L = 24 closed
    ring, 32 trajectories, 24 periods (48 layers plus the reference's random
    extra even layer), p cycled over 16 values, final half-chain S_2, FP32;
    FermionRPPU (fermionic closure folded into the closure gate, fermionic
    partial trace) and qRPPU."""
    import mipt_gb300 as mg
    from oracle import pyoracle as orc
    n, periods, count = 24, 24, 32
    seeds = np.array([mg.trajectory_seed(6, i) for i in range(count)], np.uint64)
    ps = P_GRID[np.arange(count) % 16]
    out = {"config": "6: RPPU/qRPPU L=24 closed ring, 32 trajectories x (48 + extra) layers, final S_2(half), FP32",
           "unit": UNIT}
    for circuit, name in ((2, "fermion_rppu"), (4, "qrppu")):
        b = mg.Batch(n, periods, count, fp64=False, observables=mg.OBS_S2_HALF, fermion_trace=circuit == 2,
                     circuit=circuit)
        b.run(seeds, ps)
        b.set_profiling(True)
        r, dt = _timed(lambda: b.run(seeds, ps))
        layers = count * 2 * periods  # the extra even layers are not counted
        stats = b.kernel_stats()
        out[name] = {"value": layers / dt, "trajectory_layers": layers, "seconds": dt,
                     "kernel_ms": {k: v[0] for k, v in stats.items()}}
        b.close()
    threads = orc.max_threads()
    sample = [int(s) for s in seeds[:threads]]
    _, cdt = _oracle_pool(lambda sd: orc.run_rppu_trajectory(sd, n, 1, 0.2, orc.RPPU_JW), sample, threads)
    out["value"] = out["fermion_rppu"]["value"]
    out["cpu_baseline"] = {"value": len(sample) * 2 / cdt, "unit": UNIT, "cores": threads, "kind": "port",
                           "sample": f"{len(sample)} FermionRPPU trajectories of 2 layers (+ extra), FP64 oracle, "
                                     "one per host thread, no final entropy"}
    return out


def run_config(k):
    import torch
    torch.cuda.set_device(0)
    fn = [config0, config1, config2, config3, config4, config5, config6][k]
    line = fn()
    line["data"] = "synthetic"
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tile", type=int, default=0, help="local qubits per pass tile (0 = library default)")
    ap.add_argument("--config", type=int, default=-1, help="measure workload configuration 0..6 instead")
    ap.add_argument("--per-layer", dest="per_layer", type=int, default=1,
                    help="also time the workload with the half-chain S_2 after every layer (1 = on)")
    ap.add_argument("--kernels-only", dest="kernels_only", action="store_true",
                    help="time the batched device run only (for profiler captures)")
    args = ap.parse_args()
    if args.config >= 0:
        return run_config(args.config)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
