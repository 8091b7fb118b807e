#!/usr/bin/env python
"""Benchmark of the Hydrangea fused-loop hot path on GB300.

Default workload (one step): the fused weighted histogram
    scatter (+) (fill [B] 0) (map (x % B) data) (map (x * x) data)
over data = 2^27 int64 uniform in [0, 2^20) (seed 2, 1 GiB, device-resident),
for both B = 64 and B = 65536 (two launches per step).  The metric is the
fused kernels' HBM throughput in GB/s of algorithmic bytes (8 B read per
element per launch, plus the B*8 B histogram write).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the C-backend restatement (the oracle port, OpenMP on
all host cores) on the same configuration; under torchrun only rank 0 runs it.
Other workloads of the suite run with --workload dot|heat|batched|serve.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_ELEMS = 1 << 27
BINS = (64, 65536)
SEED = 2
VALUE_BOUND = 1 << 20
METRIC = "fused-kernel HBM GB/s (% of peak); served req/s + p50/p99 vs plain per-call"
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="histogram", choices=["histogram"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback (6.8 TB/s, earlier GB300 copy measurement)"


def profile_traffic(kernel_key):
    """Per-launch DRAM bytes of `kernel_key` recorded from an ncu capture in
    profiles/traffic.txt (lines `kernel_key bytes_per_launch`), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel_key and not line.startswith("#"):
                try:
                    return float(parts[1])
                except ValueError:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        rows = [r.split(",") for r in self.tmp.read().strip().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------------
def run_gpu(args):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__ as g
    hc = g.package()
    hc.lib()
    hc.check(hc.lib().hyd_cuda_init())
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    data = torch.empty(N_ELEMS, dtype=torch.int64, device=dev)
    hc.fill_uniform_i64(data, SEED, VALUE_BOUND)
    hists = {b: torch.zeros(b, dtype=torch.int64, device=dev) for b in BINS}
    L = hc.lib()
    dptr = data.data_ptr()

    def launch(b):
        st = L.hyd_cuda_weighted_histogram_i64(dptr, N_ELEMS, b, hists[b].data_ptr(), 0, sh)
        if st:
            hc.check(st)

    # per-kernel CUDA-event timing (on the launching stream); the destination's
    # `fill [B] 0` is a memset outside the per-kernel window
    def step(evs=None):
        for i, b in enumerate(BINS):
            hists[b].zero_()
            if evs is not None:
                evs[i][0].record(stream)
            launch(b)
            if evs is not None:
                evs[i][1].record(stream)

    sampler = ClockSampler(local)
    sampler.start()
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    hc.check(hc.device_check())

    per_kernel = {b: [] for b in BINS}
    ev_pairs = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
                 for _ in BINS] for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(args.steps):
        step(ev_pairs[k])
    t1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    elapsed_ms = t0.elapsed_time(t1)
    for k in range(args.steps):
        for i, b in enumerate(BINS):
            per_kernel[b].append(ev_pairs[k][i][0].elapsed_time(ev_pairs[k][i][1]))
    if dist:
        t = torch.tensor([elapsed_ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())

    # correctness guard on the measured buffers (bins sum = sum of squares)
    host = data.cpu().numpy()
    import numpy as np
    sq = int((host.astype(np.uint64) * host.astype(np.uint64)).sum(dtype=np.uint64))
    for b in BINS:
        assert int(hists[b].cpu().numpy().astype(np.uint64).sum(dtype=np.uint64)) == sq, b

    bytes_per_launch = {b: 8 * N_ELEMS + 8 * b for b in BINS}
    bytes_per_step = sum(bytes_per_launch.values())
    value = world * bytes_per_step * args.steps / (elapsed_ms / 1e3) / 1e9
    peak, peak_src = measured_peak()
    avg = {b: statistics.mean(per_kernel[b]) for b in BINS}
    dom = max(BINS, key=lambda b: avg[b])
    achieved = bytes_per_launch[dom] / (avg[dom] / 1e3) / 1e9
    traffic = profile_traffic("weighted_histogram_i64_B%d" % dom)

    # e2e through the C-ABI host-pointer entry point: H2D of the step's input from
    # pinned host memory and D2H of the histogram inside the timed region.
    pinned = torch.empty(N_ELEMS, dtype=torch.int64, pin_memory=True)
    pinned.copy_(data)
    out_host = {b: torch.zeros(b, dtype=torch.int64, pin_memory=True) for b in BINS}
    e2e_steps = max(3, min(args.steps, 20))

    def e2e_step():
        for b in BINS:
            hc.check(L.hyd_cuda_weighted_histogram_host(pinned.data_ptr(), N_ELEMS, b,
                                                        out_host[b].data_ptr(), 0))
    for _ in range(2):
        e2e_step()
    if dist:
        dist.barrier()
    te = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = time.perf_counter() - te
    if dist:
        t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    for b in BINS:
        assert torch.equal(out_host[b], hists[b].cpu()), "e2e result differs"
    e2e_value = world * bytes_per_step * e2e_steps / e2e_s / 1e9

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(host)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": round(value, 2),
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": elapsed_ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "int64",
            "data": "synthetic (seeded SplitMix64, uniform int64 in [0, 2^20); no dataset)",
            "config": {
                "workload": "weighted_histogram scatter(+) x%B / x*x, N=2^27 int64, B in {64, 65536} "
                            "(both per step)",
                "n": N_ELEMS, "bins": list(BINS), "seed": SEED,
                "l2": "inputs larger than L2 (1 GiB > 129 MB); no flush needed",
                "parallelism": "replicas" if world > 1 else "single GPU",
                "strategy": "AUTO (SMEM_WARP for B=64, CLUSTER DSMEM for B=65536)",
            },
            "pct_of_peak": round(100.0 * value / world / peak, 1),
            "per_kernel_ms": {"B=%d" % b: round(avg[b], 4) for b in BINS},
            "per_kernel_gbs": {"B=%d" % b: round(bytes_per_launch[b] / (avg[b] / 1e3) / 1e9, 1) for b in BINS},
            "roofline": {
                "bound": "hbm",
                "kernel": "hist_*_kernel<WeightedHistSource> B=%d" % dom,
                "achieved": round(achieved, 1),
                "peak": peak,
                "peak_source": peak_src + "; burst figure (kernel timed alone)",
                "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": traffic,
                "algorithmic_bytes_per_launch": bytes_per_launch[dom],
            },
            "e2e": {
                "value": round(e2e_value, 2), "unit": "GB/s",
                "h2d_bytes_per_step": 8 * N_ELEMS * len(BINS),
                "d2h_bytes_per_step": 8 * sum(BINS),
                "call": "hyd_cuda_weighted_histogram_host (pinned host input, 64 MiB chunks, 2 streams)",
                "steps": e2e_steps,
            },
            "gpu_launches": len(BINS) * args.steps,
            "clocks": clocks,
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def cpu_baseline(host_data, budget_s=20.0):
    """The oracle (C-backend restatement, OpenMP on all host cores) on the same
    data: full N, both bin counts per step, as many steps as fit the budget."""
    from oracle import oracle as O
    import numpy as np
    cores = O.lib().orc_max_threads()
    host_data = np.ascontiguousarray(host_data)
    t = time.perf_counter()
    for b in BINS:
        O.weighted_hist(host_data, b)  # warm-up
    one = time.perf_counter() - t
    reps = max(1, min(10, int(budget_s / max(one, 1e-3))))
    t = time.perf_counter()
    for _ in range(reps):
        for b in BINS:
            O.weighted_hist(host_data, b)
    dt = time.perf_counter() - t
    bytes_per_step = sum(8 * len(host_data) + 8 * b for b in BINS)
    return {"value": round(bytes_per_step * reps / dt / 1e9, 3), "unit": "GB/s", "cores": cores,
            "kind": "port",
            "sample": "full workload: N=2^27, B=64 and B=65536, %d steps, privatized OpenMP template" % reps}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    cores = O.lib().orc_max_threads()
    data = O.uniform_i64(N_ELEMS, SEED, VALUE_BOUND)
    # size each step's sample so the whole run stays within ~2 minutes
    t = time.perf_counter()
    for b in BINS:
        O.weighted_hist(data, b)
    one = time.perf_counter() - t
    total = args.steps + args.warmup
    frac = min(1.0, 100.0 / max(total * one, 1e-9))
    n = max(1 << 16, int(N_ELEMS * frac) // 4 * 4)
    sample = np.ascontiguousarray(data[:n])
    for _ in range(args.warmup):
        for b in BINS:
            O.weighted_hist(sample, b)
    t = time.perf_counter()
    for _ in range(args.steps):
        for b in BINS:
            O.weighted_hist(sample, b)
    dt = time.perf_counter() - t
    bytes_per_step = sum(8 * n + 8 * b for b in BINS)
    value = bytes_per_step * args.steps / dt / 1e9
    desc = "oracle port of the privatized OpenMP scatter template on %d host threads; " \
           "each step = B=64 and B=65536 over the first %d of the 2^27 elements" % (cores, n)
    print(json.dumps({
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
        "data": "synthetic (seeded SplitMix64, uniform int64 in [0, 2^20))",
        "config": {"workload": "weighted_histogram scatter(+) x%B / x*x, N=2^27 int64, B in {64, 65536} "
                               "(both per step)", "n": N_ELEMS, "bins": list(BINS), "seed": SEED},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": desc},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
