"""Multisplit benchmark on GB300.

Default workload (one step = one stable key-value multisplit):
    2^28 (uint32 key, uint32 value) pairs, values = original index, keys uniform
    over [0, 2^32) (splitmix64, seed 3), 256 buckets by delta bucketing
    (bucket = key * 256 >> 32).
Inputs (2 GiB) and outputs (2 GiB) are far larger than the 129 MB L2, so no
flush is needed between steps.

`value` is whole-job Gkeys/s (one key-value pair = one key) with inputs resident
in HBM; the step runs prescan, scan and postscan through the C ABI's stage
entry points with CUDA events between them, which also yields the postscan's
own duration for the roofline.  `e2e` is the same metric through the one-call
public API with pinned host buffers: host->device copy of keys and values, the
multisplit, and device->host copy of both outputs inside every timed step.

--impl reference times the CPU implementation of the same path (the oracle's
multi-threaded restatement of the reference's cpu_multisplit_pairs_general,
oracle/oracle.c) on the host cores.

Multi-GPU (torchrun): every rank runs its own replica of the workload (weak
scaling, no collective on the data path); timing is the max over ranks.
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

METRIC = "Gkeys/s & %HBM roofline at 2^28 keys; batched-vs-plain Gkeys/s, p50/p99 lat"
UNIT = "Gkeys/s"
CLOCK_SOAK_S = 1.5


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--log2n", type=int, default=28)
    p.add_argument("--buckets", type=int, default=256)
    p.add_argument("--dist", default="uniform", choices=["uniform", "zipf"])
    p.add_argument("--identifier", default="delta", choices=["delta", "range"])
    p.add_argument("--keys-only", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline time budget")
    p.add_argument("--no-batched", action="store_true", help="skip the batched-form measurement")
    p.add_argument("--only-batched", action="store_true", help="print only the batched-form summary")
    p.add_argument("--only-tiny-segments", action="store_true",
                   help="print only the many-small-segments summary (one warp per segment against tiles)")
    p.add_argument("--autotune", action="store_true",
                   help="batched form: autotune the tile table first instead of keeping the built-in one")
    p.add_argument("--no-serving", action="store_true", help="skip the serving-form measurement")
    p.add_argument("--only-serving", action="store_true", help="print only the serving-form summary")
    p.add_argument("--serve-seconds", type=float, default=10.0)
    p.add_argument("--serve-rate", type=float, default=20000.0)
    p.add_argument("--sweep-part", default="all", choices=["all", "base", "wide", "big"],
                   help="with --sweep: all cases, or only the 32-bit cases (base), the 64-bit key / value cases "
                        "(wide) or the cases with more than 256 buckets (big)")
    p.add_argument("--no-sweep", action="store_true",
                   help="leave the 32-bit sweep (one entry per 2^28 case) out of the headline line")
    p.add_argument("--sweep", action="store_true",
                   help="time every 2^28 case of the key-value sweep, key-only, compaction, histogram and sort "
                        "(one JSON line per case) instead of the headline line")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_config(a):
    n = 1 << a.log2n
    return {
        "workload": f"{'key-only' if a.keys_only else 'key-value'} stable multisplit, 2^{a.log2n} "
                    f"{'keys' if a.keys_only else 'pairs (values = index)'}, {a.buckets} buckets, "
                    f"{a.identifier} identifier, {a.dist} uint32 keys",
        "n": n,
        "buckets": a.buckets,
        "identifier": "delta (key*B>>32)" if a.identifier == "delta" else "range (B sorted splitters, s[0]=0)",
        "distribution": a.dist if a.dist == "uniform" else "zipf s=1.1 over 2^20 distinct keys",
        "key_value": not a.keys_only,
        "l2": "inputs larger than L2 (no flush needed)",
    }


def algorithmic_bytes(a):
    # prescan reads keys (4 B); postscan reads keys (+values) and writes them.
    per_key_step = 12 if a.keys_only else 20
    per_key_post = 8 if a.keys_only else 16
    return per_key_step, per_key_post


def make_inputs(a, device):
    from gpumultisplit_gb300 import datagen

    n = 1 << a.log2n
    keys = (datagen.uniform_u32 if a.dist == "uniform" else datagen.zipf_u32)(n, 3, device=device)
    vals = None if a.keys_only else datagen.index_values(n, device)
    spl = datagen.range_splitters(a.buckets, 5, device) if a.identifier == "range" else None
    return keys, vals, spl


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="gms_clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        pw = [num(r[3]) for r in rows if num(r[3]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "samples": len(rows), "reasons": reasons}


def bind_to_gpu_cpus(local: int) -> dict:
    """Pins this process to the CPUs of the GPU's own NUMA node (the PCI
    device's local_cpulist), so the pinned host buffers of the end-to-end steps
    are allocated in the memory nearest the GPU rather than wherever the
    process happened to start.  Returns what it did, for the JSON line."""
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(local), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30).stdout.strip()
        dom, rest = bus.split(":", 1)
        dev = f"/sys/bus/pci/devices/{dom[-4:].lower()}:{rest.lower()}"
        with open(os.path.join(dev, "local_cpulist")) as f:
            spec = f.read().strip()
        cpus = set()
        for part in spec.split(","):
            a, _, b = part.partition("-")
            cpus.update(range(int(a), int(b or a) + 1))
        cpus &= os.sched_getaffinity(0)
        if not cpus:
            return {"cpus": None, "note": f"no usable CPU in {spec}"}
        os.sched_setaffinity(0, cpus)
        node = None
        try:
            with open(os.path.join(dev, "numa_node")) as f:
                node = int(f.read().strip())
        except (OSError, ValueError):
            pass
        return {"cpus": spec, "numa_node": node, "cpus_used": len(cpus)}
    except (OSError, ValueError, subprocess.SubprocessError) as e:
        return {"cpus": None, "note": f"not bound: {e}"}


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel: str, n: int):
    """Per-launch DRAM bytes of `kernel` from a committed ncu capture summary,
    scaled to n keys (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            rec = json.load(f)[kernel]
        return rec["dram_bytes_per_key"] * n
    except (OSError, KeyError, ValueError):
        return None


def run_batched(dev, reps: int = 3, tune: bool = True):
    """Batched form (4096 segments, log-uniform sizes in [1024, 4194304], seed 7,
    B in {2, 8, 32, 256}, delta or range identifier, key-value) against the plain
    per-call loop over the same segments; returns a summary dict."""
    import torch

    import gpumultisplit_gb300 as gms
    from gpumultisplit_gb300 import datagen

    sizes, buckets, kinds = datagen.batched_spec()
    # segment starts padded to 32 elements so every segment is 16-byte aligned
    starts = np.concatenate([[0], np.cumsum((sizes + 31) // 32 * 32)[:-1]]).astype(np.int64)
    total_alloc = int(starts[-1] + (sizes[-1] + 31) // 32 * 32)
    total = int(sizes.sum())
    keys = datagen.uniform_u32(total_alloc, 11, device=dev)
    vals = datagen.index_values(total_alloc, dev)
    kout, vout = torch.zeros_like(keys), torch.zeros_like(vals)
    kref, vref = torch.zeros_like(keys), torch.zeros_like(vals)
    segs, plain = [], []
    for i, (n, B, kind) in enumerate(zip(sizes.tolist(), buckets.tolist(), kinds)):
        o = int(starts[i])
        ident = gms.delta_bucket() if kind == "delta" else gms.range_bucket(datagen.range_splitters(B, 1000 + i, dev))
        segs.append(gms.Segment(keys[o:o + n], kout[o:o + n], n, B, ident, vals[o:o + n], vout[o:o + n]))
        plain.append((keys[o:o + n], vals[o:o + n], kref[o:o + n], vref[o:o + n], n, B, ident))
    ctxs = {}
    for B in sorted(set(buckets.tolist())):
        ctx = gms.multisplit_context(B)
        gms.multisplit_allocate_key_value(int(sizes[buckets == B].max()), ctx)
        ctxs[B] = ctx

    def plain_loop():
        for ki, vi, ko, vo, n, B, ident in plain:
            gms.multisplit_key_value(ki, vi, ko, vo, n, ctxs[B], ident)

    # Tile shapes per (B, size class) for this device, then the plan from the tuned table.
    t0 = time.perf_counter()
    if tune:
        gms.autotune(buckets=(2, 8, 32, 256), key_value=(True,), keys_per_trial=1 << 25, reps=5)
    autotune_s = time.perf_counter() - t0 if tune else None
    table = gms.tuning_table()
    chosen = {f"B{B}": [gms.tile_variant_shape(table[(B, True, c)])[2] for c in range(8)] for B in (2, 8, 32, 256)}
    plan = gms.BatchedMultisplit(segs)
    plan_fixed = gms.BatchedMultisplit(segs, variant=0)

    def timed(fn, count):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record()
        for _ in range(count):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / count, (time.perf_counter() - t0) * 1e3 / count

    plain_loop()
    plan.run(use_graph=True)
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    plain_ms, plain_wall = timed(plain_loop, reps)
    # The same plain per-call loop captured into one CUDA graph: the plain
    # path's device rate, with no host dispatch between the calls (every call
    # is its three launches, one after the other on one stream).
    plain_graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(plain_graph):
        plain_loop()
    plain_graph.replay()
    torch.cuda.synchronize()
    plain_graph_ms, _ = timed(plain_graph.replay, max(reps, 5))
    kref.zero_()
    vref.zero_()
    plain_graph.replay()
    torch.cuda.synchronize()
    graph_ms, _ = timed(lambda: plan.run(use_graph=True), max(reps, 5))
    nograph_ms, _ = timed(lambda: plan.run(use_graph=False), max(reps, 5))
    identical = bool(torch.equal(kout, kref) and torch.equal(vout, vref))
    plan_fixed.run(use_graph=True)
    fixed_ms, _ = timed(lambda: plan_fixed.run(use_graph=True), max(reps, 5))
    identical = identical and bool(torch.equal(kout, kref) and torch.equal(vout, vref))
    plan_fixed.close()
    # The same segments as one persistent launch over a device-side work list.
    kout.zero_()
    vout.zero_()
    plan_queue = gms.BatchedMultisplit(segs, schedule="queue")
    plan_queue.run(use_graph=True)
    torch.cuda.synchronize()
    queue_identical = bool(torch.equal(kout, kref) and torch.equal(vout, vref))
    queue_ms, _ = timed(lambda: plan_queue.run(use_graph=True), max(reps, 5))
    queue_identical = queue_identical and bool(torch.equal(kout, kref) and torch.equal(vout, vref))
    queue_error = plan_queue.device_error()
    queue_launches = plan_queue.launches
    plan_queue.close()
    peak, _ = hbm_peak()
    res = {
        "workload": f"{len(sizes)} key-value segments, sizes log-uniform in [1024, 4194304] (seed 7), "
                    f"B in {{2,8,32,256}}, delta or range identifier; {total} pairs",
        "pairs": total,
        "batched_graph_ms": graph_ms,
        "batched_graph_gkeys": total / (graph_ms * 1e-3) / 1e9,
        "batched_nograph_ms": nograph_ms,
        "batched_one_tile_shape_ms": fixed_ms,
        "autotune_s": autotune_s,
        "tuned_tile_keys_by_size_class": chosen,
        "plain_per_call_ms": plain_ms,
        "plain_per_call_gkeys": total / (plain_ms * 1e-3) / 1e9,
        "plain_host_wall_ms": plain_wall,
        "plain_graph_ms": plain_graph_ms,
        "plain_graph_gkeys": total / (plain_graph_ms * 1e-3) / 1e9,
        "speedup_vs_plain": plain_ms / graph_ms,
        "speedup_vs_plain_graph": plain_graph_ms / graph_ms,
        "batched_hbm_frac": 20.0 * total / (graph_ms * 1e-3) / 1e9 / peak,
        "launches_per_run": plan.launches,
        "plain_launches_per_run": 3 * len(sizes),
        "identical_to_plain": identical,
        "device_error": plan.device_error(),
        "queue": {
            "schedule": "one persistent launch over a device-side work list (gms_batch_set_schedule QUEUE)",
            "ms": queue_ms,
            "gkeys": total / (queue_ms * 1e-3) / 1e9,
            "hbm_frac": 20.0 * total / (queue_ms * 1e-3) / 1e9 / peak,
            "vs_classes_graph": graph_ms / queue_ms,
            "speedup_vs_plain_graph": plain_graph_ms / queue_ms,
            "launches_per_run": queue_launches,
            "identical_to_plain": queue_identical,
            "device_error": queue_error,
        },
    }
    plan.close()
    del plain_graph
    del keys, vals, kout, vout, kref, vref, segs, plain
    torch.cuda.empty_cache()
    return res


def run_tuning_check(dev, reps: int = 10):
    """Whether the tuning table matters: 4096 key-value segments with
    log-uniform sizes in [1024, 65536] (seed 8), B in {2, 8, 32, 256}, delta or
    range, run as one graph with (a) the built-in table (the plain path's
    4096-key tile for every class), (b) tiles that just hold segments of up to
    2048 keys (1024- and 2048-key tiles for the two smallest size classes),
    (c) the table the autotuner measured on this device.  Outputs are compared
    across the three."""
    import torch

    import gpumultisplit_gb300 as gms
    from gpumultisplit_gb300 import datagen

    sizes, buckets, kinds = datagen.batched_spec(seed=8, lo=1024, hi=65536)
    starts = np.concatenate([[0], np.cumsum((sizes + 31) // 32 * 32)[:-1]]).astype(np.int64)
    total_alloc = int(starts[-1] + (sizes[-1] + 31) // 32 * 32)
    total = int(sizes.sum())
    keys = datagen.uniform_u32(total_alloc, 12, device=dev)
    vals = datagen.index_values(total_alloc, dev)
    outs = [(torch.zeros_like(keys), torch.zeros_like(vals)) for _ in range(3)]
    spl = {}

    def segs(ko, vo):
        out = []
        for i, (n, B, kind) in enumerate(zip(sizes.tolist(), buckets.tolist(), kinds)):
            o = int(starts[i])
            if kind == "range" and i not in spl:
                spl[i] = datagen.range_splitters(B, 2000 + i, dev)
            ident = gms.delta_bucket() if kind == "delta" else gms.range_bucket(spl[i])
            out.append(gms.Segment(keys[o:o + n], ko[o:o + n], n, B, ident, vals[o:o + n], vo[o:o + n]))
        return out

    def timed(plan):
        plan.run(use_graph=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            plan.run(use_graph=True)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    saved = gms.tuning_table()
    gms.reset_tuning()
    builtin = gms.BatchedMultisplit(segs(*outs[0]))
    gms.set_tuning({(B, True, c): v for B in (2, 8, 32, 256) for c, v in ((0, 2), (1, 1))})
    small = gms.BatchedMultisplit(segs(*outs[1]))
    gms.reset_tuning()
    builtin_ms, small_ms = timed(builtin), timed(small)
    t0 = time.perf_counter()
    gms.autotune(buckets=(2, 8, 32, 256), key_value=(True,), keys_per_trial=1 << 25, reps=5)
    tune_s = time.perf_counter() - t0
    tuned = gms.BatchedMultisplit(segs(*outs[2]))
    tuned_ms = timed(tuned)
    same = all(bool(torch.equal(outs[0][0], o[0]) and torch.equal(outs[0][1], o[1])) for o in outs[1:])
    for p in (builtin, small, tuned):
        p.close()
    gms.set_tuning(saved)
    res = {"workload": f"{len(sizes)} key-value segments, sizes log-uniform in [1024, 65536] (seed 8), "
                       f"B in {{2,8,32,256}}, delta or range; {total} pairs",
           "builtin_table_ms": builtin_ms, "small_tiles_table_ms": small_ms, "tuned_table_ms": tuned_ms,
           "autotune_s": tune_s, "builtin_vs_small_tiles": small_ms / builtin_ms,
           "builtin_vs_tuned": tuned_ms / builtin_ms, "identical": same}
    del keys, vals, outs
    torch.cuda.empty_cache()
    return res


def serving_trace(seconds: float, rate: float, seed: int = 5):
    """Poisson arrivals at `rate`/s for `seconds`; mix 60% multisplit, 20% 7-bit
    sort, 10% histogram, 10% compaction; sizes log-uniform in [4096, 16M]; half
    with values; multisplit B in {2, 8, 32, 256} (delta), histogram 256 bins."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=int(rate * seconds * 1.3) + 16)
    t = np.cumsum(gaps)
    t = t[t < seconds]
    m = len(t)
    sizes = np.exp(rng.uniform(np.log(4096), np.log(16 << 20), m)).astype(np.int64)
    ops = rng.choice(4, size=m, p=[0.6, 0.2, 0.1, 0.1])
    kv = rng.random(m) < 0.5
    buckets = rng.choice([2, 8, 32, 256], size=m)
    return t, sizes, ops, kv, buckets


def run_sweep(a, dev, out=None):
    """One JSON line per case (appended to `out` instead when given), inputs resident in HBM, CUDA events around
    `steps` calls after `warmup` calls, each case's output checked by a
    size-independent property (bucket order + permutation for multisplits,
    sortedness for sorts, total count for histograms).  Beside each GPU figure,
    the CPU implementation of the same op (the oracle's restatement of the
    reference's CPU code: the multisplits on every host thread, the others on
    one) timed on the first 2^22 keys."""
    import torch

    import gpumultisplit_gb300 as gms
    from gpumultisplit_gb300 import datagen

    n = 1 << a.log2n
    peak, _ = hbm_peak()
    inputs = {} if a.sweep_part in ("wide", "big") else {"uniform": datagen.uniform_u32(n, 3, device=dev),
                                      "zipf": datagen.zipf_u32(n, 3, device=dev),
                                      "and4": datagen.and4_u32(n, 3, device=dev)}
    vals = datagen.index_values(n, dev)
    kout, vout = torch.empty_like(vals), torch.empty_like(vals)
    steps, warm = max(3, a.steps // 2), max(3, a.warmup)

    def timed(fn):
        for _ in range(warm):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    import oracle

    if not oracle.LIB.exists():
        oracle.build(with_ref=False)
    ncpu = os.cpu_count() or 1
    sample_n = 1 << 22

    def cpu_rate(fn, threads):
        """CPU implementation of the same op (the oracle: the reference's algorithm)
        on the first sample_n keys, best of 3; Gkeys/s."""
        best = None
        for _ in range(3):
            t0 = time.perf_counter()
            fn()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        return {"gkeys": sample_n / best / 1e9, "threads": threads, "sample_keys": sample_n}

    def sample(t):
        return datagen.as_u32(t[:sample_n])

    def emit(case, ms, bytes_per_key, check, cpu=None):
        line = {"case": case, "n": n, "ms": ms, "gkeys": n / (ms * 1e-3) / 1e9,
                "algorithmic_bytes_per_key": bytes_per_key,
                "hbm_frac": bytes_per_key * n / (ms * 1e-3) / 1e9 / peak, "check": check}
        if cpu is not None:
            line["cpu"] = cpu
            line["gpu_vs_cpu"] = line["gkeys"] / cpu["gkeys"]
        if out is None:
            print(json.dumps(line), flush=True)
        else:
            out.append(line)

    def bucket_ids(x, B, ident_name, spl):
        u = x.to(torch.int64) & 0xFFFFFFFF
        if ident_name == "delta":
            return (u * B) >> 32
        s64 = spl.to(torch.int64) & 0xFFFFFFFF
        return torch.searchsorted(s64, u, right=True) - 1

    def multisplit_check(kin, ko, vo, B, ident_name, spl):
        b = bucket_ids(ko, B, ident_name, spl)
        ok = bool((b[1:] >= b[:-1]).all())
        if vo is not None:
            ok &= bool(torch.equal(kin[vo.long()], ko))
            same = b[1:] == b[:-1]
            ok &= bool((vo[1:][same] > vo[:-1][same]).all())  # stable: values = input index
        return "pass" if ok else "FAIL"

    if a.sweep_part in ("all", "base"):
        # The reference's CPU-runnable case (2^20 uniform keys, seed 1, 8 buckets by
        # key >> 29, key-only): 4 MiB stays in L2, so it is a latency figure, each
        # call timed alone (CUDA events around one call, median of 50) and checked
        # bit for bit against the oracle.
        n1 = 1 << 20
        k1 = datagen.uniform_u32(n1, 1, device=dev)
        o1 = torch.empty_like(k1)
        ctx1 = gms.multisplit_context(8)
        gms.multisplit_allocate_key_only(n1, ctx1)
        call1 = lambda: gms.multisplit_key_only(k1, o1, n1, ctx1, gms.bits_bucket(29))
        for _ in range(warm):
            call1()
        lat = []
        for _ in range(50):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            call1()
            e1.record()
            torch.cuda.synchronize()
            lat.append(e0.elapsed_time(e1))
        ms1 = statistics.median(lat)
        h1 = datagen.as_u32(k1)
        r1, _, _ = oracle.multisplit(h1, oracle.Desc(oracle.BITS, 8, shift=29), None)
        t0 = time.perf_counter()
        oracle.multisplit(h1, oracle.Desc(oracle.BITS, 8, shift=29), None)
        cpu1 = time.perf_counter() - t0
        line1 = {"case": "multisplit k B=8 key>>29, 2^20 keys (latency, L2-resident)", "n": n1, "ms": ms1,
                 "gkeys": n1 / (ms1 * 1e-3) / 1e9, "algorithmic_bytes_per_key": 12, "hbm_frac": None,
                 "check": "pass" if np.array_equal(datagen.as_u32(o1), r1) else "FAIL",
                 "cpu": {"gkeys": n1 / cpu1 / 1e9, "threads": 1, "sample_keys": n1}}
        line1["gpu_vs_cpu"] = line1["gkeys"] / line1["cpu"]["gkeys"]
        if out is None:
            print(json.dumps(line1), flush=True)
        else:
            out.append(line1)
        gms.multisplit_release_memory(ctx1)
        del k1, o1
        # key-value sweep: B x distribution x identifier
        for dist in ("uniform", "zipf"):
            for ident_name in ("delta", "range"):
                for B in (2, 32, 64, 128, 256):
                    spl = datagen.range_splitters(B, 5, dev) if ident_name == "range" else None
                    ident = gms.delta_bucket() if ident_name == "delta" else gms.range_bucket(spl)
                    ctx = gms.multisplit_context(B)
                    gms.multisplit_allocate_key_value(n, ctx)
                    kin = inputs[dist]
                    ms = timed(lambda: gms.multisplit_key_value(kin, vals, kout, vout, n, ctx, ident))
                    hk, hv = sample(kin), sample(vals)
                    desc = oracle.Desc(oracle.DELTA if ident_name == "delta" else oracle.RANGE, B,
                                       splitters=None if spl is None else datagen.as_u32(spl))
                    emit(f"multisplit kv B={B} {dist} {ident_name}", ms, 20,
                         multisplit_check(kin, kout, vout, B, ident_name, spl),
                         cpu_rate(lambda: oracle.multisplit_mt(hk, desc, hv, ncpu), ncpu))
                    gms.multisplit_release_memory(ctx)
        for B in (2, 32, 256):
            ctx = gms.multisplit_context(B)
            gms.multisplit_allocate_key_only(n, ctx)
            kin = inputs["uniform"]
            ms = timed(lambda: gms.multisplit_key_only(kin, kout, n, ctx, gms.delta_bucket()))
            ok = multisplit_check(kin, kout, None, B, "delta", None)
            ok = ok if bool(torch.equal(torch.sort(kout.long() & 0xFFFFFFFF)[0],
                                        torch.sort(kin.long() & 0xFFFFFFFF)[0])) else "FAIL"
            hk = sample(kin)
            emit(f"multisplit k B={B} uniform delta", ms, 12, ok,
                 cpu_rate(lambda: oracle.multisplit_mt(hk, oracle.Desc(oracle.DELTA, B), None, ncpu), ncpu))
            gms.multisplit_release_memory(ctx)
        # compaction, predicate key & 1
        for kv in (False, True):
            ctx = gms.compaction_context()
            kin = inputs["uniform"]
            if kv:
                gms.compaction_allocate_key_value(n, ctx)
                ms = timed(lambda: gms.compaction_key_value(kin, vals, kout, vout, n, ctx, gms.test_bucket(1)))
            else:
                gms.compaction_allocate_key_only(n, ctx)
                ms = timed(lambda: gms.compaction_key_only(kin, kout, n, ctx, gms.test_bucket(1)))
            b = kout & 1
            hk, hv = sample(kin), (sample(vals) if kv else None)
            emit(f"compaction {'kv' if kv else 'k'} key&1 uniform", ms, 20 if kv else 12,
                 "pass" if bool((b[1:] >= b[:-1]).all()) else "FAIL",
                 cpu_rate(lambda: oracle.compaction(hk, oracle.Desc(oracle.BITS, 2), hv), 1))
            gms.compaction_release_memory(ctx)
        # 256-bin histograms
        hist = torch.zeros(256, dtype=torch.int32, device=dev)
        kin = inputs["uniform"]
        ms = timed(lambda: gms.multisplit_histogram(kin, n, hist, 256, gms.delta_bucket()))
        hist.zero_()
        gms.multisplit_histogram(kin, n, hist, 256, gms.delta_bucket())
        hk = sample(kin)
        emit("histogram 256 bins delta uniform", ms, 4, "pass" if int(hist.sum()) == n else "FAIL",
             cpu_rate(lambda: oracle.histogram(hk, oracle.Desc(oracle.DELTA, 256)), 1))
        ms = timed(lambda: gms.histogram_even(kin, n, hist, 256, 0, 0xFFFFFFFF, 256.0 / 2**32))
        emit("histogram 256 bins even-float uniform", ms, 4, "pass",
             cpu_rate(lambda: oracle.histogram(hk, oracle.Desc(oracle.EVEN_FLOAT, 256, inverse_delta=256.0 / 2**32)), 1))
        # sorts (the 7-bit ones by both digit methods)
        for bits, method in ((7, "auto"), (7, "onesweep"), (4, "auto"), (5, "auto"), (6, "auto"), (8, "auto")):
            gms.set_sort_method(method)
            for dist in (("uniform", "and4") if bits == 7 else ("uniform",)):
                for kv in ((False, True) if bits == 7 else (True,)):
                    ctx = gms.ms_sort_context()
                    kin = inputs[dist]
                    fn = f"multisplit_sort_{bits}bit"
                    if kv:
                        getattr(gms, fn + "_allocate_pairs")(n, ctx)
                        ms = timed(lambda: getattr(gms, fn + "_pairs")(kin, kout, vals, vout, n, ctx))
                    else:
                        getattr(gms, fn + "_allocate")(n, ctx)
                        ms = timed(lambda: getattr(gms, fn)(kin, kout, n, ctx))
                    u = kout.long() & 0xFFFFFFFF
                    ok = bool((u[1:] >= u[:-1]).all())
                    if kv:
                        ok &= bool(torch.equal(kin[vout.long()], kout))
                    passes = {4: 8, 5: 7, 6: 6, 7: 5, 8: 4}[bits]
                    hk, hv = sample(kin), (sample(vals) if kv else None)
                    label = " (one-sweep passes)" if method == "onesweep" else ""
                    emit(f"sort {bits}-bit {'kv' if kv else 'k'} {dist}{label}", ms, passes * (20 if kv else 12),
                         "pass" if ok else "FAIL", cpu_rate(lambda: oracle.sort(hk, hv, bits), 1))
                    gms.multisplit_sort_release_memory(ctx)
            gms.set_sort_method("auto")
    del inputs, kout, vout
    torch.cuda.empty_cache()
    if a.sweep_part in ("all", "wide"):
        sweep_wide(n, dev, timed, emit, cpu_rate, sample, sample_n)
    if a.sweep_part in ("all", "big"):
        sweep_big(n, dev, timed, emit, cpu_rate, sample)


def sweep_wide(n, dev, timed, emit, cpu_rate, sample, sample_n):
    """64-bit keys and values: multisplit (B = 256, delta on the 64-bit key) and
    sorts.  Algorithmic bytes: prescan reads the key, postscan reads and writes
    key and value (the bucket bytes, 2 B/key, are not counted)."""
    import torch

    import gpumultisplit_gb300 as gms
    import oracle
    from gpumultisplit_gb300 import datagen

    k64 = datagen.uniform_u64(n, 3, device=dev)
    k32 = datagen.uniform_u32(n, 3, device=dev)
    v64 = torch.arange(n, dtype=torch.int64, device=dev)
    v32 = datagen.index_values(n, dev)
    sign = torch.tensor(-(1 << 63), dtype=torch.int64, device=dev)

    def wide_check(kin, ko, vo, top):
        """Bucket order (top 8 key bits), a permutation of the input, stable."""
        b = (ko >> (top - 8)) & 0xFF
        ok = bool((b[1:] >= b[:-1]).all())
        if vo is not None:
            idx = vo.long() & 0xFFFFFFFF
            ok &= bool(torch.equal(kin[idx], ko))
            same = b[1:] == b[:-1]
            ok &= bool((idx[1:][same] > idx[:-1][same]).all())
        return "pass" if ok else "FAIL"

    for kname, kin, vname, vin in (("u64", k64, None, None), ("u64", k64, "u32", v32), ("u64", k64, "u64", v64),
                                   ("u32", k32, "u64", v64)):
        kb, vb = kin.element_size(), 0 if vin is None else vin.element_size()
        ctx = gms.multisplit_context(256)
        gms.multisplit_wide_allocate(n, ctx, kb, vb)
        ko = torch.empty_like(kin)
        vo = None if vin is None else torch.empty_like(vin)
        ms = timed(lambda: gms.multisplit_wide(kin, ko, n, ctx, gms.delta_bucket(), vin, vo))
        check = wide_check(kin, ko, vo, 8 * kb) if kb == 8 else wide_check(kin.long() & 0xFFFFFFFF,
                                                                            ko.long() & 0xFFFFFFFF, vo, 32)
        if kb == 8:
            hk = datagen.as_u64(kin[:sample_n])
            hv = None if vin is None else vin[:sample_n].cpu().numpy()
            cpu = cpu_rate(lambda: oracle.multisplit64(hk, oracle.Desc64(oracle.DELTA, 256), hv), 1)
        else:
            hk, hv = sample(kin), sample(v32)
            cpu = cpu_rate(lambda: oracle.multisplit(hk, oracle.Desc(oracle.DELTA, 256), hv), 1)
        emit(f"multisplit {kname} keys{'' if vname is None else ' ' + vname + ' values'} B=256 delta", ms,
             kb + 2 * (kb + vb), check, cpu)
        del ctx, ko, vo
    for vname, vin in ((None, None), ("u64", v64)):
        ctx = gms.ms_sort_context()
        gms.multisplit_sort_wide_allocate(n, ctx, 8, 0 if vin is None else 8, 0, 64, 8)
        ko = torch.empty_like(k64)
        vo = None if vin is None else torch.empty_like(vin)
        ms = timed(lambda: gms.multisplit_sort_wide(k64, ko, n, ctx, vin, vo))
        u = ko ^ sign
        ok = bool((u[1:] >= u[:-1]).all())
        if vo is not None:
            ok &= bool(torch.equal(k64[vo], ko))
        hk = datagen.as_u64(k64[:sample_n])
        hv = None if vin is None else vin[:sample_n].cpu().numpy()
        emit(f"sort 64-bit keys{'' if vname is None else ' u64 values'} 8-bit digits", ms,
             8 * (8 + 2 * (8 + (0 if vin is None else 8))), "pass" if ok else "FAIL",
             cpu_rate(lambda: oracle.sort_bits64(hk, hv, 0, 64, 8), 1))
        del ctx, ko, vo


def sweep_big(n, dev, timed, emit, cpu_rate, sample):
    """More than 256 buckets: two digit passes, each with the traffic of a
    multisplit plus its bucket bytes; the algorithmic bytes are those of one
    multisplit (20 B/pair), so the HBM fraction shows the cost of the second
    pass."""
    import torch

    import gpumultisplit_gb300 as gms
    import oracle
    from gpumultisplit_gb300 import datagen

    kin = datagen.uniform_u32(n, 3, device=dev)
    vin = datagen.index_values(n, dev)
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    for B, ident_name in ((1000, "delta"), (4096, "delta"), (4096, "range"), (65536, "delta")):
        spl = datagen.range_splitters(B, 5, dev) if ident_name == "range" else None
        ident = gms.delta_bucket() if spl is None else gms.range_bucket(spl)
        ctx = gms.multisplit_context(B)
        gms.multisplit_allocate_key_value(n, ctx)
        ms = timed(lambda: gms.multisplit_key_value(kin, vin, kout, vout, n, ctx, ident))
        u = kout.long() & 0xFFFFFFFF
        if spl is None:
            b = (u * B) >> 32
        else:
            b = torch.searchsorted(spl.long() & 0xFFFFFFFF, u, right=True) - 1
        same = b[1:] == b[:-1]
        ok = bool((b[1:] >= b[:-1]).all()) and bool(torch.equal(kin[vout.long()], kout)) and \
            bool((vout[1:][same] > vout[:-1][same]).all())
        hk, hv = sample(kin), sample(vin)
        desc = oracle.Desc(oracle.DELTA if spl is None else oracle.RANGE, B,
                           splitters=None if spl is None else datagen.as_u32(spl))
        emit(f"multisplit kv B={B} uniform {ident_name} (two digit passes)", ms, 20, "pass" if ok else "FAIL",
             cpu_rate(lambda: oracle.multisplit(hk, desc, hv), 1))
        gms.multisplit_release_memory(ctx)
        hist = torch.zeros(B, dtype=torch.int32, device=dev)
        ms = timed(lambda: gms.multisplit_histogram(kin, n, hist, B, ident))
        hist.zero_()
        gms.multisplit_histogram(kin, n, hist, B, ident)
        emit(f"histogram {B} bins uniform {ident_name}", ms, 4, "pass" if int(hist.sum()) == n else "FAIL",
             cpu_rate(lambda: oracle.histogram(hk, desc), 1))

def run_tiny_segments(dev, count: int = 200000, seed: int = 9):
    """Many small multisplits: `count` key-value segments of 1..512 keys (uniform
    sizes, seed), B = 256 delta.  The tuned plan multisplits each segment with
    one warp in one launch; a forced 1024-key tile shape runs the tiled path
    (prescan, scan, postscan) on the same segments; the plain per-call loop is
    timed on a sample of 1000 segments and scaled.  Outputs are compared."""
    import torch

    import gpumultisplit_gb300 as gms
    from gpumultisplit_gb300 import datagen

    sizes = np.random.default_rng(seed).integers(1, 513, count)
    starts = np.concatenate([[0], np.cumsum(sizes)])
    total = int(starts[-1])
    keys = datagen.uniform_u32(total, seed, device=dev)
    vals = datagen.index_values(total, dev)
    kout, vout = torch.empty_like(keys), torch.empty_like(vals)
    segs = [gms.Segment(keys[a:b], kout[a:b], int(b - a), 256, gms.delta_bucket(), vals[a:b], vout[a:b])
            for a, b in zip(starts[:-1].tolist(), starts[1:].tolist())]
    warp_plan = gms.BatchedMultisplit(segs)
    tiled_plan = gms.BatchedMultisplit(segs, variant=2)

    def timed(fn, reps=10):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    warp_ms = timed(lambda: warp_plan.run(use_graph=True))
    ref_k, ref_v = kout.clone(), vout.clone()
    tiled_ms = timed(lambda: tiled_plan.run(use_graph=True))
    same = bool(torch.equal(kout, ref_k)) and bool(torch.equal(vout, ref_v))
    ctx = gms.multisplit_context(256)
    gms.multisplit_allocate_key_value(512, ctx)
    sample = segs[:1000]

    def plain():
        for sg in sample:
            gms.multisplit_key_value(sg.keys_in, sg.values_in, sg.keys_out, sg.values_out, sg.n, ctx, sg.identifier)

    plain_ms = timed(plain, 3) * count / len(sample)
    out = {"workload": f"{count} key-value segments of 1..512 keys (uniform sizes, seed {seed}), B = 256 delta; "
                       f"{total} pairs",
           "pairs": total, "one_warp_ms": warp_ms, "one_warp_gkeys": total / (warp_ms * 1e-3) / 1e9,
           "launches": warp_plan.launches, "tiled_ms": tiled_ms, "tiled_gkeys": total / (tiled_ms * 1e-3) / 1e9,
           "tiled_launches": tiled_plan.launches, "plain_ms_scaled": plain_ms,
           "plain_gkeys": total / (plain_ms * 1e-3) / 1e9, "identical": same,
           "device_error": warp_plan.device_error()}
    warp_plan.close()
    tiled_plan.close()
    return out

def run_serving(dev, seconds: float = 3.0, rate: float = 20000.0, arena_gb: float = 64.0, verify: int = 24,
                verify_all: bool = True, plain_graph_sample: int = 2000, plain_loop: bool = True):
    """Serving form under Poisson arrivals against the plain per-request calls on
    the same trace: p50/p99 latency (arrival to result) and Gkeys/s.  With
    verify_all, every request of the trace is then served once more (untimed)
    and each result is compared with the plain call on the same input."""
    import torch

    import gpumultisplit_gb300 as gms
    from gpumultisplit_gb300 import datagen
    from gpumultisplit_gb300 import serving as srv

    t_arr, sizes, ops, kv, buckets = serving_trace(seconds, rate)
    m = len(t_arr)
    pool_n = 1 << 28
    keys_pool = datagen.uniform_u32(pool_n, 21, device=dev)
    vals_pool = torch.arange(pool_n, dtype=torch.int32, device=dev)
    rng = np.random.default_rng(6)
    offs = (rng.integers(0, pool_n - sizes, m) // 32 * 32).astype(np.int64)
    names = ["multisplit", "sort7", "histogram", "compaction"]

    def desc_for(i):
        op = names[ops[i]]
        if op == "compaction":
            return gms.test_bucket(1).desc(2), 2
        if op == "histogram":
            return gms.delta_bucket().desc(256), 256
        if op == "sort7":
            return srv.BucketDesc(), 2
        return gms.delta_bucket().desc(int(buckets[i])), int(buckets[i])

    reqs = []
    base_k, base_v = keys_pool.data_ptr(), vals_pool.data_ptr()
    for i in range(m):
        d, _ = desc_for(i)
        has_v = bool(kv[i]) and ops[i] != 2
        reqs.append(srv.GmsRequest(int(ops[i]), base_k + 4 * int(offs[i]), base_v + 4 * int(offs[i]) if has_v else None,
                                   int(sizes[i]), d))
    total_keys = int(sizes.sum())

    # ---- served
    server = gms.Server(arena_bytes=int(arena_gb * (1 << 30)))
    lib = srv._lib_server()
    h = server._h
    rid = ctypes.c_uint64()
    res = srv.GmsResult()
    ids = [0] * m
    id_index = {}
    lat = np.zeros(m)
    done_t = np.zeros(m)
    sample = set(np.random.default_rng(7).choice(m, size=min(verify, m), replace=False).tolist())
    kept = {}
    ids_buf = (ctypes.c_uint64 * 8192)()
    cnt = ctypes.c_uint32()
    finished = 0

    def reap():
        nonlocal finished
        lib.gms_server_take_completed(h, ids_buf, 8192, ctypes.byref(cnt))
        for j in range(cnt.value):
            r = ids_buf[j]
            i = id_index[r]
            lib.gms_server_poll(h, r, ctypes.byref(res))
            lat[i] = res.done_s - res.submit_s
            done_t[i] = res.done_s
            if i in sample:
                kept[i] = server._result(r, res)
            else:
                lib.gms_server_release(h, r)
            finished += 1

    t0 = lib.gms_server_clock(h) + 0.05
    for i in range(m):
        target = t0 + t_arr[i]
        while lib.gms_server_clock(h) < target:
            pass
        st = lib.gms_server_submit(h, ctypes.byref(reqs[i]), ctypes.byref(rid))
        if st != 0:
            raise RuntimeError(f"submit failed: {st}")
        ids[i] = rid.value
        id_index[rid.value] = i
        server._meta[rid.value] = (names[ops[i]], int(sizes[i]), reqs[i].d_value_in is not None,
                                   desc_for(i)[1], None)
        if i % 64 == 0:
            reap()
    # Reap (and release) until every request is done: a blocking drain would
    # wait forever once unreleased results fill the arena (at saturation).
    while finished < m:
        before = finished
        reap()
        if finished == before:
            time.sleep(5e-5)
    stats = server.stats()
    served_span = float(done_t.max() - t0)
    # verify the sampled requests against the plain calls alone
    ok = True
    for i, r in kept.items():
        op, n = names[ops[i]], int(sizes[i])
        kin = keys_pool[offs[i]:offs[i] + n]
        vin = vals_pool[offs[i]:offs[i] + n] if reqs[i].d_value_in else None
        ident = gms.test_bucket(1) if op == "compaction" else gms.delta_bucket()
        ref = _plain_request(gms, op, kin, vin, n, desc_for(i)[1], ident)
        if op == "histogram":
            ok &= bool(torch.equal(r.histogram, ref[0]))
        else:
            ok &= bool(torch.equal(r.keys, ref[0])) and (vin is None or bool(torch.equal(r.values, ref[1])))
            if op == "compaction":
                ok &= r.num_bucket0 == ref[2]
    for i in kept:
        server.release(ids[i])
    server.close()
    kept.clear()
    del server

    # ---- every request, untimed: served result == plain call, bit for bit
    verified_all = None
    if verify_all:
        server = gms.Server(arena_bytes=int(arena_gb * (1 << 30)))
        h = server._h
        index = {}
        for i in range(m):
            st = lib.gms_server_submit(h, ctypes.byref(reqs[i]), ctypes.byref(rid))
            if st != 0:
                raise RuntimeError(f"submit failed: {st}")
            index[rid.value] = i
            server._meta[rid.value] = (names[ops[i]], int(sizes[i]), reqs[i].d_value_in is not None,
                                       desc_for(i)[1], None)
        vctx = {}
        vk = torch.empty(16 << 20, dtype=torch.int32, device=dev)
        vv = torch.empty(16 << 20, dtype=torch.int32, device=dev)
        vh = torch.empty(256, dtype=torch.int32, device=dev)
        checked, bad = 0, 0
        while checked < m:
            done_ids = server.take_completed()
            if not done_ids:
                time.sleep(2e-4)
                continue
            for r in done_ids:
                i = index[r]
                lib.gms_server_poll(h, r, ctypes.byref(res))
                got = server._result(r, res)
                op, n = names[ops[i]], int(sizes[i])
                kin = keys_pool[offs[i]:offs[i] + n]
                vin = vals_pool[offs[i]:offs[i] + n] if reqs[i].d_value_in else None
                ident = gms.test_bucket(1) if op == "compaction" else gms.delta_bucket()
                ref = _plain_request(gms, op, kin, vin, n, desc_for(i)[1], ident, vctx, vk, vv, vh)
                if op == "histogram":
                    same = bool(torch.equal(got.histogram, ref[0]))
                else:
                    same = bool(torch.equal(got.keys, ref[0])) and (vin is None or bool(torch.equal(got.values, ref[1])))
                    if op == "compaction":
                        same &= got.num_bucket0 == ref[2]
                bad += 0 if (same and res.status == 0) else 1
                server.release(r)
                checked += 1
        server.close()
        del server, vk, vv, vh, vctx
        verified_all = bad == 0

    # ---- plain per-request calls on the same trace (one stream, in arrival order)
    plain_lat = np.zeros(m)
    ctxs = {}
    kout = torch.empty(16 << 20, dtype=torch.int32, device=dev)
    vout = torch.empty(16 << 20, dtype=torch.int32, device=dev)
    hist = torch.empty(256, dtype=torch.int32, device=dev)
    tp0 = time.perf_counter() + 0.05
    for i in (range(m) if plain_loop else ()):
        target = tp0 + t_arr[i]
        while time.perf_counter() < target:
            pass
        op, n = names[ops[i]], int(sizes[i])
        kin = keys_pool[offs[i]:offs[i] + n]
        vin = vals_pool[offs[i]:offs[i] + n] if reqs[i].d_value_in else None
        _plain_request(gms, op, kin, vin, n, desc_for(i)[1],
                       gms.test_bucket(1) if op == "compaction" else gms.delta_bucket(), ctxs, kout, vout, hist)
        torch.cuda.synchronize()
        plain_lat[i] = time.perf_counter() - tp0 - t_arr[i]
    plain_span = time.perf_counter() - tp0

    # ---- the plain per-request path's device rate: the first requests of the
    # trace, each through its plain calls, captured into one CUDA graph and
    # replayed back to back (no host dispatch, no arrival gaps).  A compaction
    # is captured as its two-bucket multisplit: the plain call also reads the
    # bucket-0 count back to the host, which a graph cannot.
    plain_graph = None
    if plain_graph_sample:
        sample = range(min(plain_graph_sample, m))

        def plain_calls():
            for i in sample:
                op, n = names[ops[i]], int(sizes[i])
                kin = keys_pool[offs[i]:offs[i] + n]
                vin = vals_pool[offs[i]:offs[i] + n] if reqs[i].d_value_in else None
                if op == "compaction":
                    op = "multisplit"
                _plain_request(gms, op, kin, vin, n, desc_for(i)[1],
                               gms.test_bucket(1) if names[ops[i]] == "compaction" else gms.delta_bucket(), ctxs,
                               kout, vout, hist)

        plain_calls()  # contexts exist before the capture
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            plain_calls()
        graph.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            graph.replay()
        e1.record()
        torch.cuda.synchronize()
        g_ms = e0.elapsed_time(e1) / 3
        g_keys = int(sizes[:len(sample)].sum())
        plain_graph = {"requests": len(sample), "keys": g_keys, "ms": g_ms, "gkeys": g_keys / (g_ms * 1e-3) / 1e9}
        del graph
    del keys_pool, vals_pool, kout, vout
    torch.cuda.empty_cache()
    return {
        "workload": f"Poisson arrivals at {rate:.0f}/s for {seconds:.1f} s ({m} requests): 60% multisplit, "
                    "20% 7-bit sort, 10% histogram, 10% compaction; sizes log-uniform in [4096, 16M]; "
                    f"half with values; {arena_gb:.0f} GB arena",
        "requests": m,
        "keys": total_keys,
        "served_gkeys": total_keys / served_span / 1e9,
        "served_p50_ms": float(np.percentile(lat, 50) * 1e3),
        "served_p99_ms": float(np.percentile(lat, 99) * 1e3),
        # the same over requests that arrive after the first 0.5 s (start-up
        # costs such as the staging buffers' first growth fall before it)
        "served_p50_ms_after_0p5s": float(np.percentile(lat[t_arr >= 0.5], 50) * 1e3) if (t_arr >= 0.5).any() else None,
        "served_p99_ms_after_0p5s": float(np.percentile(lat[t_arr >= 0.5], 99) * 1e3) if (t_arr >= 0.5).any() else None,
        "plain_gkeys": total_keys / plain_span / 1e9 if plain_loop else None,
        "plain_p50_ms": float(np.percentile(plain_lat, 50) * 1e3) if plain_loop else None,
        "plain_p99_ms": float(np.percentile(plain_lat, 99) * 1e3) if plain_loop else None,
        "throughput_vs_plain": (total_keys / served_span) / (total_keys / plain_span) if plain_loop else None,
        "plain_graph": plain_graph,
        "rounds": int(stats["rounds"]),
        "max_requests_in_round": int(stats["max_requests_in_round"]),
        "launches": int(stats["launches"]),
        "arena_peak_gb": stats["arena_peak_bytes"] / (1 << 30),
        "verified_identical": bool(ok) and verified_all is not False,
        "verified_requests": m if verify_all else len(kept),
    }


def _plain_request(gms, op, kin, vin, n, B, ident, ctxs=None, kout=None, vout=None, hist=None):
    """One request through the plain per-call API (contexts cached by shape)."""
    import torch

    ctxs = {} if ctxs is None else ctxs
    kv = vin is not None
    ko = (kout[:n] if kout is not None else torch.empty(n, dtype=torch.int32, device=kin.device))
    vo = (vout[:n] if vout is not None else torch.empty(n, dtype=torch.int32, device=kin.device)) if kv else None
    cap = 16 << 20
    if op == "histogram":
        h = hist if hist is not None else torch.empty(B, dtype=torch.int32, device=kin.device)
        h.zero_()
        gms.multisplit_histogram(kin, n, h, B, ident)
        return h, None, None
    if op == "sort7":
        key = ("sort", kv)
        if key not in ctxs:
            ctxs[key] = gms.ms_sort_context()
            (gms.multisplit_sort_7bit_allocate_pairs if kv else gms.multisplit_sort_7bit_allocate)(cap, ctxs[key])
        if kv:
            gms.multisplit_sort_7bit_pairs(kin, ko, vin, vo, n, ctxs[key])
        else:
            gms.multisplit_sort_7bit(kin, ko, n, ctxs[key])
        return ko, vo, None
    if op == "compaction":
        key = ("compaction", kv)
        if key not in ctxs:
            ctxs[key] = gms.compaction_context()
            (gms.compaction_allocate_key_value if kv else gms.compaction_allocate_key_only)(cap, ctxs[key])
        c = (gms.compaction_key_value(kin, vin, ko, vo, n, ctxs[key], ident) if kv
             else gms.compaction_key_only(kin, ko, n, ctxs[key], ident))
        return ko, vo, c
    key = ("ms", B, kv)
    if key not in ctxs:
        ctxs[key] = gms.multisplit_context(B)
        (gms.multisplit_allocate_key_value if kv else gms.multisplit_allocate_key_only)(cap, ctxs[key])
    if kv:
        gms.multisplit_key_value(kin, vin, ko, vo, n, ctxs[key], ident)
    else:
        gms.multisplit_key_only(kin, ko, n, ctxs[key], ident)
    return ko, vo, None


def cpu_baseline(a, keys_dev, vals_dev, seconds):
    """Times the oracle's multi-threaded restatement on a bounded sample."""
    import oracle
    from gpumultisplit_gb300 import datagen

    threads = os.cpu_count() or 1
    n = keys_dev.numel()
    keys = datagen.as_u32(keys_dev)
    vals = None if vals_dev is None else datagen.as_u32(vals_dev)
    spl = None
    if a.identifier == "range":
        spl = datagen.as_u32(datagen.range_splitters(a.buckets, 5))
    d = oracle.Desc(oracle.DELTA if a.identifier == "delta" else oracle.RANGE, a.buckets, splitters=spl)
    oracle.multisplit_mt(keys[: 1 << 20], d, None if vals is None else vals[: 1 << 20], threads)  # warm
    reps, t0 = 0, time.perf_counter()
    while True:
        oracle.multisplit_mt(keys, d, vals, threads)
        reps += 1
        if time.perf_counter() - t0 >= seconds or reps >= 50:
            break
    el = time.perf_counter() - t0
    return {"value": reps * n / el / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reps} full multisplits of the same 2^{a.log2n}-key workload, "
                      f"{threads} threads (oracle/oracle.c oracle_multisplit_mt), {el:.1f} s"}


def run_reference(a):
    """--impl reference: the CPU implementation of the path on the host cores."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle
    from gpumultisplit_gb300 import datagen

    if not oracle.LIB.exists():
        oracle.build(with_ref=False)
    n = 1 << a.log2n
    keys_t, vals_t, spl_t = make_inputs(a, "cpu")
    keys = datagen.as_u32(keys_t)
    vals = None if vals_t is None else datagen.as_u32(vals_t)
    spl = None if spl_t is None else datagen.as_u32(spl_t)
    d = oracle.Desc(oracle.DELTA if a.identifier == "delta" else oracle.RANGE, a.buckets, splitters=spl)
    threads = os.cpu_count() or 1
    for _ in range(a.warmup):
        oracle.multisplit_mt(keys, d, vals, threads)
    times = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        oracle.multisplit_mt(keys, d, vals, threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = a.steps * n / tot / 1e9
    # The reference's CPU multisplit is single-threaded: the same algorithm on
    # one core (oracle_multisplit, a restatement of cpu_multisplit_pairs_general),
    # on the first 2^24 keys, best of 3.
    m = min(n, 1 << 24)
    k1, v1 = keys[:m], None if vals is None else vals[:m]
    best = None
    for _ in range(3):
        t0 = time.perf_counter()
        oracle.multisplit(k1, d, v1)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * tot / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic", "config": workload_config(a),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"full 2^{a.log2n}-key workload per step, {threads} threads "
                                   "(oracle/oracle.c oracle_multisplit_mt: the reference's "
                                   "cpu_multisplit_pairs_general algorithm, chunked across threads)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_baseline_1core": {"value": m / best / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"first 2^{m.bit_length() - 1} keys of the workload, best of 3, one thread "
                                         "(oracle/oracle.c oracle_multisplit: the reference's single-threaded "
                                         "cpu_multisplit_pairs_general; the reference's own build of that function "
                                         "ran within 3 % of it on x86, where its sources are available)"},
    }
    print(json.dumps(line), flush=True)


def pinned_buffer_gbs(buffers, dev, reps=2):
    """Copy rate (GB/s) of each pinned host buffer on its own: name -> (host,
    device, "h2d" | "d2h").  A buffer whose pages sit far from the GPU (another
    NUMA node of the host) shows up here as a slow copy."""
    import torch

    out = {}
    st = torch.cuda.Stream(device=dev)
    for name, (h, d, way) in buffers.items():
        if h is None or d is None:
            continue
        with torch.cuda.stream(st):
            (d.copy_(h, non_blocking=True) if way == "h2d" else h.copy_(d, non_blocking=True))
        st.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(st)
        with torch.cuda.stream(st):
            for _ in range(reps):
                (d.copy_(h, non_blocking=True) if way == "h2d" else h.copy_(d, non_blocking=True))
        t1.record(st)
        st.synchronize()
        out[name] = h.numel() * h.element_size() * reps / (t0.elapsed_time(t1) * 1e-3) / 1e9
    return out


def host_link_gbs(h_src, d_buf, h_dst, dev, reps=3):
    """Pinned host<->device copy bandwidth measured on this machine just before the
    end-to-end steps (the end-to-end figure is bounded by it): H2D alone, D2H
    alone, and both at once on two streams (GB/s each direction)."""
    import torch

    nbytes = h_src.numel() * h_src.element_size()
    s1, s2 = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        s1.wait_event(t0)
        s2.wait_event(t0)
        for _ in range(reps):
            fn()
        for st in (s1, s2):
            ev = torch.cuda.Event()
            ev.record(st)
            torch.cuda.current_stream().wait_event(ev)
        t1.record()
        torch.cuda.synchronize()
        return nbytes * reps / (t0.elapsed_time(t1) * 1e-3) / 1e9

    def h2d():
        with torch.cuda.stream(s1):
            d_buf.copy_(h_src, non_blocking=True)

    def d2h():
        with torch.cuda.stream(s2):
            h_dst.copy_(d_buf, non_blocking=True)

    def both():
        h2d()
        d2h()

    return {"h2d_gbs": timed(h2d), "d2h_gbs": timed(d2h), "concurrent_gbs_each": timed(both)}


def run_ours(a):
    rank, world, local = dist_env()
    affinity = bind_to_gpu_cpus(local)
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if a.only_batched or a.only_serving or a.only_tiny_segments:
        from gpumultisplit_gb300 import build as gbuild

        gbuild.build()
        if a.only_tiny_segments:
            out = run_tiny_segments(dev)
        else:
            out = (run_batched(dev, tune=a.autotune) if a.only_batched
                   else run_serving(dev, a.serve_seconds, a.serve_rate))
        print(json.dumps(out), flush=True)
        return
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    import gpumultisplit_gb300 as gms
    from gpumultisplit_gb300 import build as gbuild

    gbuild.build()
    gms.load()
    if a.sweep:
        run_sweep(a, dev)
        return

    n = 1 << a.log2n
    B = a.buckets
    keys, vals, spl = make_inputs(a, dev)
    kout = torch.empty_like(keys)
    vout = None if vals is None else torch.empty_like(vals)
    ident = gms.delta_bucket() if a.identifier == "delta" else gms.range_bucket(spl)
    ctx = gms.multisplit_context(B)
    (gms.multisplit_allocate_key_only if a.keys_only else gms.multisplit_allocate_key_value)(n, ctx)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    def step(ev=None):
        gms.multisplit_stages(keys, vals, kout, vout, n, ctx, ident, events=ev)

    for _ in range(max(3, a.warmup)):
        step()
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(a.steps)]
    with ClockSampler(local) as clk:
        # The timed steps last tens of milliseconds, less than one sampling
        # period, so untimed steps run back to back for CLOCK_SOAK_S first: the
        # samples then show the clocks under the load the timed steps run in.
        t_end = time.perf_counter() + CLOCK_SOAK_S
        while time.perf_counter() < t_end:
            for _ in range(20):
                step()
            torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        for i in range(a.steps):
            step(evs[i])
        torch.cuda.synchronize()
        barrier()
    clocks = clk.summary()
    clocks["window"] = f"{CLOCK_SOAK_S} s of back-to-back untimed steps, then the timed steps"
    assert gms.read_device_error(ctx) == 0
    total_ms = evs[0][0].elapsed_time(evs[-1][3])
    pre = [e[0].elapsed_time(e[1]) for e in evs]
    scan = [e[1].elapsed_time(e[2]) for e in evs]
    post = [e[2].elapsed_time(e[3]) for e in evs]
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / a.steps
    value = world * n / (ms_per_step * 1e-3) / 1e9

    # End to end through the one-call public API, host buffers, copies inside the
    # step: every step copies its keys (and values) in from pinned host memory,
    # runs the multisplit and copies both outputs back.  Steps alternate between
    # two streams with their own buffers, so one step's copies overlap the
    # neighbouring steps' work, as a caller streaming batches would run it.
    e2e = None
    if not a.no_e2e:
        hk = torch.empty(n, dtype=torch.int32, pin_memory=True)
        hk.copy_(keys)
        hv = torch.empty(n, dtype=torch.int32, pin_memory=True) if vals is not None else None
        if hv is not None:
            hv.copy_(vals)
        lanes = []
        for _ in range(2):
            lane_ctx = gms.multisplit_context(B)
            (gms.multisplit_allocate_key_only if a.keys_only else gms.multisplit_allocate_key_value)(n, lane_ctx)
            lanes.append({
                "stream": torch.cuda.Stream(device=dev), "ctx": lane_ctx,
                "dk": torch.empty_like(keys), "dv": torch.empty_like(vals) if vals is not None else None,
                "dko": torch.empty_like(keys), "dvo": torch.empty_like(vals) if vals is not None else None,
                "hko": torch.empty(n, dtype=torch.int32, pin_memory=True),
                "hvo": torch.empty(n, dtype=torch.int32, pin_memory=True) if vals is not None else None,
            })

        for ln in lanes:
            ln["h2d"] = [torch.cuda.Stream(device=dev) for _ in range(2)]
            ln["d2h"] = [torch.cuda.Stream(device=dev) for _ in range(2)]
            ln["ev_ms"], ln["ev_d2h"] = None, []

        def e2e_step(i):
            # Keys and values move on separate copy streams (separate copy
            # engines); a lane's next inputs may arrive once its multisplit has
            # read the previous ones, its next outputs once they were copied out.
            ln = lanes[i % 2]
            S = ln["stream"]
            h2d_pairs = [(ln["dk"], hk)] + ([(ln["dv"], hv)] if hv is not None else [])
            for cs, (dst, src) in zip(ln["h2d"], h2d_pairs):
                if ln["ev_ms"] is not None:
                    cs.wait_event(ln["ev_ms"])
                with torch.cuda.stream(cs):
                    dst.copy_(src, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                S.wait_event(ev)
            for ev in ln["ev_d2h"]:
                S.wait_event(ev)
            if hv is None:
                gms.multisplit_key_only(ln["dk"], ln["dko"], n, ln["ctx"], ident, stream=S)
            else:
                gms.multisplit_key_value(ln["dk"], ln["dv"], ln["dko"], ln["dvo"], n, ln["ctx"], ident, stream=S)
            ev_ms = torch.cuda.Event()
            ev_ms.record(S)
            ln["ev_ms"], ln["ev_d2h"] = ev_ms, []
            d2h_pairs = [(ln["hko"], ln["dko"])] + ([(ln["hvo"], ln["dvo"])] if hv is not None else [])
            for cs, (dst, src) in zip(ln["d2h"], d2h_pairs):
                cs.wait_event(ev_ms)
                with torch.cuda.stream(cs):
                    dst.copy_(src, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                ln["ev_d2h"].append(ev)

        def run_steps(count):
            start = torch.cuda.Event(enable_timing=True)
            stop = torch.cuda.Event(enable_timing=True)
            start.record()
            for ln in lanes:
                for st in [ln["stream"]] + ln["h2d"] + ln["d2h"]:
                    st.wait_event(start)
            for i in range(count):
                e2e_step(i)
            for ln in lanes:
                for st in [ln["stream"]] + ln["h2d"] + ln["d2h"]:
                    ev = torch.cuda.Event()
                    ev.record(st)
                    torch.cuda.current_stream().wait_event(ev)
            stop.record()
            return start, stop

        link = host_link_gbs(hk, lanes[0]["dk"], lanes[0]["hko"], dev)
        link["by_buffer_gbs"] = pinned_buffer_gbs(
            {"keys_in": (hk, lanes[0]["dk"], "h2d"), "values_in": (hv, lanes[0]["dv"], "h2d"),
             "keys_out_lane0": (lanes[0]["hko"], lanes[0]["dko"], "d2h"),
             "values_out_lane0": (lanes[0]["hvo"], lanes[0]["dvo"], "d2h"),
             "keys_out_lane1": (lanes[1]["hko"], lanes[1]["dko"], "d2h"),
             "values_out_lane1": (lanes[1]["hvo"], lanes[1]["dvo"], "d2h")}, dev)
        # Untimed steps for at least 1.5 s first: on some boxes the host link
        # runs at about half its rate for the first fraction of a second of
        # sustained copies after being idle (measured: 24 ms steps, then 13.5).
        t_warm = time.perf_counter()
        warm_steps = 0
        while warm_steps < max(3, a.warmup) or time.perf_counter() - t_warm < 1.5:
            run_steps(2)
            torch.cuda.synchronize()
            warm_steps += 2
        e_steps = max(4, a.steps // 2)
        # Five timed trials of e_steps steps each; the median trial is the
        # figure (a trial can meet a transient slowdown of the host link on a
        # shared host: one measured 34 ms per step between two of 13.5), and
        # every trial is reported.
        trial_ms = []
        for _ in range(5):
            barrier()
            torch.cuda.synchronize()
            s0, s1 = run_steps(e_steps)
            torch.cuda.synchronize()
            barrier()
            trial_ms.append(s0.elapsed_time(s1) / e_steps)
        e_ms = sorted(trial_ms)[len(trial_ms) // 2]
        if world > 1:
            import torch.distributed as dist

            t = torch.tensor([e_ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e_ms = float(t.item())
        nb = n * 4 * (1 if vals is None else 2)
        e2e = {"value": world * n / (e_ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": e_ms,
               "trials_ms_per_step": trial_ms, "steps_per_trial": e_steps, "warmup_steps": warm_steps,
               "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb,
               "pipeline": "one-call API from pinned host buffers; steps alternate over 2 streams, keys and "
                           "values copied on their own streams, so a step's copies overlap its neighbours' work",
               "host_link": link,
               "cpu_affinity": affinity,
               "link_frac": (nb / (e_ms * 1e-3) / 1e9) / link["concurrent_gbs_each"]}
        # every lane's last output is the same multisplit as the device-resident step
        ref_k = kout.cpu()
        for ln in lanes:
            assert torch.equal(ln["hko"], ref_k)
            if hv is not None:
                assert torch.equal(ln["hvo"], vout.cpu())
        del lanes

    per_key_step, per_key_post = algorithmic_bytes(a)
    peak, peak_src = hbm_peak()
    post_ms = statistics.mean(post)
    achieved = per_key_post * n / (post_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": "postscan_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": per_key_post * n,
                "traffic": ncu_traffic("postscan_kv" if vals is not None else "postscan_k", n)}
    step_gbs = per_key_step * n / (ms_per_step * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic", "config": workload_config(a),
        "roofline": roofline,
        "step_roofline": {"achieved": step_gbs, "frac": step_gbs / peak, "unit": "GB/s",
                          "algorithmic_bytes_per_key": per_key_step},
        "stages_ms": {"prescan": statistics.mean(pre), "scan": statistics.mean(scan), "postscan": post_ms},
        "clocks": clocks, "gpu_launches": 3 * a.steps, "e2e": e2e,
    }
    if not a.no_batched:
        del keys, vals, kout, vout
        torch.cuda.empty_cache()
        line["batched"] = run_batched(dev, tune=a.autotune)
        line["batched"]["tuning_check"] = run_tuning_check(dev)
    if not a.no_serving:
        line["serving"] = run_serving(dev, a.serve_seconds, a.serve_rate)
        # the server's capacity: arrivals at 200,000/s for 0.5 s, far above what it carries
        sat = run_serving(dev, 0.5, 200000.0, verify_all=False, plain_graph_sample=0, plain_loop=False)
        pg = line["serving"]["plain_graph"]
        line["serving"]["saturation"] = {
            k: sat[k] for k in ("workload", "requests", "served_gkeys", "served_p50_ms", "served_p99_ms",
                                "max_requests_in_round", "verified_identical")}
        if pg:
            line["serving"]["saturation"]["capacity_vs_plain_graph"] = sat["served_gkeys"] / pg["gkeys"]
    if not a.no_sweep:
        # every 2^28 case of the 32-bit sweep (key-value B x identifier x
        # distribution, key-only, compaction, histograms, sorts): one entry each
        sw = argparse.Namespace(**vars(a))
        sw.sweep_part = "base"
        sw.steps, sw.warmup = 6, 3
        cases = []
        run_sweep(sw, dev, cases)
        line["sweep"] = cases
    if rank == 0 and not a.no_cpu_baseline:
        keys, vals, _ = make_inputs(a, dev)
        line["cpu_baseline"] = cpu_baseline(a, keys, vals, a.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
