"""Benchmark: one 1,048,576 x 1,048,576-limb product on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full product of two SplitMix64 operands (seeds 3 and 4) of
1,048,576 uint64 limbs each (2,097,152-limb result; by default 2^21-point
transforms of whole 64-bit limbs over five primes, PREC_GPU_WIDE_DIGITS=0:
2^22-point transforms of 32-bit digits over three).  Printed as ONE JSON
line on rank 0:
  value  device time per product, operands already resident in HBM, L2
         flushed (256 MiB write) between timed steps; CUDA events on the
         stream the kernels run on
  e2e    the same product through the public host API prec_gpu_mul with
         pinned host buffers: host->device copy of both operands, the
         product, device->host copy of the result, every step
  roofline  the dominant kernel's algorithmic bytes (per-stage split of
         144*N + 16*(La+Lb)) over its live event time, against the measured
         HBM copy bandwidth
  cpu_baseline  the oracle restatement of the reference NTT multiply, one
         thread, a bounded sample of the same product
  clocks nvidia-smi samples over the timed steps and a sustained window of
         at least a second of the same step back to back after them
  config1, fft_3000, batch, serve, pi_1e8  compact results of the other
         configurations (8192^2 product; 3000^2 on the FP64 band; 4096 uneven
         products batched vs plain; serving p50/p99; pi to 10^8 digits), each
         with its own exactness check (--headline-only omits them)
With --impl reference the same line is produced for the reference's CPU
algorithm (oracle port; the reference sources do not exist on the GPU
hosts) run on every host core, one independent product per core.
Under torchrun with N > 1 ranks each rank runs an independent replica on
its own GPU (the product does not shard); value = max time / products.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

AN = BN = 1 << 20
SEED_A, SEED_B = 3, 4
METRIC = "1M×1M-limb mul ms"
WORKLOAD = "1,048,576 x 1,048,576-limb uint64 product (SplitMix64 seeds 3,4)"
GOLDEN = os.path.join(ROOT, "tests", "golden", "products.json")
SUSTAIN_S = 1.2  # seconds of back-to-back steps after the timed ones, for the clock sampler


def host_link(host, devbuf, stream, reps=5):
    """Pinned host <-> device copy rates in GB/s (median of `reps` copies of
    `host`'s size each way, CUDA events on `stream`)."""
    import torch
    rates = []
    for dst, src in ((devbuf, host), (host, devbuf)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = []
        with torch.cuda.stream(stream):
            for i in range(reps + 2):
                e0.record(stream)
                dst.copy_(src, non_blocking=True)
                e1.record(stream)
                e1.synchronize()
                if i >= 2:
                    ms.append(e0.elapsed_time(e1))
        rates.append(round(host.numel() * host.element_size() / statistics.median(ms) / 1e6, 1))
    return rates


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _traffic():
    """Per-launch DRAM bytes per kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "ntt_1Mx1M_traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _golden_sha():
    try:
        with open(GOLDEN) as f:
            for r in json.load(f)["products"]:
                if r["name"] == "cfg2_1Mx1M_ntt":
                    return r["sha256"]
    except (OSError, ValueError, KeyError):
        pass
    return None


def algorithmic_bytes(la: int, lb: int):
    """Canonical bytes of the NTT path (32-bit digits, 3 primes, 4-byte
    residues) split per kernel: N = next_pow2(2(La+Lb))."""
    n = 1
    while n < 2 * (la + lb):
        n <<= 1
    io = 8 * (la + lb)
    return n, {
        "k_fwd_cols": io + 24 * n + 48 * n,   # split + forward pass 1
        "k_rows": 36 * n,                     # forward pass 2 + pointwise + inverse pass 1
        "k_inv_cols": 24 * n,                 # inverse pass 2
        "k_crt_carry": 12 * n + io,           # CRT + carry
    }


class Clocks:
    """nvidia-smi sampler (200 ms) around the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        except OSError:
            pass
        finally:
            if self.path:
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        busy = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows
                                                         if r[3].replace(".", "").isdigit())}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def ranks_max(dist, x: float, device) -> float:
    """The largest x over the ranks of the process group (x itself without
    one): the slowest replica's time is the job's."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_ms_per_product(slowest_total_ms: float, steps: int, world: int) -> float:
    """Whole-job time per product: every rank timed `steps` products of its
    own (replicas, weak scaling), so the job made steps * world products in
    the slowest rank's time."""
    return slowest_total_ms / steps / world


def cpu_time(fn, max_products: int, budget_s: float):
    """Median wall time (ms) of fn() on this host thread over at most
    `max_products` calls or `budget_s` seconds (at least one call)."""
    times = []
    t_end = time.perf_counter() + budget_s
    while len(times) < max_products and (not times or time.perf_counter() < t_end):
        t = time.perf_counter()
        fn()
        times.append(time.perf_counter() - t)
    return statistics.median(times) * 1e3, len(times)


def cpu_sample(max_products: int = 3, budget_s: float = 20.0):
    """Oracle restatement of mul_ntt on this host, one thread."""
    import oracle as O
    from preclib_gb300 import workloads
    a = workloads.operand(SEED_A, AN)
    b = workloads.operand(SEED_B, BN)
    return cpu_time(lambda: O.mul_ntt(a, b), max_products, budget_s)


def run_reference(args):
    """The reference's CPU algorithm on all host cores (oracle port), one
    independent 1M x 1M product per core per step."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle as O
    from preclib_gb300 import workloads
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    a = workloads.operand(SEED_A, AN)
    b = workloads.operand(SEED_B, BN)
    O.lib()

    def one(_):
        return O.mul_ntt(a, b)

    steps = []
    with ThreadPoolExecutor(cores) as ex:
        for i in range(args.warmup + args.steps):
            t = time.perf_counter()
            outs = list(ex.map(one, range(cores)))
            dt = time.perf_counter() - t
            if i >= args.warmup:
                steps.append(dt)
            del outs
    ms = sum(steps) / len(steps) / cores * 1e3
    line = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 4), "unit": "ms",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(sum(steps) / len(steps) * 1e3, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "an": AN, "bn": BN, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": round(ms, 4), "unit": "ms", "cores": cores, "kind": "port",
                         "sample": "%d independent 1M x 1M products per step (one per core), "
                                   "wall time / products" % cores},
        "e2e": {"value": round(ms, 4), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


CFG1_N, CFG1_SEEDS = 8192, (1, 2)


def run_config1(args, flush):
    """The plain single product of 8192 x 8192 limbs (SplitMix64 seeds 1, 2;
    NTT band, 2^15 points): device time per product with the operands
    resident (CUDA events on the launching stream, L2 flushed between
    steps), the same product end to end through prec_gpu_mul from pinned
    host buffers, bit-exactness against the reference's mul_ntt output
    (golden), and the oracle restatement of mul_ntt on one core."""
    import torch

    import oracle as O
    from preclib_gb300 import native, workloads
    dev = flush.device
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    a = workloads.operand(CFG1_SEEDS[0], CFG1_N)
    b = workloads.operand(CFG1_SEEDS[1], CFG1_N)
    ta = torch.from_numpy(a.view(np.int64)).to(dev)
    tb = torch.from_numpy(b.view(np.int64)).to(dev)
    to = torch.empty(2 * CFG1_N, dtype=torch.int64, device=dev)
    for _ in range(args.warmup):
        native.mul_device(ta.data_ptr(), CFG1_N, tb.data_ptr(), CFG1_N, to.data_ptr(), sptr)
    native.stream_check(sptr)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        evs[i][0].record(stream)
        native.mul_device(ta.data_ptr(), CFG1_N, tb.data_ptr(), CFG1_N, to.data_ptr(), sptr)
        evs[i][1].record(stream)
    torch.cuda.synchronize(dev)
    native.stream_check(sptr)
    dev_ms = statistics.median(e0.elapsed_time(e1) for e0, e1 in evs)
    with open(GOLDEN) as f:
        want = [r for r in json.load(f)["products"] if r["name"] == "cfg1_8192x8192_ntt"][0]["sha256"]

    def sha(x):
        return hashlib.sha256(np.ascontiguousarray(x, dtype="<u8").tobytes()).hexdigest()

    exact = sha(to.cpu().numpy().view(np.uint64)) == want
    ha = torch.from_numpy(a.view(np.int64)).pin_memory()
    hb = torch.from_numpy(b.view(np.int64)).pin_memory()
    ho = torch.empty(2 * CFG1_N, dtype=torch.int64).pin_memory()
    pa, pb, po = (x.numpy().view(np.uint64) for x in (ha, hb, ho))
    L = native.lib()
    for _ in range(args.warmup):
        native.check(L.prec_gpu_mul(native._p(pa), CFG1_N, native._p(pb), CFG1_N, native._p(po)))
    e2e = []
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        native.check(L.prec_gpu_mul(native._p(pa), CFG1_N, native._p(pb), CFG1_N, native._p(po)))
        e2e.append(time.perf_counter() - t)
    plan = native.last_stats()
    exact = exact and sha(po) == want
    # host calls from 1 and from 4 threads (each thread its own stream and
    # workspace; ctypes releases the interpreter lock during a call)
    from concurrent.futures import ThreadPoolExecutor
    per = 200
    outs = [np.empty(2 * CFG1_N, np.uint64) for _ in range(4)]

    def worker(t):
        o = outs[t]
        for _ in range(per):
            native.check(L.prec_gpu_mul(native._p(pa), CFG1_N, native._p(pb), CFG1_N, native._p(o)))
        return sha(o) == want

    threads = {}
    for nt in (1, 4):
        with ThreadPoolExecutor(nt) as ex:
            list(ex.map(worker, range(nt)))  # warm-up: each thread's lane
            t = time.perf_counter()
            ok = all(ex.map(worker, range(nt)))
            threads[str(nt)] = round(nt * per / (time.perf_counter() - t), 1)
        exact = exact and ok
    out = {"workload": "8192 x 8192-limb uint64 product (SplitMix64 seeds 1,2), NTT band",
           "transform_points": 1 << plan.log2_n, "primes": plan.primes, "digit_bits": plan.digit_bits,
           "device_ms": round(dev_ms, 4), "e2e_ms": round(statistics.median(e2e) * 1e3, 4),
           "h2d_bytes_per_step": 16 * CFG1_N, "d2h_bytes_per_step": 16 * CFG1_N,
           "steps": args.steps, "bit_exact": bool(exact),
           "host_calls_products_per_s_by_threads": threads,
           "l2": "flushed between timed steps (256 MiB write)"}
    if not args.skip_cpu:
        cpu_ms, nprod = cpu_time(lambda: O.mul_ntt(a, b), max_products=200, budget_s=2.0)
        out["cpu_baseline"] = {"value": round(cpu_ms, 4), "unit": "ms", "cores": 1, "kind": "port",
                               "sample": "%d single-threaded 8192 x 8192 products with the oracle restatement "
                                         "of mul_ntt (16-bit digits, 2 primes), median" % nprod}
    return out


def sub_results(args, flush):
    """Compact results of the other benchmark configurations for the default
    line, each with its own exactness check: the 8192^2 product, the FP64
    band at 3000^2, the 4096-product batch, the serving loop and pi to 10^8
    digits (fewer steps than their own workloads take)."""
    sub = argparse.Namespace(**vars(args))
    sub.steps = max(3, min(args.steps, 5))
    sub.warmup = 3
    res = {"config1": run_config1(args, flush)}
    f = run_fft(sub, emit=False)
    res["fft_3000"] = {"device_ms": f["value"], "e2e_ms": f["e2e"]["value"],
                       "digit_bits": f["config"]["digit_bits"], "transform_points": f["config"]["transform_points"],
                       "max_rounding_distance": f["max_rounding_distance"],
                       "reference_max_rounding_distance": f["reference_max_rounding_distance"],
                       "bit_exact": f["bit_exact"], "cpu_baseline": f.get("cpu_baseline")}
    bt = run_batch(sub, emit=False)
    res["batch"] = {"workload": bt["config"]["workload"], "length_classes": bt["config"]["length_classes"],
                    "batched_products_per_s": bt["value"], "plain_products_per_s": bt["plain_products_per_s"],
                    "batched_vs_plain": bt["batched_vs_plain"], "device": bt["device"],
                    "mismatches_vs_plain": bt["mismatches_vs_plain"], "steps": bt["steps"]}
    sv = run_serve(sub, emit=False)
    mid = [x for x in sv["loads"] if x["load"] == 0.5][0]
    res["serve"] = {"workload": sv["config"]["workload"], "capacity_products_per_s": sv["capacity_products_per_s"],
                    "p50_ms_at_50pct": mid["p50_ms"], "p99_ms_at_50pct": mid["p99_ms"], "loads": sv["loads"],
                    "mismatches_alone_vs_mixed": sv["mismatches_alone_vs_mixed"], "checked": sv["checked"]}
    sub.steps = 1
    pi = run_pi(sub, emit=False)
    res["pi_1e8"] = {"whole_program_s": pi["value"], "phases_s": pi["phases_s"], "bit_exact": pi["bit_exact"],
                     "runs": pi["steps"]}
    return res


def run_ours(args):
    import torch

    from preclib_gb300 import native, workloads
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    native.init(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    a = workloads.operand(SEED_A, AN)
    b = workloads.operand(SEED_B, BN)
    ta = torch.from_numpy(a.view(np.int64)).to(dev)
    tb = torch.from_numpy(b.view(np.int64)).to(dev)
    to = torch.empty(AN + BN, dtype=torch.int64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step():
        native.mul_device(ta.data_ptr(), AN, tb.data_ptr(), BN, to.data_ptr(), sptr)

    for _ in range(args.warmup):
        step()
        flush.fill_(1)
    native.stream_check(sptr)

    # ---- timed region: device-resident operands, L2 flushed between steps;
    # each product timed by CUDA events on the launching stream (the library
    # forks its per-prime chains from that stream and joins them back)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    launches0 = native.launch_count()
    with Clocks(local) as clk:
        for i in range(args.steps):
            evs[i][0].record(stream)
            step()
            evs[i][1].record(stream)
            flush.fill_(i & 0xFF)
        torch.cuda.synchronize(dev)
        launches = native.launch_count() - launches0
        # sustained window: the same step back to back for at least a second,
        # so the clock sampler (200 ms) sees the kernels under load
        sus = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(64)]
        sus_ms = []
        t_sus = time.perf_counter()
        while time.perf_counter() - t_sus < args.sustain:
            for j, (e0, e1) in enumerate(sus):
                e0.record(stream)
                step()
                e1.record(stream)
                flush.fill_(j & 0xFF)
            torch.cuda.synchronize(dev)
            sus_ms.extend(e0.elapsed_time(e1) for e0, e1 in sus)
        sus_s = time.perf_counter() - t_sus
    clocks = clk.summary()
    native.stream_check(sptr)
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    total_ms = sum(step_ms)

    # ---- per-kernel durations (events between the kernels, one stream):
    # the dominant kernel's roofline and the stage breakdown
    stage_tot = {}
    nprof = max(3, min(args.steps, 10))
    for i in range(nprof):
        for name, ms in native.mul_device_profile(ta.data_ptr(), AN, tb.data_ptr(), BN, to.data_ptr(), sptr):
            stage_tot[name] = stage_tot.get(name, 0.0) + ms
        flush.fill_(i & 0xFF)
    native.stream_check(sptr)
    total_ms = ranks_max(dist, total_ms, dev)
    out = to.cpu().numpy().view(np.uint64)
    sha = hashlib.sha256(np.ascontiguousarray(out, dtype="<u8").tobytes()).hexdigest()
    golden = _golden_sha()
    bit_exact = golden is not None and sha == golden

    # ---- end to end through the public host API (pinned host buffers)
    ha = torch.from_numpy(a.view(np.int64)).pin_memory()
    hb = torch.from_numpy(b.view(np.int64)).pin_memory()
    ho = torch.empty(AN + BN, dtype=torch.int64).pin_memory()
    pa = ha.numpy().view(np.uint64)
    pb = hb.numpy().view(np.uint64)
    po = ho.numpy().view(np.uint64)
    L = native.lib()
    for _ in range(max(1, args.warmup)):
        native.check(L.prec_gpu_mul(native._p(pa), AN, native._p(pb), BN, native._p(po)))
    e2e = []
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        native.check(L.prec_gpu_mul(native._p(pa), AN, native._p(pb), BN, native._p(po)))
        e2e.append(time.perf_counter() - t)
    e2e_exact = hashlib.sha256(np.ascontiguousarray(po, dtype="<u8").tobytes()).hexdigest() == golden
    plan = native.last_stats()  # the plan of the product: transform length, primes, digit width
    e2e_ms = ranks_max(dist, statistics.mean(e2e) * 1e3, dev)
    link = host_link(ho, to, stream)

    # ---- roofline of the dominant kernel (live events) and of the whole product
    peak, peak_kind = _peaks()
    n, alg = algorithmic_bytes(AN, BN)
    avg = {k: v / nprof for k, v in stage_tot.items()}
    dom = max(avg, key=avg.get)
    dom_gbs = alg[dom] / (avg[dom] * 1e-3) / 1e9
    traffic = _traffic().get(dom)
    total_alg = sum(alg.values())
    per_product_ms = job_ms_per_product(total_ms, args.steps, ws)

    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        cpu_ms, nprod = cpu_sample()
        cpu = {"value": round(cpu_ms, 3), "unit": "ms", "cores": 1, "kind": "port",
               "sample": "%d single-threaded 1M x 1M products with the oracle restatement of "
                         "mul_ntt (16-bit digits, 2 primes), median" % nprod}
    subs = None
    if rank == 0 and ws == 1 and not args.headline_only:
        subs = sub_results(args, flush)
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(per_product_ms, 4), "unit": "ms", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "an": AN, "bn": BN,
                       "transform_points": 1 << plan.log2_n, "primes": plan.primes,
                       "digit_bits": plan.digit_bits, "canonical_points": n,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "products_per_s": round(1e3 / per_product_ms, 2),
            "bit_exact": bool(bit_exact and e2e_exact),
            "stage_ms": {k: round(v, 4) for k, v in avg.items()},
            "stage_ms_note": "kernels run back to back on one stream; the timed products run each "
                             "prime's three transform kernels on its own stream",
            "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(dom_gbs, 1),
                         "peak": peak, "unit": "GB/s", "frac": round(dom_gbs / peak, 4),
                         "peak_source": peak_kind,
                         "traffic": traffic, "algorithmic_bytes": alg[dom]},
            "roofline_passes": {k: round(alg[k] / (avg[k] * 1e-3) / 1e9 / peak, 4) for k in avg if k in alg},
            "roofline_product": {"bytes": total_alg,
                                 "achieved": round(total_alg / (per_product_ms * 1e-3 * ws) / 1e9, 1),
                                 "frac": round(total_alg / (per_product_ms * 1e-3 * ws) / 1e9 / peak, 4),
                                 "unit": "GB/s"},
            "e2e": {"value": round(e2e_ms, 4), "unit": "ms", "h2d_bytes_per_step": 8 * (AN + BN),
                    "d2h_bytes_per_step": 8 * (AN + BN)},
            "host_link": {"h2d_gbs": link[0], "d2h_gbs": link[1],
                          "transfer_ms": round(8 * (AN + BN) * (1 / link[0] + 1 / link[1]) / 1e6, 4),
                          "note": "pinned copies of the product's size in each direction (CUDA events); "
                                  "the e2e copies of both operands in and the product out take transfer_ms "
                                  "at these rates"},
            "gpu_launches": launches,
            "clocks": clocks,
            "clocks_window": "the %d timed steps, then the same step back to back for %.2f s "
                             "(sustained)" % (args.steps, sus_s),
            "sustained": {"seconds": round(sus_s, 3), "products": len(sus_ms),
                          "median_ms": round(statistics.median(sus_ms), 4) if sus_ms else None},
            "cpu_baseline": cpu,
        }
        if subs:
            line.update(subs)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


BATCH_COUNT, BATCH_SEED = 4096, 7


def run_batch(args, emit=True):
    """Batched uneven products: 4096 products, lo log-uniform in [200, 65536]
    limbs, hi = lo * U[1, 2], SplitMix64 operands.  A step is the whole set.
    Batched: one H2D of all operands, one graph replay, one D2H of all
    results.  Plain: prec_gpu_mul per product (host pointers, one call per
    product).  Both measured end to end, and device-resident.  Returns the
    line (printed when `emit`)."""
    import torch

    from preclib_gb300 import native, workloads
    native.init(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    lo, hi = workloads.batch_sizes(BATCH_SEED, BATCH_COUNT)
    sizes = [(int(h), int(l)) for l, h in zip(lo, hi)]
    offs, o = [], 0
    for a, b in sizes:
        offs.append(o)
        o += a + b
    host = workloads.splitmix64(BATCH_SEED, o)
    host_in = torch.from_numpy(host.view(np.int64)).pin_memory()
    host_out = torch.empty(o, dtype=torch.int64).pin_memory()
    d_in = torch.empty(o, dtype=torch.int64, device=dev)
    d_out = torch.empty(o, dtype=torch.int64, device=dev)
    bi, bo = d_in.data_ptr(), d_out.data_ptr()
    items = [(bi + 8 * off, a, bi + 8 * (off + a), b, bo + 8 * off) for off, (a, b) in zip(offs, sizes)]
    # kernel configuration of every four-step length class of the batch
    # picked by the autotuner before the batch is planned (untimed)
    kmax = max(native.ntt_log2(a, b) for a, b in sizes)
    t_tune = time.perf_counter()
    tuned = native.autotune(13, kmax)
    tune_s = time.perf_counter() - t_tune
    batch = native.Batch(items)
    ncls, nbytes = batch.info()

    def batched_e2e():
        d_in.copy_(host_in, non_blocking=True)
        batch.run(sptr)
        host_out.copy_(d_out, non_blocking=True)
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        batched_e2e()
    native.stream_check(sptr)
    launches0 = native.launch_count()
    t = time.perf_counter()
    for _ in range(args.steps):
        batched_e2e()
    batched_s = (time.perf_counter() - t) / args.steps
    launches = native.launch_count() - launches0
    batched_out = host_out.numpy().view(np.uint64).copy()
    # device-resident batch (graph replay only)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        batch.run(sptr)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    batched_dev_s = e0.elapsed_time(e1) / 1e3 / args.steps

    # plain path: one prec_gpu_mul call per product, host pointers
    pin = host_in.numpy().view(np.uint64)
    pout = host_out.numpy().view(np.uint64)
    L = native.lib()
    base_i = pin.ctypes.data
    base_o = pout.ctypes.data
    u64p = native._u64p
    calls = [(ctypes_cast(base_i + 8 * off, u64p), a, ctypes_cast(base_i + 8 * (off + a), u64p), b,
              ctypes_cast(base_o + 8 * off, u64p)) for off, (a, b) in zip(offs, sizes)]
    plain_steps = max(1, min(args.steps, 3))
    for c in calls[:64]:
        native.check(L.prec_gpu_mul(*c))
    t = time.perf_counter()
    for _ in range(plain_steps):
        for c in calls:
            native.check(L.prec_gpu_mul(*c))
    plain_s = (time.perf_counter() - t) / plain_steps
    mismatches = sum(not np.array_equal(batched_out[off:off + a + b], pout[off:off + a + b])
                     for off, (a, b) in zip(offs, sizes))
    # plain device-resident: prec_gpu_mul_device per product
    e0.record(stream)
    for it in items:
        native.check(L.prec_gpu_mul_device(*it, sptr or None))
    e1.record(stream)
    torch.cuda.synchronize(dev)
    plain_dev_s = e0.elapsed_time(e1) / 1e3
    batch.close()
    n = BATCH_COUNT
    line = {
        "metric": "batched products/s (4096 uneven products)", "value": round(n / batched_s, 1),
        "unit": "products/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(batched_s * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "4096 products, lo log-uniform [200, 65536] limbs, hi = lo*U[1,2], "
                               "SplitMix64 seed 7", "limbs_in": o, "length_classes": ncls,
                   "device_bytes": nbytes, "l2": "inputs (%.0f MB) exceed L2" % (16 * o / 1e6)},
        "plain_products_per_s": round(n / plain_s, 1),
        "batched_vs_plain": round(plain_s / batched_s, 2),
        "device": {"batched_products_per_s": round(n / batched_dev_s, 1),
                   "plain_products_per_s": round(n / plain_dev_s, 1),
                   "batched_vs_plain": round(plain_dev_s / batched_dev_s, 2)},
        "mismatches_vs_plain": int(mismatches),
        "autotune": {"seconds": round(tune_s, 3),
                     "classes": {str(t["log2_n"]): [t["log2_cols"], t["col_group"], t["col_radix_cap"],
                                                    t["rows_per_cta"], t["split_primes"]] for t in tuned},
                     "fields": "log2_cols, col_group, col_radix_cap, rows_per_cta, split_primes"},
        "e2e": {"value": round(n / batched_s, 1), "unit": "products/s", "h2d_bytes_per_step": 8 * o,
                "d2h_bytes_per_step": 8 * o},
        "gpu_launches": launches,
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


SERVE_SEED = 11


def run_serve(args, emit=True):
    """Serving loop: requests with device-resident operands (slices of one
    random device buffer), an = bn = s with s log-uniform in [256, 4194304]
    limbs.  Capacity = products/s with every request queued at once; then
    Poisson arrivals at 10..90 % of capacity, p50/p99 latency per load.
    A sample of results is recomputed alone and compared with the mix.
    Returns the line (printed when `emit`)."""
    import hashlib

    import torch

    from preclib_gb300 import native, workloads
    native.init(0)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(SERVE_SEED)
    n_cap, n_load = 400, 300
    pool_limbs = 1 << 23
    d_pool = torch.from_numpy(workloads.splitmix64(SERVE_SEED, pool_limbs).view(np.int64)).to(dev)
    base = d_pool.data_ptr()

    def make(n):
        s = np.rint(np.exp(rng.uniform(np.log(256), np.log(4194304), n))).astype(np.int64)
        reqs, tot = [], 0
        for x in s:
            x = int(x)
            oa = int(rng.integers(0, pool_limbs - x + 1))
            ob = int(rng.integers(0, pool_limbs - x + 1))
            reqs.append((base + 8 * oa, x, base + 8 * ob, x, tot))
            tot += 2 * x
        return reqs, tot

    budget = 24 << 30
    srv = native.Server(budget, slots=16)

    def run_set(reqs, out, rate):
        ob = out.data_ptr()
        tickets = []
        t0 = time.perf_counter()
        t_next = t0
        for (a, an, b, bn, off) in reqs:
            if rate:
                t_next += rng.exponential(1.0 / rate)
                while time.perf_counter() < t_next:
                    pass
            tickets.append(srv.submit(a, an, b, bn, ob + 8 * off))
        srv.drain(600)
        lat = np.array([srv.wait(t, 1.0) for t in tickets])
        span = time.perf_counter() - t0
        return lat, len(reqs) / span

    # warm-up, then capacity (all queued at once)
    reqs, tot = make(64)
    out = torch.empty(tot, dtype=torch.int64, device=dev)
    run_set(reqs, out, 0)
    reqs, tot = make(n_cap)
    out = torch.empty(tot, dtype=torch.int64, device=dev)
    lat, capacity = run_set(reqs, out, 0)
    # alone vs mixed on a sample of the capacity run
    mismatches = 0
    for (a, an, b, bn, off) in reqs[::20]:
        alone = torch.empty(an + bn, dtype=torch.int64, device=dev)
        native.mul_device(a, an, b, bn, alone.data_ptr())
        native.stream_check()
        h1 = hashlib.sha256(alone.cpu().numpy().tobytes()).hexdigest()
        h2 = hashlib.sha256(out[off:off + an + bn].cpu().numpy().tobytes()).hexdigest()
        mismatches += h1 != h2
    del out
    loads = []
    launches0 = native.launch_count()
    for load in (0.1, 0.3, 0.5, 0.7, 0.9):
        reqs, tot = make(n_load)
        out = torch.empty(tot, dtype=torch.int64, device=dev)
        lat, rate = run_set(reqs, out, load * capacity)
        loads.append({"load": load, "offered_per_s": round(load * capacity, 1), "products_per_s": round(rate, 1),
                      "p50_ms": round(float(np.percentile(lat, 50)), 3),
                      "p99_ms": round(float(np.percentile(lat, 99)), 3)})
        del out
    st = srv.stats()
    srv.close()
    mid = [x for x in loads if x["load"] == 0.5][0]
    line = {
        "metric": "serving p99 latency ms at 50% load (Poisson arrivals)", "value": mid["p99_ms"], "unit": "ms",
        "n_gpus": 1, "steps": len(loads), "warmup": 1, "ms_per_step": None, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "an = bn = s, s log-uniform [256, 4194304] limbs, device-resident operands, "
                               "SplitMix64 seed 11", "hbm_budget_bytes": budget, "slots": 16,
                   "requests_capacity_run": n_cap, "requests_per_load": n_load},
        "capacity_products_per_s": round(capacity, 1),
        "loads": loads,
        "peak_in_flight": st.peak_in_flight, "peak_workspace_bytes": st.peak_bytes,
        "mismatches_alone_vs_mixed": int(mismatches), "checked": len(range(0, n_cap, 20)),
        "gpu_launches": native.launch_count() - launches0,
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


FFT_N, FFT_SEEDS = 3000, (5, 6)


def run_fft(args, emit=True):
    """The FP64 FFT band at 3000 x 3000 limbs (SplitMix64 seeds 5, 6): device
    time per product through prec_gpu_mul_fft's kernels (operands resident:
    timed by events around the host call's device part, reported by the
    library), the digit width, the maximum rounding distance of the product,
    and bit-exactness against the reference's mul_fft output (golden).  The
    CPU baseline is the oracle restatement of mul_fft on one core, a bounded
    sample of the same product.  Returns the line (printed when `emit`)."""
    import torch

    import oracle as O
    from preclib_gb300 import native, workloads
    native.init(0)
    a = workloads.operand(FFT_SEEDS[0], FFT_N)
    b = workloads.operand(FFT_SEEDS[1], FFT_N)
    ha = torch.from_numpy(a.view(np.int64)).pin_memory()
    hb = torch.from_numpy(b.view(np.int64)).pin_memory()
    ho = torch.empty(2 * FFT_N, dtype=torch.int64).pin_memory()
    pa, pb, po = (x.numpy().view(np.uint64) for x in (ha, hb, ho))
    L = native.lib()
    for _ in range(args.warmup):
        native.check(L.prec_gpu_mul_fft(native._p(pa), FFT_N, native._p(pb), FFT_N, native._p(po)))
    dev_ms, e2e, dist = [], [], 0.0
    launches0 = native.launch_count()
    with Clocks(0) as clk:
        for _ in range(args.steps):
            t = time.perf_counter()
            native.check(L.prec_gpu_mul_fft(native._p(pa), FFT_N, native._p(pb), FFT_N, native._p(po)))
            e2e.append(time.perf_counter() - t)
            st = native.last_stats()
            dev_ms.append(st.device_ms)
            dist = max(dist, st.fft_max_distance)
    launches = native.launch_count() - launches0
    with open(GOLDEN) as f:
        want = [r for r in json.load(f)["products"] if r["name"] == "cfg2_3000x3000_fft"][0]
    exact = hashlib.sha256(np.ascontiguousarray(po, dtype="<u8").tobytes()).hexdigest() == want["sha256"]
    value = statistics.median(dev_ms)
    line = {
        "metric": "3000x3000-limb FP64 FFT-band mul ms", "value": round(value, 4), "unit": "ms", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "3000 x 3000-limb uint64 product (SplitMix64 seeds 5,6) on the FP64 FFT band",
                   "digit_bits": native.fft_digit_bits(FFT_N, FFT_N), "transform_points": 1 << st.log2_n,
                   "l2": "inputs (48 KB) fit L2; device time from the library's events"},
        "max_rounding_distance": dist, "reference_max_rounding_distance": want.get("fft_max_err"),
        "bit_exact": bool(exact),
        "e2e": {"value": round(statistics.median(e2e) * 1e3, 4), "unit": "ms", "h2d_bytes_per_step": 16 * FFT_N,
                "d2h_bytes_per_step": 16 * FFT_N},
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    if not args.skip_cpu:
        cpu_ms, nprod = cpu_time(lambda: O.mul_fft(a, b), max_products=400, budget_s=2.0)
        line["cpu_baseline"] = {"value": round(cpu_ms, 4), "unit": "ms", "cores": 1, "kind": "port",
                                "sample": "%d single-threaded 3000 x 3000 products with the oracle restatement "
                                          "of mul_fft (8-bit digits), median" % nprod}
    if emit:
        print(json.dumps(line), flush=True)
    return line


PI_DIGITS = 100000000


def run_pi(args, emit=True):
    """pi to 10^8 decimal digits (the Chudnovsky program, preclib_gb300/pi):
    a step is one whole run of the program (binary splitting with one batch
    per tree level, square root, division, decimal conversion); the output
    file must be byte-identical to preclib's own pi program (SHA-256 of its
    10^8-digit output, tests/golden/pi.json).  Returns the line (printed
    when `emit`)."""
    from preclib_gb300 import build as B
    exe = os.path.join(B.LIBDIR, B.PI_EXE)
    with open(os.path.join(ROOT, "tests", "golden", "pi.json")) as f:
        want = {r["digits"]: r for r in json.load(f)["runs"]}[PI_DIGITS]
    steps = max(1, min(args.steps, 3))
    runs, exact, launches = [], True, None
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "pi.txt")
        for i in range(1 + steps):  # one untimed warm-up run
            t = time.perf_counter()
            r = subprocess.run([exe, str(PI_DIGITS), "--phases", "--file", out], capture_output=True, text=True)
            wall = time.perf_counter() - t
            if r.returncode != 0:
                raise SystemExit("pi program failed: " + r.stderr[-500:])
            data = open(out, "rb").read()
            exact = exact and len(data) == want["bytes"] and hashlib.sha256(data).hexdigest() == want["sha256"]
            ph = {}
            for line in r.stderr.splitlines():
                parts = line.split()
                if len(parts) >= 3 and parts[2] == "sec":  # "name seconds sec [(note)]"
                    ph[parts[0]] = float(parts[1])
                if len(parts) == 2 and parts[0] == "gpu_launches":
                    launches = int(parts[1])
            if i:
                runs.append((wall, ph))
    wall = statistics.median(w for w, _ in runs)
    phases = {k: round(statistics.median(p[k] for _, p in runs), 3) for k in runs[0][1]}
    line = {
        "metric": "pi 10^8 digits, whole program s", "value": round(wall, 3), "unit": "s", "n_gpus": 1,
        "steps": steps, "warmup": 1, "ms_per_step": round(wall * 1e3, 1), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "pi to 100,000,000 decimal digits by the Chudnovsky series",
                   "l2": "n/a (whole program)"},
        "phases_s": phases, "bit_exact": bool(exact),
        "e2e": {"value": round(wall, 3), "unit": "s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
        "gpu_launches": launches,
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


def ctypes_cast(addr, typ):
    import ctypes
    return ctypes.cast(ctypes.c_void_p(addr), typ)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="1m", choices=["1m", "batch", "serve", "pi", "fft"],
                    help="1m: the 1M x 1M product (default line); batch: 4096 uneven products; "
                         "serve: serving loop under Poisson arrivals; pi: pi to 10^8 digits; "
                         "fft: 3000 x 3000 limbs on the FP64 band")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU-baseline sample")
    ap.add_argument("--sustain", type=float, default=SUSTAIN_S,
                    help="seconds of back-to-back products after the timed steps, for the clock sampler "
                         "(0 for profiling runs)")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload: omit the other configurations' sub-results")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)  # at least three untimed warm-up steps
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "pi":
        run_pi(args)
    elif args.workload == "fft":
        run_fft(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
