"""Benchmark: gate bootstraps/sec on one GB300 (batched circuit layer).

Workload (one "step"): a circuit layer of 4096 independent gate bootstraps,
mixed NAND/AND/XOR/OR drawn uniformly from a seed, default 110-bit parameter
set (n=630, N=1024, k=1, l=3, Bgbit=7, t=8, basebit=2), one cloud key from
seed 0, input bits from seed 4.  Synthetic data: no dataset is involved.

  value  -- bootstraps/s of the split-FP32 form with inputs resident in HBM,
            timed with CUDA events around each step on the launching stream,
            L2 flushed (a 256 MB write) between steps outside the timed
            intervals; max over ranks.
  e2e    -- the same metric through the host-buffer C entry point
            (tfhe_gpu_bootsGates_host): pinned host ciphertexts in, results
            out, copies inside the timed region.
  roofline -- the dominant kernels (the blind-rotation launches of the
            step, k_blind_rotate_ring for the 4096-gate layer) timed alone
            with CUDA events: algorithmic FP work 162.6 MFLOP per bootstrap
            (FFT-form count) over their duration, against the FP32 FMA-pipe
            peak measured in the same run (tfhe_gpu_measure_fp32_peak).
  roofline_smem -- the same kernels against the resource that bounds them:
            shared-memory wavefronts per bootstrap (ncu counts of the same
            kernels) over their duration, against one wavefront per SM clock.
  cpu_baseline -- the CPU oracle (restated reference path) on the host's
            cores on a bounded sample; beside it (fast_cpu) the same gates
            through a CPU bootstrap with the upstream library's N/2-point
            transform (oracle/tfhe_cpu_fast.cpp).

`--impl reference` times the reference's CPU path instead (the oracle
restatement; the upstream library the reference links is not available) and
prints the same line with "impl": "reference".

Multi-GPU (torchrun): the layer's gate list is split into contiguous,
balanced shards, one per rank; each rank bootstraps its shard on its own GPU
with its own copy of the cloud key (the gates of a layer are independent),
and the output ciphertexts are gathered to rank 0 in layer order on the host
(a gloo group) -- the only exchange between layers.  value = the whole
layer's bootstraps / max rank time; "scaling": "strong".  --replicas runs
the whole layer on every rank instead ("scaling": "weak").
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOP_PER_BOOTSTRAP = 162.6e6      # FFT-form algorithmic count, default set
# DRAM bytes of the blind-rotation kernels, from full ncu captures of the
# ring and pair kernels: every launch reads the 61.9 MB key once, and each
# ciphertext moves 2.5 KB in and 4.5 KB out (66.5 MB measured for one
# 608-gate wave of the batched ring kernel, 66.2 MB by this rule).
DRAM_KEY_BYTES_PER_LAUNCH = 61.9e6
# Shared-memory wavefronts per bootstrap of the two batched ring kernels
# (the shared-memory wavefront count of a full ncu capture of each: 1.58 G
# for a 912-gate wave, 0.74 G for a 448-gate wave; the capture is
# summarised in profiles/blind_rotate_ring_pairs_batched_keyswitch_batch1360.md).
# The shared-memory pipe serves one wavefront per SM clock.
SMEM_WAVEFRONTS_PER_BOOTSTRAP = {
    "k_blind_rotate_ring<float,2,6,3,4,inline,nb2>": 1.58e9 / 912,
    "k_blind_rotate_ring<float,2,4,3,4,inline,nb3>": 0.74e9 / 448,
}
DRAM_IO_BYTES_PER_BOOTSTRAP = 2.52e3 + 4.5e3
BATCH = 4096
GATE_SET = (0, 1, 3, 2)           # NAND, AND, XOR, OR
GATE_NAMES = {0: "NAND", 1: "AND", 2: "OR", 3: "XOR"}
L2_FLUSH_BYTES = 256 << 20
SMS = 152
FP32_LANES_PER_SM = 128


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--form", default="split_fp32", choices=["split_fp32", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner")
    ap.add_argument("--split-bits", type=int, default=0,
                    help="split point s of the split-FP32 key (0 = the engine's choice)")
    ap.add_argument("--serve-forms", default="split_fp32,fp64",
                    help="transform forms the serving workload runs, in order")
    ap.add_argument("--no-graph", action="store_true", help="launch the gate pipeline eagerly")
    ap.add_argument("--workload", default="layer",
                    choices=["layer", "extprod", "stress", "failures", "serve"],
                    help="layer: 4096-gate circuit layer (default, the headline); extprod: 1024 "
                         "external products; stress: 65536 NAND on the n=500/l=2/Bgbit=10 set; "
                         "failures: 10^6 gates as chained layers, decryption checked; serve: "
                         "64 Poisson clients submitting circuits to the continuous-batching server")
    ap.add_argument("--clients", type=int, default=64)
    ap.add_argument("--requests", type=int, default=8, help="requests per client (serve)")
    ap.add_argument("--rate", type=float, default=8.0, help="requests/s per client (serve)")
    ap.add_argument("--pool-slots", type=int, default=131072,
                    help="ciphertext slots of the server's device pool (serve)")
    ap.add_argument("--groups", type=int, default=0,
                    help="ciphertexts per CTA of the split-FP32 blind rotation (0 = engine default)")
    ap.add_argument("--stress-gates", type=int, default=65536, help="NAND gates of the stress workload")
    ap.add_argument("--stress-forms", default="split_fp32,fp64", help="forms the stress workload runs")
    ap.add_argument("--layers", type=int, default=245,
                    help="chained 4096-gate layers of the failures workload (245: about 10^6 gates)")
    ap.add_argument("--replicas", action="store_true",
                    help="N > 1: every rank runs the whole layer (weak scaling) instead of a shard of it")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP64 / single-gate / CPU side measurements")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, world, device):
    """The maximum of a per-rank number over all ranks of the job (the job's
    time is its slowest rank's); the value itself on one rank."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, max_ms):
    """Whole-job units per second: every rank processed units_per_rank
    independent units (replicas), the job took the slowest rank's time."""
    return world * units_per_rank / (max_ms / 1000.0)


def layer_config(batch, world=1, replicas=False):
    """The workload's `config`, identical in both arms (the reference arm
    times a bounded sample of this workload and says so in its
    cpu_baseline.sample)."""
    if world <= 1:
        par = "one GPU"
    elif replicas:
        par = "replicas: the whole layer on each of %d GPUs" % world
    else:
        par = "layer split: contiguous shards over %d GPUs, host-side gather to rank 0" % world
    return {"workload": "batched circuit layer: %d independent gate bootstraps, mixed NAND/AND/XOR/OR "
                        "(seed 4), default 110-bit set (n=630, N=1024, k=1, l=3, Bgbit=7, t=8, basebit=2), "
                        "one cloud key (seed 0)" % batch,
            "batch": batch, "l2": "flushed (256 MB write) between timed steps", "parallelism": par}


def layer_shards(count, world):
    """Contiguous, balanced shards [lo, hi) of a layer's `count` gates over
    `world` ranks (sizes differ by at most one, in rank order)."""
    return [(r * count // world, (r + 1) * count // world) for r in range(world)]


def gather_layer(shard_out, count, world, rank, group=None):
    """Host-side gather of the ranks' output shards (int32 [hi - lo, n + 1]
    each) to rank 0 in layer order: the whole layer's outputs on rank 0,
    None on the other ranks.  Shards are padded to the largest size for the
    collective."""
    if world <= 1:
        return shard_out
    import torch
    import torch.distributed as dist
    shards = layer_shards(count, world)
    rows = max(hi - lo for lo, hi in shards)
    buf = torch.zeros((rows, shard_out.shape[1]), dtype=torch.int32)
    buf[:len(shard_out)] = torch.from_numpy(np.ascontiguousarray(shard_out, np.int32))
    parts = [torch.zeros_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, parts, dst=0, group=group)
    if rank != 0:
        return None
    return np.concatenate([parts[r][:hi - lo].numpy() for r, (lo, hi) in enumerate(shards)])


def make_inputs(pkg, P, lwe_key, batch, seed=4):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 2, batch)
    b = rng.integers(0, 2, batch)
    gates = np.array(GATE_SET, np.int32)[rng.integers(0, len(GATE_SET), batch)]
    pkg.set_seed([seed])
    ca = pkg.encrypt_bits(P, a, lwe_key)
    cb = pkg.encrypt_bits(P, b, lwe_key)
    return a, b, gates, ca, cb


class ClockSampler:
    """nvidia-smi samples of SM clock / throttle reasons during the timed
    region: entering starts nvidia-smi and waits (up to 3 s) for its first
    sample, so that the sampler is live when the timed work starts; the
    summary uses the samples taken after that one."""

    INTERVAL_MS = 100

    def __init__(self, index):
        self.index = index
        self.lines = []
        self.first = 0
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                 "-lms", str(self.INTERVAL_MS)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.005)
            self.first = len(self.lines)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[self.first:] or self.lines
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(seconds, batch_hint):
    """The oracle (restated reference path) on all host cores, bounded."""
    from oracle import pyoracle
    o = pyoracle.get()
    P = pyoracle.default_params()
    lwe, tlwe, ks, bk = o.gate_keyset(P, [0])
    bk_fft = o.bk_to_fft(P, bk)
    threads = o.max_threads()
    rng = np.random.default_rng(4)
    n = max(threads, 1) * 2
    a = rng.integers(0, 2, n)
    b = rng.integers(0, 2, n)
    gates = np.array(GATE_SET, np.int32)[rng.integers(0, len(GATE_SET), n)]
    want = np.array([pyoracle.GATE_FN[name](x, y) for name, x, y in
                     zip([GATE_NAMES[g] for g in gates], a, b)])
    o.set_seed([4])
    ca = o.encrypt_bits(P, a, lwe)
    cb = o.encrypt_bits(P, b, lwe)
    done = 0
    t0 = time.perf_counter()
    while True:
        o.boots_gate_batch(P, bk_fft, ks, gates, ca, cb, threads)
        done += n
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    # one core: the per-gate latency of the CPU path (a few seconds)
    one, t1 = 0, time.perf_counter()
    while True:
        o.boots_gate_batch(P, bk_fft, ks, gates[:1], ca[:1], cb[:1], 1)
        one += 1
        el1 = time.perf_counter() - t1
        if el1 >= min(4.0, seconds / 2):
            break
    return {"value": done / el, "unit": "bootstraps/s", "cores": threads, "kind": "port",
            "sample": "%d gate bootstraps (mixed NAND/AND/XOR/OR, default set) in %.1f s on %d threads"
                      % (done, el, threads),
            "single_core": {"bootstraps_per_s": one / el1, "gate_latency_ms": 1000.0 * el1 / one,
                            "sample": "%d gates one after another on 1 thread in %.1f s" % (one, el1)},
            "fast_cpu": cpu_fast_baseline(P, bk, ks, gates, ca, cb, want, threads, seconds / 2, o, lwe)}


def cpu_fast_baseline(P, bk, ks, gates, ca, cb, want, threads, seconds, o, lwe):
    """The same gates through the faster CPU bootstrap (N/2-point twisted
    transform, the upstream library's method) on all host cores and on one:
    the CPU figure without the reference's 2N-point transform.  Its
    decrypted bits are checked against the plaintext truth `want`."""
    from oracle import pyoracle
    fast = pyoracle.CpuFast(P, bk, ks)
    try:
        done, t0 = 0, time.perf_counter()
        while True:
            out = fast.boots_gates(gates, ca, cb, threads)
            done += len(gates)
            el = time.perf_counter() - t0
            if el >= seconds:
                break
        wrong = int((o.decrypt_bits(P, out, lwe) != want).sum())
        one, t1 = 0, time.perf_counter()
        while True:
            fast.boots_gates(gates[:1], ca[:1], cb[:1], 1)
            one += 1
            el1 = time.perf_counter() - t1
            if el1 >= min(3.0, seconds / 2):
                break
    finally:
        fast.close()
    return {"bootstraps_per_s": done / el, "cores": threads,
            "gate_latency_ms_one_core": 1000.0 * el1 / one, "wrong": wrong,
            "method": "N/2-point twisted complex transform in FP64 (the upstream TFHE library's method), "
                      "radix-2, split real/imaginary arrays, one gate per thread",
            "sample": "%d gates in %.1f s on %d threads; %d gates on 1 thread in %.1f s"
                      % (done, el, threads, one, el1)}


def run_reference(args, world, rank):
    """--impl reference: the reference's CPU path (restated) on host cores."""
    if world > 1 and rank != 0:
        return
    from oracle import pyoracle
    o = pyoracle.get()
    P = pyoracle.default_params()
    lwe, tlwe, ks, bk = o.gate_keyset(P, [0])
    bk_fft = o.bk_to_fft(P, bk)
    threads = o.max_threads()
    n = max(2 * threads, 8)  # bounded sample of the 4096-gate layer per step
    rng = np.random.default_rng(4)
    a = rng.integers(0, 2, n)
    b = rng.integers(0, 2, n)
    gates = np.array(GATE_SET, np.int32)[rng.integers(0, len(GATE_SET), n)]
    o.set_seed([4])
    ca = o.encrypt_bits(P, a, lwe)
    cb = o.encrypt_bits(P, b, lwe)
    for _ in range(args.warmup):
        o.boots_gate_batch(P, bk_fft, ks, gates, ca, cb, threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.boots_gate_batch(P, bk_fft, ks, gates, ca, cb, threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n * args.steps / total
    line = {
        "metric": "gate bootstraps/sec", "value": value, "unit": "bootstraps/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": layer_config(args.batch, world, getattr(args, "replicas", False)),
        "cpu_baseline": {"value": value, "unit": "bootstraps/s", "cores": threads, "kind": "port",
                         "sample": "each step a bounded sample of %d gates of the %d-gate layer (same gate "
                                   "mix, keys and inputs), %d steps, FP64 2N-point transform restatement "
                                   "of the reference path on %d host threads"
                                   % (n, args.batch, args.steps, threads)},
        "e2e": {"value": value, "unit": "bootstraps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# side workloads (one JSON line each; the default run is the layer above)
# ---------------------------------------------------------------------------
def _engine_setup(P, seed, local, forms=("fp64", "split_fp32")):
    import torch
    import __graft_entry__ as ge
    torch.cuda.set_device(local)
    ge.build()
    pkg = ge.load_package()
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, seed)
    eng = pkg.Engine(P, device=local)
    eng.upload_bootstrapping_key(bk, forms=forms)
    eng.upload_keyswitch_key(ks)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    return torch, pkg, eng, (lwe, tlwe, ks, bk), stream


def _time_steps(torch, stream, fn, steps, warmup, flush=None):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ms = []
    for s in range(steps):
        if flush is not None:
            flush.fill_(s)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return ms


def workload_extprod(args, world, rank, local):
    """1024 independent TGSW x TRLWE products (tGswFFTExternMulToTLwe):
    TRLWE coefficients uniform int32 (numpy seed 2), TGSW = encryption of X^e,
    e uniform in [0, 2N) (seed 3); the split-FP32 result is compared with the
    FP64 form's.
    Roofline: HBM (each product reads its own 98,304-byte TGSW)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    P = pkg.default_params()
    torch, pkg, eng, keys, stream = _engine_setup(P, [0], local, forms=("fp64",))
    lwe, tlwe, ks, bk = keys
    count = 1024
    rng = np.random.default_rng(2)
    acc = rng.integers(-2 ** 31, 2 ** 31, (count, 2 * P.N)).astype(np.int32)
    es = np.random.default_rng(3).integers(0, 2 * P.N, count)
    # TGSW(X^e): the bootstrapping key's samples BK_i with s_i = 1 are TGSW
    # encryptions of 1 under the TLWE key; every row rotated by X^e
    bkr = bk.reshape(P.n, P.kpl, 2, P.N)
    base = [bkr[i] for i in np.nonzero(lwe == 1)[0][:16]]

    def mul_by_xai(poly, e):
        e %= 2 * P.N
        sign = 1
        if e >= P.N:
            e -= P.N
            sign = -1
        r = np.empty_like(poly)
        r[e:] = poly[:P.N - e]
        r[:e] = -poly[P.N - e:]
        return (sign * r.astype(np.int64)).astype(np.int32)

    gsw = np.empty((count, P.kpl * 2 * P.N), np.int32)
    for c in range(count):
        g = base[c % len(base)]
        gsw[c] = np.stack([[mul_by_xai(g[p, j], int(es[c])) for j in range(2)]
                           for p in range(P.kpl)]).reshape(-1)
    sp = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    d_gsw_time = torch.from_numpy(gsw).cuda()
    d_acc0 = torch.from_numpy(acc).cuda()
    res, got = {}, {}
    for form in ("fp64", "split_fp32"):
        nb = eng.tgsw_fft_bytes(form)
        d_g = torch.empty(count * nb, dtype=torch.uint8, device="cuda")
        eng.tgsw_to_fft(d_gsw_time, d_g, count, form, stream=sp)
        d_acc = d_acc0.clone()
        # the product's work does not depend on the values: time it in place
        ms = _time_steps(torch, stream,
                         lambda: eng.tGswFFTExternMulToTLwe(d_acc, d_g, count, form, stream=sp),
                         args.steps, args.warmup, flush)
        kms = statistics.median(ms)
        d_acc.copy_(d_acc0)
        eng.tGswFFTExternMulToTLwe(d_acc, d_g, count, form, stream=sp)
        torch.cuda.synchronize()
        got[form] = d_acc.cpu().numpy().astype(np.int64)
        bytes_per = nb + 2 * 2 * P.N * 4
        res[form] = {"products_per_s": count / (kms / 1000.0), "kernel_ms": kms,
                     "hbm_gbs": count * bytes_per / (kms / 1000.0) / 1e9}
    # split-FP32 against the FP64 form (itself within 2 units of the exact
    # int64 product: tests/test_gpu_primitives.py)
    d = (got["split_fp32"] - got["fp64"] + 2 ** 31) % 2 ** 32 - 2 ** 31
    res["split_fp32"]["max_abs_diff_vs_fp64_units"] = int(np.abs(d).max())
    peak = _measured_peak("hbm_gbs")
    f = res["split_fp32"]
    line = {"metric": "external products/sec", "value": f["products_per_s"], "unit": "products/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": f["kernel_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "1024 independent TGSW x TRLWE external products, N=1024, k=1, l=3, "
                                   "Bgbit=7; TRLWE uniform int32 (seed 2), TGSW = encryption of X^e "
                                   "(seed 3); L2 flushed between steps", "batch": count},
            "forms": res,
            "roofline": {"bound": "hbm", "achieved": f["hbm_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": f["hbm_gbs"] / peak if peak else None, "traffic": None,
                         "algorithmic_bytes_per_unit": eng.tgsw_fft_bytes("split_fp32") + 16384,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs"}}
    print(json.dumps(line), flush=True)


def _measured_peak(key):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)[key])
    except (OSError, KeyError, ValueError):
        return 6800.0 if key == "hbm_gbs" else None


def run_stress(torch, pkg, local, split_bits=0, total=65536, batch=8192, forms=("split_fp32", "fp64"),
               chunk=262144):
    """`total` NAND bootstraps on the alternative set n=500, l=2, Bgbit=10,
    LWE 2^-15, TRLWE 2^-24 (keys seed 0, inputs seed 4), in batches of
    `batch`, per form: throughput, decryption failures and the output phase
    error against the ideal +-1/8.  Inputs are encrypted, run and checked
    `chunk` gates at a time so that large counts fit in host memory; only
    the GPU work is timed.  (Parity of this set against the oracle and the
    exact int64 bootstrap is in the GPU tests.)"""
    P = pkg.stress_params()
    P.split_bits = split_bits
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [0])
    eng = pkg.Engine(P, device=local)
    try:
        eng.upload_bootstrapping_key(bk, forms=forms)
        eng.upload_keyswitch_key(ks)
        stream = torch.cuda.current_stream()
        sp = stream.cuda_stream
        rng = np.random.default_rng(4)
        a = rng.integers(0, 2, total)
        b = rng.integers(0, 2, total)
        truth = 1 - (a & b)
        chunk = min(chunk, total)
        d_ca = torch.empty((chunk, P.n + 1), dtype=torch.int32, device="cuda")
        d_cb = torch.empty_like(d_ca)
        d_out = torch.empty_like(d_ca)
        mu = 2 ** 29
        res = {"gates": total, "split_bits": eng.params.split_bits}
        for form in forms:
            pkg.set_seed([4])
            ms_total = 0.0
            wrong = []
            err_max = err_sum = sq_sum = lin_sum = 0.0
            for c0 in range(0, total, chunk):
                m = min(chunk, total - c0)
                d_ca[:m].copy_(torch.from_numpy(pkg.encrypt_bits(P, a[c0:c0 + m], lwe)))
                d_cb[:m].copy_(torch.from_numpy(pkg.encrypt_bits(P, b[c0:c0 + m], lwe)))

                def run_chunk():
                    for s0 in range(0, m, batch):
                        n_ = min(batch, m - s0)
                        eng.bootsGate("NAND", d_out[s0:s0 + n_], d_ca[s0:s0 + n_], d_cb[s0:s0 + n_],
                                      n_, form, stream=sp)
                ms_total += _time_steps(torch, stream, run_chunk, 1, 1 if c0 == 0 else 0)[0]
                out = d_out[:m].cpu().numpy()
                t = truth[c0:c0 + m]
                bits = pkg.decrypt_bits(P, out, lwe)
                wrong.extend(int(c0 + i) for i in np.nonzero(bits != t)[0])
                ph = pkg.phases(out, lwe).astype(np.int64)
                err = np.abs(np.abs(ph) - mu) / 2.0 ** 32
                signed = ((ph - np.where(t == 1, mu, -mu) + 2 ** 31) % 2 ** 32 - 2 ** 31) / 2.0 ** 32
                err_max = max(err_max, float(err.max()))
                err_sum += float(err.sum())
                lin_sum += float(signed.sum())
                sq_sum += float((signed * signed).sum())
            mean = lin_sum / total
            res[form] = {"bootstraps_per_s": total / (ms_total / 1000.0), "failures": len(wrong),
                         "failed_gates": wrong[:16],
                         "phase_err_max_turn": err_max,
                         "phase_err_sigma_turn": float(np.sqrt(max(sq_sum / total - mean * mean, 0.0))),
                         "phase_err_mean_turn": err_sum / total}
    finally:
        eng.close()
    return res


def workload_stress(args, world, rank, local):
    """Precision stress: 65,536 NAND on the n=500/l=2/Bgbit=10 set, split-FP32
    vs FP64 (one JSON line)."""
    import __graft_entry__ as ge
    import torch
    torch.cuda.set_device(local)
    ge.build()
    pkg = ge.load_package()
    torch.cuda.set_stream(torch.cuda.Stream())
    forms = tuple(args.stress_forms.split(","))
    res = run_stress(torch, pkg, local, args.split_bits, total=args.stress_gates, forms=forms)
    f = res[forms[0]]
    total = res["gates"]
    line = {"metric": "gate bootstraps/sec", "value": f["bootstraps_per_s"], "unit": "bootstraps/s",
            "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": total / f["bootstraps_per_s"] * 1000,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "precision stress: %d NAND bootstraps, n=500, N=1024, k=1, l=2, "
                                   "Bgbit=10, ks t=8 basebit=2, LWE 2^-15, TRLWE 2^-24 (keys seed 0, "
                                   "inputs seed 4)" % total, "batch": 8192, "split_bits": res["split_bits"]},
            "dtype_note": "value = the %s form" % forms[0],
            "forms": {k: v for k, v in res.items() if k in ("split_fp32", "fp64")}}
    print(json.dumps(line), flush=True)


GATE_FNS = [lambda x, y: 1 - (x & y), lambda x, y: x & y, lambda x, y: x | y, lambda x, y: x ^ y,
            lambda x, y: 1 - (x ^ y), lambda x, y: 1 - (x | y), lambda x, y: (1 - x) & y,
            lambda x, y: x & (1 - y), lambda x, y: (1 - x) | y, lambda x, y: x | (1 - y)]


def run_failures(torch, pkg, eng, P, lwe, width=4096, layers=245, form="split_fp32"):
    """width x layers gate bootstraps as chained layers of random gates (all
    10 gate types, random wiring, seed 7): each layer's inputs are outputs
    of the previous layer; every output decrypted and compared with the
    plaintext evaluation of the same circuit."""
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    err_sum = err_sq = 0.0
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 2, width)
    pkg.set_seed([7])
    cur = torch.from_numpy(pkg.encrypt_bits(P, bits, lwe)).cuda()
    out = torch.empty_like(cur)
    failures = 0
    worst = 0.0
    t0 = time.perf_counter()
    gpu_ms = 0.0
    for layer in range(layers):
        ia = rng.integers(0, width, width)
        ib = rng.integers(0, width, width)
        g = rng.integers(0, 10, width).astype(np.int32)
        ca = cur[torch.from_numpy(ia).cuda()].contiguous()
        cb = cur[torch.from_numpy(ib).cuda()].contiguous()
        d_g = torch.from_numpy(g).cuda()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.bootsGates(d_g, out, ca, cb, width, form, stream=sp)
        e1.record(stream)
        torch.cuda.synchronize()
        gpu_ms += e0.elapsed_time(e1)
        nb = np.array([GATE_FNS[gi](bits[x], bits[y]) for gi, x, y in zip(g, ia, ib)])
        host = out.cpu().numpy()
        got = pkg.decrypt_bits(P, host, lwe)
        failures += int((got != nb).sum())
        ph = pkg.phases(host, lwe).astype(np.int64)
        worst = max(worst, float(np.abs(np.abs(ph) - 2 ** 29).max() / 2.0 ** 32))
        e = ((ph - np.where(nb == 1, 2 ** 29, -(2 ** 29)) + 2 ** 31) % 2 ** 32 - 2 ** 31) / 2.0 ** 32
        err_sum += float(e.sum())
        err_sq += float((e * e).sum())
        bits = nb  # continue from the plaintext truth; the ciphertexts carry on
        cur, out = out, cur
    total = width * layers
    return {"gates": total, "failures": failures, "bootstraps_per_s": total / (gpu_ms / 1000.0),
            "worst_phase_error_turn": worst,
            "phase_error_sigma_turn": (err_sq / total - (err_sum / total) ** 2) ** 0.5,
            "form": form, "split_bits": eng.params.split_bits, "gpu_ms_per_layer": gpu_ms / layers,
            "wall_s": time.perf_counter() - t0,
            "workload": "%d chained layers of %d random gates (all 10 gate types, random wiring, seed 7), "
                        "default set, %s" % (layers, width, form)}


def workload_failures(args, world, rank, local):
    """10^6 gate bootstraps (default set, split-FP32) as 245 chained layers of
    4096 random gates (--layers for more), decryption checked (one JSON
    line)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    P = pkg.default_params()
    P.split_bits = args.split_bits
    torch, pkg, eng, keys, stream = _engine_setup(P, [0], local, forms=("split_fp32",))
    r = run_failures(torch, pkg, eng, P, keys[0], layers=args.layers)
    line = {"metric": "decryption failures", "value": r["failures"], "unit": "failures",
            "gates": r["gates"], "n_gpus": 1, "steps": args.layers, "warmup": 0,
            "ms_per_step": r["gpu_ms_per_layer"], "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "%d gate bootstraps: " % r["gates"] + r["workload"]},
            "bootstraps_per_s": r["bootstraps_per_s"],
            "worst_phase_error_turn": r["worst_phase_error_turn"],
            "phase_error_sigma_turn": r["phase_error_sigma_turn"],
            "split_bits": r["split_bits"], "wall_s": r["wall_s"]}
    print(json.dumps(line), flush=True)
    eng.close()


def serving_requests(pkg, P, lwe, clients, requests, rate, seed=5):
    """Poisson request streams: `clients` clients, `rate` requests/s each;
    each request a random circuit (32-bit ripple-carry adder, 16-bit
    comparator, 8-bit multiplexer) with random operands."""
    import importlib
    circuits = importlib.import_module("tfhe_gb300.circuits")
    rng = np.random.default_rng(seed)
    kinds = [("adder", circuits.ripple_carry_adder(32)), ("cmp", circuits.comparator(16)),
             ("mux", circuits.multiplexer(8))]
    reqs = []
    pkg.set_seed([seed])
    for cl in range(clients):
        t = 0.0
        for _ in range(requests):
            t += rng.exponential(1.0 / rate)
            k = int(rng.integers(0, 3))
            name, (gates, ni, outs) = kinds[k]
            bits = rng.integers(0, 2, ni).astype(np.int32)
            reqs.append({"t": t, "kind": name, "gates": gates, "ni": ni, "outs": outs,
                         "ct": pkg.encrypt_bits(P, bits, lwe),
                         "want": circuits.evaluate(gates, bits, outs)})
    reqs.sort(key=lambda r: r["t"])
    total_boots = sum(circuits.bootstraps(r["gates"]) for r in reqs)
    return reqs, total_boots


def run_serving(pkg, eng, P, lwe, reqs, total_boots, form, pool_slots=131072, max_batch=4096):
    """Replay the request streams against the continuous-batching server:
    requests are submitted at their arrival times, the server steps while
    work is pending, every output is decrypted and checked.  Per-gate
    latency = gate ready -> bootstrapped; request latency = arrival ->
    outputs back on the host."""
    srv = pkg.Server(eng, pool_slots=pool_slots, max_batch=max_batch, form=form)
    t0 = time.perf_counter()
    nxt = 0
    pending = {}
    lat = {"adder": [], "cmp": [], "mux": []}
    wrong = 0
    while nxt < len(reqs) or pending:
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt]["t"] <= now:
            r = reqs[nxt]
            pending[srv.submit(r["gates"], r["ni"], r["ct"], r["outs"])] = r
            nxt += 1
        ran = srv.step()
        for rid in list(pending):
            got = srv.poll(rid)
            if got is not None:
                r = pending.pop(rid)
                lat[r["kind"]].append(time.perf_counter() - t0 - r["t"])  # from arrival
                wrong += int((pkg.decrypt_bits(P, got[0], lwe) != r["want"]).any())
        if ran == 0 and not pending and nxt < len(reqs):
            time.sleep(max(0.0, reqs[nxt]["t"] - (time.perf_counter() - t0)))
    makespan = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    gl = np.array(st["gate_latency_s"]) * 1000
    allr = np.concatenate([np.array(v) for v in lat.values() if v]) * 1000
    return {
        "bootstraps_per_s": total_boots / makespan, "makespan_s": makespan,
        "busy_s": st["busy_s"], "bootstraps_per_busy_s": total_boots / st["busy_s"],
        "bootstraps": total_boots,
        "gate_latency_ms": {"p50": float(np.percentile(gl, 50)), "p99": float(np.percentile(gl, 99))},
        "request_latency_ms": {"p50": float(np.percentile(allr, 50)), "p99": float(np.percentile(allr, 99))},
        "request_latency_ms_by_circuit": {k: {"p50": float(np.percentile(np.array(v) * 1000, 50)),
                                              "p99": float(np.percentile(np.array(v) * 1000, 99)),
                                              "n": len(v)} for k, v in lat.items() if v},
        "requests": len(reqs), "wrong_requests": wrong}


def workload_serve(args, world, rank, local):
    """Serving: `clients` simulated clients with Poisson arrivals submitting
    circuits to the continuous-batching server under one cloud key (one
    JSON line)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    P = pkg.default_params()
    torch, pkg, eng, keys, stream = _engine_setup(P, [0], local)
    lwe = keys[0]
    reqs, total_boots = serving_requests(pkg, P, lwe, args.clients, args.requests, args.rate)
    result = {}
    for form in args.serve_forms.split(","):
        result[form] = run_serving(pkg, eng, P, lwe, reqs, total_boots, form, pool_slots=args.pool_slots)
    first = args.serve_forms.split(",")[0]
    f = result[first]
    line = {"metric": "gate bootstraps/sec (serving)", "value": f["bootstraps_per_s"],
            "unit": "bootstraps/s", "n_gpus": 1, "steps": len(reqs), "warmup": 0,
            "ms_per_step": f["makespan_s"] * 1000 / len(reqs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if first == "split_fp32" else "f64",
            "data": "synthetic",
            "config": {"workload": "serving: %d clients x %d requests, Poisson arrivals %.1f req/s per "
                                   "client (seed 5); circuits uniform over 32-bit ripple-carry adder, "
                                   "16-bit comparator, 8-bit multiplexer; one cloud key; value = %s form; "
                                   "%d bootstraps in total" % (args.clients, args.requests, args.rate, first,
                                                               total_boots)},
            "latency_ms": {"gate_p50": f["gate_latency_ms"]["p50"], "gate_p99": f["gate_latency_ms"]["p99"],
                           "request_p50": f["request_latency_ms"]["p50"],
                           "request_p99": f["request_latency_ms"]["p99"]},
            "forms": result}
    print(json.dumps(line), flush=True)
    eng.close()


WORKLOADS = {"extprod": workload_extprod, "stress": workload_stress, "failures": workload_failures,
             "serve": workload_serve}


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload != "layer":
        WORKLOADS[args.workload](args, world, rank, local)
        return
    import torch
    import __graft_entry__ as ge

    torch.cuda.set_device(local)
    host_group = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        host_group = dist.new_group(backend="gloo")  # the host-side ciphertext gather
    # one rank compiles (an up-to-date tree is left as it is); the others
    # wait, so no two ranks write the same build files
    if rank == 0:
        ge.build()
    if world > 1:
        torch.distributed.barrier(group=host_group)
    if rank != 0:
        ge.build()
    pkg = ge.load_package()
    P = pkg.default_params()
    P.split_bits = args.split_bits
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [0])
    eng = pkg.Engine(P, device=local)
    eng.upload_bootstrapping_key(bk, forms=("fp64", "split_fp32"))
    eng.upload_keyswitch_key(ks)
    split = world > 1 and not args.replicas
    lo, hi = layer_shards(args.batch, world)[rank] if split else (0, args.batch)
    batch = hi - lo  # this rank's gates
    layer_units = args.batch if split else world * args.batch  # bootstraps of the job per step
    tuned = None
    if args.groups:
        eng.set_groups_per_cta(args.form, args.groups)
    elif not args.no_tune:
        # project autotuner: time every launch shape on this batch size
        shape, br_ms = eng.autotune(args.form, batch)
        tuned = {"shape": shape, "blind_rotate_ms": br_ms}
    a_all, b_all, gates_all, ca_all, cb_all = make_inputs(pkg, P, lwe, args.batch)
    a, b, gates, ca, cb = (x[lo:hi] for x in (a_all, b_all, gates_all, ca_all, cb_all))
    dev = torch.device("cuda", local)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    # a non-default stream: the engine maps a NULL stream to its own stream,
    # so events must be recorded on the stream the engine launches on
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp, "need a non-null stream handle"
    d_ca = torch.from_numpy(ca).to(dev)
    d_cb = torch.from_numpy(cb).to(dev)
    d_g = torch.from_numpy(gates).to(dev)
    d_out = torch.empty_like(d_ca)
    torch.cuda.synchronize()

    # the whole gate pipeline of the batch as one CUDA graph (its creation
    # runs the batch once); the FP64 side figures run eagerly
    graph = None if args.no_graph else eng.graph_gates(d_g, d_out, d_ca, d_cb, batch, args.form)

    def step(form):
        if graph is not None and form == args.form:
            graph.launch(stream=sp)
        else:
            eng.bootsGates(d_g, d_out, d_ca, d_cb, batch, form, stream=sp)

    # warm-up (also sizes the engine's scratch)
    for _ in range(args.warmup):
        step(args.form)
    torch.cuda.synchronize()

    def timed(form, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for s in range(steps):
            flush.fill_(s)  # evict L2 between steps (outside the timed interval)
            evs[s][0].record(stream)
            step(form)
            evs[s][1].record(stream)
        torch.cuda.synchronize()
        return [e0.elapsed_time(e1) for e0, e1 in evs]

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = timed(args.form, args.steps)
    torch.cuda.synchronize()
    total_ms = max_over_ranks(sum(ms), world, dev)
    value = layer_units * args.steps / (total_ms / 1000.0)
    truth = {0: lambda x, y: 1 - (x & y), 1: lambda x, y: x & y, 2: lambda x, y: x | y,
             3: lambda x, y: x ^ y}
    d_out.zero_()
    step(args.form)
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    if split:
        out = gather_layer(out, args.batch, world, rank, host_group)
    ok = None
    if out is not None:  # rank 0 checks the whole layer it holds
        ga, aa, ba = (gates_all, a_all, b_all) if split else (gates, a, b)
        ok = bool((pkg.decrypt_bits(P, out, lwe)
                   == np.array([truth[int(g)](x, y) for g, x, y in zip(ga, aa, ba)])).all())

    # e2e through the host-buffer entry point (pinned host buffers)
    h_ca = torch.from_numpy(ca).pin_memory()
    h_cb = torch.from_numpy(cb).pin_memory()
    h_g = torch.from_numpy(gates).pin_memory()
    h_out = torch.empty_like(h_ca).pin_memory()
    lib = pkg.lib()
    e2e_ms = []
    for s in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = lib.tfhe_gpu_bootsGates_host(
            eng.ctx, pkg.ctypes.cast(h_g.data_ptr(), pkg.I32P), 0,
            pkg.ctypes.cast(h_out.data_ptr(), pkg.I32P), pkg.ctypes.cast(h_ca.data_ptr(), pkg.I32P),
            pkg.ctypes.cast(h_cb.data_ptr(), pkg.I32P), batch, pkg.FORMS[args.form])
        if st:
            raise RuntimeError("bootsGates_host failed: %d" % st)
        if split:  # the between-layer exchange: outputs to rank 0 in layer order
            gather_layer(h_out.numpy(), args.batch, world, rank, host_group)
        if s >= args.warmup:
            e2e_ms.append(1000 * (time.perf_counter() - t0))
    e2e_total = max_over_ranks(sum(e2e_ms), world, dev)
    e2e_value = layer_units * args.steps / (e2e_total / 1000.0)
    lwe_bytes = batch * (P.n + 1) * 4

    # dominant kernels alone: blind rotation + extraction on resident inputs
    u = torch.empty((batch, P.k * P.N + 1), dtype=torch.int32, device=dev)
    kms = []
    for s in range(max(3, args.steps)):
        flush.fill_(s)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.tfhe_bootstrap_woKS_FFT(u, d_ca, 2 ** 29, batch, args.form, stream=sp)
        e1.record(stream)
        torch.cuda.synchronize()
        kms.append(e0.elapsed_time(e1))
    k_ms = statistics.median(kms)
    br_launches = len(blind_rotate_kernels(args.form, eng.get_groups_per_cta(args.form), batch))
    achieved = FLOP_PER_BOOTSTRAP * batch / (k_ms / 1000.0) / 1e12
    clocks = clk.summary()
    sm_max = clocks.get("sm_max_mhz") or 2070.0
    nominal_peak = SMS * FP32_LANES_PER_SM * 2 * sm_max * 1e6 / 1e12
    # the FP32 FMA-pipe peak measured on this GPU now (packed FMA chains on
    # every SM; MEASURED_PEAKS.json has no FP32 figure)
    with ClockSampler(local) as clk_peak:
        peak, peak_ms = pkg.measure_fp32_peak(local)

    extras = {}
    if not args.no_extras and rank == 0:
        # plain FP64 form, same batch
        for _ in range(1):
            step("fp64")
        torch.cuda.synchronize()
        f64 = timed("fp64", 2)
        extras["fp64_batched_bootstraps_per_s"] = batch * 2 / (sum(f64) / 1000.0)
        # the plain FP64 form's roofline: the same algorithmic work over the
        # FP64 FMA-pipe peak measured now
        f64_peak, f64_peak_ms = pkg.measure_fp64_peak(local)
        f64_achieved = FLOP_PER_BOOTSTRAP * extras["fp64_batched_bootstraps_per_s"] / 1e12
        extras["fp64_roofline"] = {
            "bound": "fp64", "achieved": f64_achieved, "peak": f64_peak, "unit": "TFLOP/s",
            "frac": f64_achieved / f64_peak,
            "note": "whole FP64 gate step (blind rotation + key switch) per 162.6 MFLOP bootstrap; peak "
                    "measured in this run by tfhe_gpu_measure_fp64_peak (independent FP64 FMA chains, "
                    "%.1f ms)" % f64_peak_ms}
        # plain FP64 single-gate form (one gate per call), the >=10x denominator
        one_ms = []
        for s in range(4):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.bootsGates(d_g, d_out, d_ca, d_cb, 1, "fp64", stream=sp)
            e1.record(stream)
            torch.cuda.synchronize()
            one_ms.append(e0.elapsed_time(e1))
        one = statistics.median(one_ms[1:])
        # a single gate on the automatic shape (the spread kernel over a
        # two-SM cluster), whatever shape the autotuner kept for the batch
        saved_shape = eng.get_groups_per_cta("split_fp32")
        eng.set_groups_per_cta("split_fp32", 0)
        one32 = []
        for s in range(4):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.bootsGates(d_g, d_out, d_ca, d_cb, 1, "split_fp32", stream=sp)
            e1.record(stream)
            torch.cuda.synchronize()
            one32.append(e0.elapsed_time(e1))
        # its blind rotation alone: the whole key streamed once for one gate
        u1 = torch.empty((1, P.k * P.N + 1), dtype=torch.int32, device=dev)
        br1 = []
        for s in range(4):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.tfhe_bootstrap_woKS_FFT(u1, d_ca[:1], 2 ** 29, 1, "split_fp32", stream=sp)
            e1.record(stream)
            torch.cuda.synchronize()
            br1.append(e0.elapsed_time(e1))
        br1_ms = statistics.median(br1[1:])
        eng.set_groups_per_cta("split_fp32", saved_shape)
        extras["split_fp32_single_gate_ms"] = statistics.median(one32[1:])
        key_bytes = 61931520.0
        extras["single_gate_key_stream"] = {
            "blind_rotate_ms": br1_ms, "key_bytes": key_bytes,
            "achieved_gbs": key_bytes / (br1_ms / 1000.0) / 1e9,
            "hbm_floor_us": key_bytes / (_measured_peak("hbm_gbs") * 1e9) * 1e6,
            "hbm_frac": key_bytes / (br1_ms / 1000.0) / 1e9 / _measured_peak("hbm_gbs"),
            "note": "batch 1: the 61.9 MB key streamed once through a chain of n dependent steps; "
                    "latency-bound, not bandwidth-bound"}
        extras["fp64_single_gate_ms"] = one
        extras["fp64_single_gate_bootstraps_per_s"] = 1000.0 / one
        extras["speedup_vs_fp64_single_gate"] = value / world / (1000.0 / one)
        # key generation: host arithmetic vs the TGSW products on the GPU
        # (same random values, same keys)
        t0 = time.perf_counter()
        host_keys = pkg.gate_keyset(P, [11])
        t_host = time.perf_counter() - t0
        kg = pkg.Engine(P, device=local)
        t0 = time.perf_counter()
        gpu_keys = kg.gate_keyset([11], forms=("split_fp32",))
        torch.cuda.synchronize()
        t_gpu = time.perf_counter() - t0
        kg.close()
        extras["keygen_s"] = {"host": t_host, "gpu_arithmetic_with_upload": t_gpu,
                              "identical": all(bool((x == y).all()) for x, y in zip(host_keys, gpu_keys))}
        extras.update(side_paths(pkg, torch, eng, P, (lwe, tlwe, ks, bk), d_ca, d_cb, batch, stream, sp))
        # the hard targets measured in the same run: decryption failures over
        # 10^6 chained gates, the stress set's failure rate and noise in both
        # forms, and serving latency under Poisson load
        extras["failures"] = run_failures(torch, pkg, eng, P, lwe)
        reqs, boots = serving_requests(pkg, P, lwe, args.clients, args.requests, args.rate)
        extras["serving"] = run_serving(pkg, eng, P, lwe, reqs, boots, "split_fp32")
        extras["serving"]["workload"] = ("%d clients x %d requests, Poisson %.1f req/s per client (seed 5), "
                                         "32-bit adders, 16-bit comparators, 8-bit multiplexers, split-FP32"
                                         % (args.clients, args.requests, args.rate))
        # saturating load: arrivals above the engine's capacity, so the
        # queue builds up and admission and batching bind
        reqs, boots = serving_requests(pkg, P, lwe, 64, 32, 50.0, seed=6)
        sat = run_serving(pkg, eng, P, lwe, reqs, boots, "split_fp32", pool_slots=1 << 20)
        sat["workload"] = ("64 clients x 32 requests, Poisson 50 req/s per client (seed 6): offered "
                           "%.0f bootstraps/s, above capacity; pool of 2^20 ciphertext slots, split-FP32"
                           % (boots / max(r["t"] for r in reqs)))
        sat["fraction_of_layer_engine"] = sat["bootstraps_per_s"] / value
        extras["serving_saturated"] = sat
        extras["stress"] = run_stress(torch, pkg, local, args.split_bits)
        cpu = cpu_baseline(args.cpu_seconds, batch)
    else:
        cpu = None

    if rank == 0:
        p50 = statistics.median(ms)
        p99 = float(np.percentile(ms, 99))
        line = {
            "metric": "gate bootstraps/sec", "value": value, "unit": "bootstraps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "strong" if split else "weak",
            "vs_baseline": None, "dtype": "f32" if args.form == "split_fp32" else "f64",
            "data": "synthetic",
            "config": layer_config(args.batch, world, args.replicas),
            "engine": {"form": args.form, "split_bits": eng.params.split_bits, "gates_per_rank": batch,
                       "groups_per_cta": eng.get_groups_per_cta(args.form),
                       "autotune": tuned, "cuda_graph": graph is not None},
            "latency_ms": {"p50": p50, "p99": p99,
                           "note": "per-gate latency = completion time of its batch"},
            "decrypt_ok": ok,
            "e2e": {"value": e2e_value, "unit": "bootstraps/s",
                    "h2d_bytes_per_step": 2 * lwe_bytes + batch * 4, "d2h_bytes_per_step": lwe_bytes},
            # eager: combine + per blind-rotation launch one key-switch launch
            # (a split blind rotation has its key switch split the same way)
            "gpu_launches": (graph.kernels if graph is not None else 1 + 2 * br_launches) * args.steps,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "traffic": br_launches * DRAM_KEY_BYTES_PER_LAUNCH + batch * DRAM_IO_BYTES_PER_BOOTSTRAP,
                         "traffic_note": "DRAM bytes of the blind-rotation launches of one step, scaled from "
                                         "ncu captures of the same kernels (1360 gates): key once per "
                                         "launch + per-ciphertext I/O",
                         "kernel": " + ".join(blind_rotate_kernels(args.form, eng.get_groups_per_cta(args.form),
                                                                   batch)) + " (blind rotation + extraction)",
                         "kernel_ms": k_ms,
                         "peak_source": "measured in this run: tfhe_gpu_measure_fp32_peak (independent packed "
                                        "FP32 FMA chains on every SM, CUDA events, %.1f ms; SM clock %s MHz); "
                                        "MEASURED_PEAKS.json has no FP32 figure" % (peak_ms,
                                                                                     clk_peak.summary().get("sm_mhz")),
                         "nominal_peak": nominal_peak,
                         "frac_of_nominal": achieved / nominal_peak},
            "roofline_smem": smem_roofline(blind_rotate_kernels(args.form, eng.get_groups_per_cta(args.form),
                                                                batch), batch, k_ms, clocks),
            "clocks": clocks,
        }
        line.update(extras)
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if graph is not None:
        graph.close()
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def side_paths(pkg, torch, eng, P, keys, d_ca, d_cb, batch, stream, sp):
    """Throughput of the paths either side of the gate bootstrap, on the same
    batch: bootsMUX (two bootstraps and one key switch per output), the
    programmable bootstrap with a lookup table, and the cloud-key file
    (write, then read straight into a fresh context's device keys)."""
    import tempfile
    lwe, tlwe, ks, bk = keys
    out = {}

    def timed_ms(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1)
            best = t if best is None or t < best else best
        return best

    d_out = torch.empty_like(d_ca)
    # three independent inputs (a selector equal to an input would make one
    # of the two bootstraps act on a noiseless trivial sample, which skips)
    d_cc = d_cb.flip(0).contiguous()
    ms = timed_ms(lambda: eng.bootsMUX(d_out, d_ca, d_cb, d_cc, batch, "split_fp32", stream=sp))
    out["mux_outputs_per_s"] = batch / (ms / 1000.0)
    out["mux_bootstraps_per_s"] = 2 * batch / (ms / 1000.0)
    table = [pkg.mod_switch_to_torus32((3 * m + 1) % 8, 16) for m in range(8)]
    d_tv = torch.from_numpy(pkg.test_vector(P.N, table)).cuda()
    ms = timed_ms(lambda: eng.bootstrap_tv(d_out, d_ca, d_tv, batch, "split_fp32", stream=sp))
    out["lookup_table_bootstraps_per_s"] = batch / (ms / 1000.0)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "cloud.key")
        t0 = time.perf_counter()
        pkg.save_cloud_key(path, P, bk, ks)
        t_save = time.perf_counter() - t0
        size = os.path.getsize(path)
        e2 = pkg.Engine(P, device=torch.cuda.current_device())
        t0 = time.perf_counter()
        e2.upload_cloud_key_file(path, forms=("split_fp32",))
        t_load = time.perf_counter() - t0
        e2.close()
    out["cloud_key_file"] = {"bytes": size, "save_s": t_save, "load_to_device_s": t_load}
    return out


def smem_roofline(kernels, batch, k_ms, clocks):
    """The blind rotation against the resource that bounds it: shared-memory
    wavefronts (ncu counts per bootstrap of the same kernels) over the
    kernels' time in this run, against one wavefront per SM clock at the SM
    clock sampled during the timed region.  None when a kernel of the step
    has no counted figure."""
    total = 0.0
    for name in kernels:
        base, _, cnt = name.partition(" x ")
        if base not in SMEM_WAVEFRONTS_PER_BOOTSTRAP:
            return None
        total += SMEM_WAVEFRONTS_PER_BOOTSTRAP[base] * (int(cnt) if cnt else batch)
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    achieved = total / (k_ms / 1000.0) / 1e9
    peak = SMS * mhz * 1e6 / 1e9
    return {"bound": "shared-memory pipe", "achieved": achieved, "peak": peak, "unit": "G wavefronts/s",
            "frac": achieved / peak, "wavefronts_per_step": total,
            "note": "wavefronts per bootstrap from ncu counts of the same kernels, time from this run"}


def blind_rotate_kernels(form, shape, batch, l=3):
    """Names of the blind-rotation kernels a launch of `batch` runs with
    launch shape `shape` (the engine's dispatch rules)."""
    if form == "fp64":
        if shape == 16 or (shape == 0 and batch <= SMS):
            return ["k_blind_rotate_spread2_f64<%d>" % l]
        return (["k_external_product<double,1,BlindRotate,3,%d>" % l] if shape in (0, 3)
                else ["k_blind_rotate_ring<double,1,4,%d,4,inline>" % l])
    ring = "k_blind_rotate_ring<float,2,%d,%d,4,%s>"
    batched = "k_blind_rotate_ring<float,2,4,%d,4,inline,nb%d>" % (l, max(l, 2))
    pairs = "k_blind_rotate_ring<float,2,6,%d,4,inline,nb2>" % l
    pair = "k_blind_rotate_pair<float,2,%d,%d,4>"
    spread = "k_blind_rotate_spread<%d>" % l
    spread2 = "k_blind_rotate_spread2<%d>" % l
    if shape in (0, 15):
        wave = 6 * SMS
        full, rest = (batch // wave) * wave, batch - (batch // wave) * wave
        if rest == 0 or rest > 4 * SMS:
            return [pairs]
        names = [pairs + " x %d" % full] if full else []
        if rest > 2 * SMS:
            return names + [batched + " x %d" % rest]
        if rest > SMS and shape == 0:
            return names + [pair % (2, l) + " x %d" % rest]
        if rest > SMS // 2:
            return names + [spread + " x %d" % rest]
        return names + [spread2 + " x %d" % rest]
    if shape == 14:
        return [spread]
    if shape == 16:
        return [spread2]
    if shape == 9:
        return [batched]
    if shape == 10:
        return [pairs]
    if shape in (11, 12, 13):
        return [pair % (shape - 10, l)]
    if shape in (1, 2, 4):
        return ["k_external_product<float,2,BlindRotate,%d,%d>" % (shape, l)]
    return [ring % (shape, l, "producer-warp" if shape == 5 else "inline")]


if __name__ == "__main__":
    main()
