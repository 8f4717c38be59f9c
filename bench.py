#!/usr/bin/env python
"""Benchmark: exact signed big-integer matrix multiplication C = A*B.

One step = one complete exact product through gbmm's public C ABI
(gbmm_matmul) on synthetic seeded matrices already resident in HBM.  The
metric is 64-bit limb-MACs per second:
    limb-MACs = sum_k (sum_i L64(A_ik)) * (sum_j L64(B_kj)),
L64 = 64-bit limb count of an entry's magnitude (schoolbook-equivalent work,
so Winograd / Karatsuba / CRT savings count as speed).

`--impl reference` times the reference's CPU implementation of the path
instead (the mat-cpu algorithm; the reference binary when it was built on this
machine, else the CPU restatement in oracle/) on a bounded row sample of the
same workload with all host cores.

Multi-GPU: the product does not shard across this run's GPUs; under torchrun
every rank runs an independent replica (weak scaling) and value is the
aggregate over ranks.
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
PKG = os.path.join(ROOT, "bachelor-thesis_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WORKLOADS = {
    # 256x256x256, 2048-bit signed entries, 5% exact zeros, 5% shortened to 64 bits
    "cfg2": dict(K=256, M=256, N=256, bits=2048, zero=0.05, short=0.05, short_bits=64, cutoff=32,
                 label="256x256x256 2048-bit signed, 5% zero, 5% 64-bit entries"),
    # 512x512x512, 4096-bit uniform signed entries
    "cfg3": dict(K=512, M=512, N=512, bits=4096, zero=0.0, short=0.0, short_bits=0, cutoff=32,
                 label="512x512x512 4096-bit signed"),
    # 64x64x64, 1024-bit uniform signed entries
    "cfg1": dict(K=64, M=64, N=64, bits=1024, zero=0.0, short=0.0, short_bits=0, cutoff=32,
                 label="64x64x64 1024-bit signed"),
    # 64 independent products: m, n, k log-uniform in [16, 512], bit length per
    # matrix log-uniform in [64, 16384], 10% zero entries; one batched call
    "cfg4": dict(K=0, M=0, N=0, bits=0, zero=0.1, short=0.0, short_bits=0, cutoff=32, jobs=64,
                 label="64 uneven products: m,n,k log-uniform [16,512], bits log-uniform [64,16384], 10% zeros"),
    # learned dispatch: jobs drawn as configuration 4 plus rectangular 1024x64x1024
    # products at bit lengths log-uniform in [256, 8192]; the model trains on the
    # autotuner's timings of four such batches and dispatches a held-out batch and
    # a stream of 10^4 jobs
    "cfg5": dict(K=0, M=0, N=0, bits=0, zero=0.1, short=0.0, short_bits=0, cutoff=32, jobs=64, rect=8,
                 label="learned dispatch: batches of 64 jobs as cfg4 + 8 rectangular 1024x64x1024 at "
                       "[256,8192] bits; model trained on the autotuner's timings of 4 separately drawn "
                       "batches; evaluated on a held-out batch and a 10^4-job stream"),
    # the limb form's batched mpn / mpz kernels one by one, on batches larger than L2
    "limbkernels": dict(K=0, M=0, N=0, bits=0, zero=0.0, short=0.0, short_bits=0, cutoff=32,
                        label="limb-form kernels: batched mpn_add_n/sub_n/mul_1/addmul_1/submul_1, "
                              "mul_basecase, toom22_mul, mpz_add/sub/mul/addmul over 2^21-operand batches"),
}
DEFAULT_WORKLOAD = "cfg3"
DEFAULT_PATH = "crt"
L2_BYTES = 129 * 1024 * 1024


def gen_planes(rng, n, bits, zero, short, short_bits):
    """Seeded synthetic entries: magnitudes uniform in [0, 2^bits), fair sign,
    a fraction of exact zeros and of entries shortened to short_bits."""
    L = (bits + 31) // 32
    limbs = rng.integers(0, 2**32, size=(L, n), dtype=np.uint64).astype(np.uint32)
    top = bits - 32 * (L - 1)
    if top < 32:
        limbs[L - 1] &= np.uint32((1 << top) - 1)
    u = rng.random(n)
    zmask = u < zero
    smask = (u >= zero) & (u < zero + short)
    limbs[:, zmask] = 0
    if short_bits:
        Ls = (short_bits + 31) // 32
        limbs[Ls:, smask] = 0
    nz = limbs != 0
    rev = nz[::-1]
    size = np.where(nz.any(axis=0), L - rev.argmax(axis=0), 0).astype(np.int32)
    sign = rng.random(n) < 0.5
    size[sign] = -size[sign]
    return limbs, size


def limb_macs(K, M, N, As, Bs):
    """sum_k (sum_i L64(A_ik)) (sum_j L64(B_kj)) with 64-bit limb counts."""
    a64 = ((np.abs(As.astype(np.int64)) + 1) // 2).reshape(K, M)
    b64 = ((np.abs(Bs.astype(np.int64)) + 1) // 2).reshape(M, N)
    return int((a64.sum(axis=0) * b64.sum(axis=1)).sum())


def entry_int(limbs, sizes, e):
    s = int(sizes[e])
    m = int.from_bytes(np.ascontiguousarray(limbs[:, e]).tobytes(), "little")
    return -m if s < 0 else m


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons every 200 ms."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sms)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        import torch
        if not torch.cuda.is_available():
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------
# CPU leg (the reference's algorithm on the host cores)
# ------------------------------------------------------------------------------------
CPU_JOBSZ, CPU_BASESZ = 128, 32   # mat-cpu's -J / -B for -m 31 (its defaults in BASELINE's timing plan)


def workload_config(W, seed):
    """The `config` both arms print (identical dicts, so the two lines compare)."""
    return {"workload": W["label"], "seed": seed,
            "l2": "GPU arm: flushed between timed steps (512 MiB write); CPU arm: host caches as they are"}


class CpuSampler:
    """Bounded samples of C = A*B by the reference's methods on the host cores,
    timing the multiplication only (mat-cpu's "Multiplication took"):
      -m 1  : the naive mat_mul order (mat-cpu/mat.c:72-82) on the first `rows` rows;
      -m 31 : jobsz-block products with Winograd leaves (mat-cpu/matj.c:571-660)
              on the first block row of C.
    A sample's share of the full product is rows / K, so its limb-MAC/s is the
    full product's rate; `calibrate` times each method once and keeps the faster.
    (-m 35, the full-depth Winograd job DAG of mat-cpu/matj.c:214-417, cannot be cut
    into row samples; the reference's own timings put it behind -m 31 on this
    workload: 75.7 s against 42.6 s on 8 x86 cores.)"""

    def __init__(self, W, Al, As, Bl, Bs, nthreads, target_s):
        import oracle as orc
        self.orc = orc
        self.W, self.A, self.B = W, (Al, As), (Bl, Bs)
        self.nthreads, self.target_s = nthreads, target_s
        self.gmp = orc.gmp_available()
        self.rows = {}
        self.cn = 2 * max(Al.shape[0], Bl.shape[0]) + 4

    def _run(self, method, rows):
        K, M, N = self.W["K"], self.W["M"], self.W["N"]
        self.orc.set_backend(1 if self.gmp else 0)
        try:
            secs, _ = self.orc.sample_rows(K, M, N, self.A, self.B, 0, rows, method=method, basesz=CPU_BASESZ,
                                           jobsz=CPU_JOBSZ, nthreads=self.nthreads, cn=self.cn)
        finally:
            self.orc.set_backend(0)
        macs = limb_macs(rows, M, N, self.A[1][:rows * M], self.B[1])
        return macs / secs, secs

    def methods(self):
        K, M, N = self.W["K"], self.W["M"], self.W["N"]
        out = [1]
        if K % CPU_JOBSZ == 0 and M % CPU_JOBSZ == 0 and N % CPU_JOBSZ == 0:
            out.append(31)
        return out

    def sample(self, method):
        """(limb-MAC/s, seconds, rows) of one sample; the first call per method sizes it."""
        K = self.W["K"]
        if method not in self.rows:
            if method == 31:
                self.rows[method] = CPU_JOBSZ
            else:
                probe = max(1, min(K, self.nthreads))
                _, t = self._run(1, probe)
                self.rows[1] = int(min(K, max(probe, probe * self.target_s / max(t, 1e-6))))
        rate, secs = self._run(method, self.rows[method])
        return rate, secs, self.rows[method]

    def calibrate(self):
        rates = {m: self.sample(m) for m in self.methods()}
        best = max(rates, key=lambda m: rates[m][0])
        return best, rates

    def describe(self, method):
        K, M, N = self.W["K"], self.W["M"], self.W["N"]
        r = self.rows[method]
        how = ("naive mat_mul order (mat-cpu -m 1)" if method == 1 else
               f"mat-cpu -m 31: {CPU_JOBSZ}-blocks with Winograd leaves to {CPU_BASESZ}")
        return (f"rows 0-{r - 1} of {K} of C ({r}x{M}x{N}), {how}, "
                f"{'libgmp.so.10' if self.gmp else 'restated GMP'} arithmetic, {self.nthreads} threads")


def run_reference(args, W, world, rank):
    if rank != 0:
        return 0
    rng = np.random.default_rng(args.seed)
    Al, As = gen_planes(rng, W["K"] * W["M"], W["bits"], W["zero"], W["short"], W["short_bits"])
    Bl, Bs = gen_planes(rng, W["M"] * W["N"], W["bits"], W["zero"], W["short"], W["short_bits"])
    nthreads = os.cpu_count() or 1
    cs = CpuSampler(W, Al, As, Bl, Bs, nthreads, args.cpu_seconds)
    best, cal = cs.calibrate()
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        v, t, _ = cs.sample(best)
        if i >= args.warmup:
            vals.append(v)
            secs.append(t)
    value = statistics.median(vals)
    full_s = limb_macs(W["K"], W["M"], W["N"], As, Bs) / value
    line = {
        "impl": "reference", "metric": "limb-MAC/s", "value": value, "unit": "limb-MAC/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": workload_config(W, args.seed),
        "run": {"step": "one bounded sample: " + cs.describe(best), "method": f"-m {best}",
                "methods_timed": {f"-m {m}": {"limb-MAC/s": r[0], "s": r[1]} for m, r in cal.items()},
                "full_product_s_at_this_rate": full_s},
        "cpu_baseline": {"value": value, "unit": "limb-MAC/s", "cores": nthreads, "kind": "port",
                         "sample": cs.describe(best)},
        "e2e": {"value": value, "unit": "limb-MAC/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------
# GPU leg
# ------------------------------------------------------------------------------------
def run_gpu(args, W, world, rank, local):
    import torch
    import gbmm
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(args.seed + 0 * rank)
    K, M, N, bits = W["K"], W["M"], W["N"], W["bits"]
    Al, As = gen_planes(rng, K * M, bits, W["zero"], W["short"], W["short_bits"])
    Bl, Bs = gen_planes(rng, M * N, bits, W["zero"], W["short"], W["short_bits"])
    macs = limb_macs(K, M, N, As, Bs)
    path = {"limb": gbmm.PATH_LIMB, "crt": gbmm.PATH_CRT, "auto": gbmm.PATH_AUTO}[args.path]
    method = {"winograd": gbmm.METHOD_WINOGRAD, "naive": gbmm.METHOD_NAIVE, "strassen": gbmm.METHOD_STRASSEN}[
        args.method]
    cutoff = args.cutoff or W["cutoff"]
    nl = Al.shape[0]
    h = gbmm.Handle()
    dA = gbmm.DeviceMatrix(K, M, nl)
    dB = gbmm.DeviceMatrix(M, N, nl)
    dA.upload(Al, As)
    dB.upload(Bl, Bs)
    cn = gbmm.limbs_needed(nl, nl, M, path=path, method=method, cutoff=cutoff)
    dC = gbmm.DeviceMatrix(K, N, cn)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device="cuda")

    def step():
        h.matmul(dC, dA, dB, path=path, method=method, cutoff=cutoff)

    # correctness on a sample of entries (bit-exact against Python integers)
    step()
    torch.cuda.synchronize()
    Cl, Cs = dC.download()
    srng = np.random.default_rng(7)
    for _ in range(args.check):
        y, x = int(srng.integers(K)), int(srng.integers(N))
        exp = sum(entry_int(Al, As, y * M + k) * entry_int(Bl, Bs, k * N + x) for k in range(M))
        got = entry_int(Cl, Cs, y * N + x)
        if got != exp:
            raise SystemExit(f"bench: C[{y}][{x}] differs from the exact product")

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = gbmm.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(i)  # evict L2 between timed steps (outside the events)
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = gbmm.kernel_launches() - launches0
    barrier(world)
    per = [a.elapsed_time(b) for a, b in ev]
    ms = sum(per) / len(per)
    ms = max_over_ranks(world, ms)

    # per-kernel CUDA-event timing over extra profiled steps (roofline of the dominant kernel)
    gbmm.profile(True)
    for i in range(max(1, args.profile_steps)):
        flush.fill_(i)
        step()
    torch.cuda.synchronize()
    prof = gbmm.profile_read()
    gbmm.profile(False)
    clocks = sampler.stop()

    # end to end through the C ABI with host buffers: gbmm_matmul_host runs `ne`
    # products back to back on pinned host planes; every product's H2D of A and B
    # and D2H of C is inside the timed region, pipelined against the neighbouring
    # products' compute (two device slots, upload / compute / download streams)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    hA, hAs, hB, hBs = pin(Al), pin(As), pin(Bl), pin(Bs)
    hC = pin(np.zeros((cn, K * N), dtype=np.uint32))
    hCs = pin(np.zeros(K * N, dtype=np.int32))
    # 40 products (or --steps, if more): the pipeline's fill (the first product's
    # upload) and drain (the last one's download) spread over the whole stream
    ne = max(40, args.steps)
    hjobs = h.host_jobs([(K, M, N, (hA, hAs), (hB, hBs), (hC, hCs))] * ne, path=path, method=method, cutoff=cutoff)
    h.matmul_host(h.host_jobs([(K, M, N, (hA, hAs), (hB, hBs), (hC, hCs))] * 2, path=path, method=method,
                              cutoff=cutoff))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h.matmul_host(hjobs)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, (time.perf_counter() - t0) / ne)
    if args.check:
        got = gbmm.planes_to_ints(hC[:, :1], hCs[:1])[0]
        exp0 = sum(entry_int(Al, As, k) * entry_int(Bl, Bs, k * N) for k in range(M))
        if got != exp0:
            raise SystemExit("bench: end-to-end product differs from the exact product")
    h2d = (Al.nbytes + As.nbytes + Bl.nbytes + Bs.nbytes)
    d2h = 4 * cn * K * N + 4 * K * N

    # roofline of the dominant kernel
    top = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("", (1, 0.0))
    kname, (klaunch, kms) = top
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    macpk = mac_peak(gbmm, stream) if kname in ("k_limb_matmul", "k_wino_leaves") else None
    roof = kernel_roofline(kname, klaunch, kms, W, args, K, M, N, nl, cn, peaks, prof, macpk)
    limb = None
    if path == gbmm.PATH_CRT and not args.no_limb:
        limb = measure_limb_path(gbmm, h, dA, dB, dC, K, M, N, nl, args, flush, stream)

    if rank != 0:
        return 0
    value = world * macs / (ms * 1e-3)
    line = {
        "metric": "limb-MAC/s", "value": value, "unit": "limb-MAC/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16" if path == gbmm.PATH_CRT else "u32", "data": "synthetic",
        "config": workload_config(W, args.seed),
        "run": {"path": args.path, "method": args.method, "cutoff": cutoff, "limb_macs_per_step": macs,
                "check": f"{args.check} entries bit-exact vs Python integers", "parallelism": f"replicas x{world}"},
        "roofline": roof,
        "kernels": {k: {"launches": v[0], "ms_total": round(v[1], 4)} for k, v in sorted(prof.items())},
        "e2e": {"value": world * macs / e2e_s, "unit": "limb-MAC/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "s_per_step": e2e_s,
                "api": f"gbmm_matmul_host, {ne} products on pinned host planes, copies pipelined against compute"},
        "gpu_launches": int(launches // max(1, args.steps)) * args.steps,
        "clocks": clocks,
    }
    if limb is not None:
        line["limb_path"] = limb
        line["crt_over_limb"] = limb["ms_per_step"] / ms
    if not args.no_cpu and world == 1:
        cs = CpuSampler(W, Al, As, Bl, Bs, os.cpu_count() or 1, args.cpu_seconds)
        best, cal = cs.calibrate()
        line["cpu_baseline"] = {"value": cal[best][0], "unit": "limb-MAC/s", "cores": os.cpu_count() or 1,
                                "kind": "port", "sample": cs.describe(best),
                                "methods_timed": {f"-m {m}": r[0] for m, r in cal.items()}}
    print(json.dumps(line), flush=True)
    return 0


def primes_desc_16():
    sieve = bytearray([1]) * 65536
    sieve[0] = sieve[1] = 0
    for i in range(2, 256):
        if sieve[i]:
            sieve[i * i::i] = bytearray(len(sieve[i * i::i]))
    return [i for i in range(65535, 2, -1) if sieve[i]]


def crt_params(bits_a, bits_b, k):
    """Moduli count P and output digit count Dout chosen by the CRT path."""
    import math
    lg = max(0, math.ceil(math.log2(max(k, 1))))
    bound = bits_a + bits_b + lg + 2 + 16
    pr = primes_desc_16()
    acc, P, mod = 0.0, 0, 1
    while acc < bound:
        acc += math.log2(pr[P])
        mod *= pr[P]
        P += 1
    modbits = 32 * ((mod.bit_length() + 31) // 32)
    return P, (modbits + 6) // 7 + 2  # base-128 output digits


# DRAM bytes (read + write) per launch of each CRT GEMM on 512x512x512 at 4096 bits,
# from a one-pass ncu capture of this workload (dram__bytes_read.sum +
# dram__bytes_write.sum; profiles/crt_512x512x512_4096b_dram_bytes.md).  The residue
# figure is the mean of its two launches (A, then B).
NCU_DRAM_BYTES_512_4096 = {
    "k_crt_residue": (269.558528e6 + 487.749376e6 + 269.553408e6 + 487.559680e6) / 2,
    "k_crt_product": 1083.140608e6 + 506.246400e6,
    "k_crt_recon": 583.059200e6 + 241.474048e6,
}
FIXED_POINT_COLUMNS = 14  # reconstruction columns that carry the 2^96 / p_i weights


def kernel_roofline(kname, klaunch, kms, W, args, K, M, N, nl, cn, peaks, prof, macpk=None):
    """Algorithmic work of the dominant kernel per launch / its mean CUDA-event time.
    Tensor kernels: useful bf16 FLOPs (2 per digit MAC, no tile padding counted).
    Memory kernels: bytes that must move (inputs read once, outputs written once)."""
    per_ms = kms / max(1, klaunch)
    hbm = peaks.get("hbm_gbs", 6800.0)
    bf16 = peaks.get("bf16_tflops", 1900.0)
    src = "measured" if peaks else "fallback"
    P, Dout = crt_params(32 * nl, 32 * nl, M)
    dx = 4 * nl
    flops = None
    note = ""
    if kname == "k_crt_product":
        flops = 2.0 * K * M * N * 4 * P
        note = f"4 digit-pair GEMMs per modulus, P={P} moduli, {K}x{M}x{N}"
    elif kname == "k_crt_residue":
        flops = 2.0 * (K * M + M * N) / 2 * dx * 2 * P  # one launch per operand (square: equal halves)
        note = f"entries x {dx} digits x {2 * P} table columns per operand"
    elif kname == "k_crt_recon":
        flops = 2.0 * K * N * 2 * P * (FIXED_POINT_COLUMNS + Dout)
        note = f"entries x {2 * P} moduli digits x {FIXED_POINT_COLUMNS + Dout} output columns"
    if flops is not None:
        ach = flops / (per_ms * 1e-3) / 1e12
        traffic = None
        if (K, M, N, W["bits"]) == (512, 512, 512, 4096) and kname in NCU_DRAM_BYTES_512_4096:
            traffic = NCU_DRAM_BYTES_512_4096[kname]
            note += "; traffic: one-pass ncu DRAM bytes of this launch at 512^3"
        return {"kernel": kname, "bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                "frac": ach / bf16, "traffic": traffic, "peak_source": src + " (bf16 dense, burst)",
                "ms_per_launch": per_ms, "note": note}
    if kname in ("k_limb_matmul", "k_wino_leaves") and macpk:
        # integer-multiply bound: 32x32-bit limb MACs of the kernel's products
        levels = 0
        if kname == "k_wino_leaves":
            cut = args.cutoff or 32
            levels = (K // cut).bit_length() - 1 if K == M == N and K > cut else 0
            while levels > 0 and K % (1 << levels):
                levels -= 1
            macs = winograd_leaf_macs(K, levels, nl, nl)
        else:
            macs = K * M * N * nl * nl
        ach = macs / (per_ms * 1e-3)
        return {"kernel": kname, "bound": "int-mul", "achieved": ach, "peak": macpk, "unit": "MAC/s",
                "frac": ach / macpk, "traffic": None, "peak_source": "measured (k_mac_peak, 96-bit column MAC step)",
                "ms_per_launch": per_ms, "levels": levels,
                "note": "32x32-bit limb MACs of the kernel's products per launch / its CUDA-event time"}
    # memory-bound kernels: algorithmic bytes per launch
    if kname == "k_crt_digits":
        bytes_ = ((K * M + M * N) / 2) * (4 * nl + 2 * ((4 * nl + 63) // 64 * 64))
    else:
        bytes_ = (4 * nl * (K * M + M * N) + 4 * (K * M + M * N) + 4 * cn * K * N + 4 * K * N) / max(1, klaunch)
        note = "integer-MAC bound kernel; algorithmic bytes = A+B read once, C written once"
    ach = bytes_ / (per_ms * 1e-3) / 1e9
    return {"kernel": kname, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "traffic": None, "peak_source": src, "ms_per_launch": per_ms, "note": note}


def mac_peak(gbmm, stream):
    """Measured 32x32-bit MAC rate of the product kernels' inner step (k_mac_peak:
    MAC96 on register operands, 8 CTAs per SM); best of 5 launches."""
    import ctypes
    import torch
    f = gbmm.lib().gbmmx_mac_peak
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
    blocks = 8 * torch.cuda.get_device_properties(0).multi_processor_count
    iters = 4000
    out = torch.zeros(blocks * 256, dtype=torch.int32, device="cuda")
    for _ in range(2):
        gbmm.check(f(out.data_ptr(), blocks, iters, stream.cuda_stream))
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gbmm.check(f(out.data_ptr(), blocks, iters, stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return blocks * 256 * iters * 64 / (best * 1e-3)


def winograd_leaf_macs(N, levels, la, lb):
    """32x32-bit MACs of the breadth-first tree's leaf products: 7^levels products of
    h = N / 2^levels; a leaf's A operand is a quadrant of A (la limbs) when its path
    takes only the A11 / A12 / A22 children (3 of 7), else a sum of la + 1 limbs;
    likewise B with B11 / B21 / B22."""
    h = N >> levels
    n_all, n_a, n_b, n_ab = 7 ** levels, 3 ** levels, 3 ** levels, 2 ** levels
    macs = ((n_all - n_a - n_b + n_ab) * (la + 1) * (lb + 1) + (n_a - n_ab) * la * (lb + 1) +
            (n_b - n_ab) * (la + 1) * lb + n_ab * la * lb)
    return macs * h ** 3


def measure_limb_path(gbmm, h, dA, dB, dC_crt, K, M, N, nl, args, flush, stream):
    """The plain limb form on the same inputs (the >= 10x comparison of the CRT form is
    against it): the per-entry kernel alone and Winograd's breadth-first tree down to
    --limb-cutoff, each timed over --limb-steps steps; the faster is the comparison
    basis.  Each result must equal the CRT result bit for bit.  Returns the record
    for the bench line."""
    import torch
    peak = mac_peak(gbmm, stream)
    forms = {}
    for form, method, cutoff in (("naive", gbmm.METHOD_NAIVE, 0), ("winograd", gbmm.METHOD_WINOGRAD, args.limb_cutoff)):
        cn = max(gbmm.limbs_needed(nl, nl, M, path=gbmm.PATH_LIMB, method=method, cutoff=cutoff), dC_crt.nlimbs)
        dL = gbmm.DeviceMatrix(K, N, cn)

        def step():
            h.matmul(dL, dA, dB, path=gbmm.PATH_LIMB, method=method, cutoff=cutoff)

        step()
        torch.cuda.synchronize()
        same = bool(torch.equal(dL.sizes_t, dC_crt.sizes_t)) and bool(
            torch.equal(dL.limbs_t[:dC_crt.nlimbs * K * N], dC_crt.limbs_t[:dC_crt.nlimbs * K * N])) and not bool(
            dL.limbs_t[dC_crt.nlimbs * K * N:].any())
        if not same:
            raise SystemExit(f"bench: the limb path ({form}) and the CRT path differ")
        times = []
        l0 = gbmm.kernel_launches()
        for i in range(args.limb_steps):
            flush.fill_(i)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        launches = (gbmm.kernel_launches() - l0) // max(1, args.limb_steps)
        gbmm.profile(True)
        flush.fill_(7)
        step()
        torch.cuda.synchronize()
        prof = gbmm.profile_read()
        gbmm.profile(False)
        del dL
        levels = 0
        if method == gbmm.METHOD_WINOGRAD and K == M == N and K > cutoff:
            # the recursion depth the library uses: floor(log2(N / cutoff)), lowered until 2^levels divides N
            levels = (K // cutoff).bit_length() - 1
            while levels > 0 and K % (1 << levels):
                levels -= 1
        lk = "k_wino_leaves" if "k_wino_leaves" in prof else "k_limb_matmul"
        lms = prof.get(lk, (1, 0.0))[1]
        macs = winograd_leaf_macs(K, levels, nl, nl) if lk == "k_wino_leaves" else K * M * N * nl * nl
        ach = macs / (lms * 1e-3)
        forms[form] = {
            "ms_per_step": statistics.median(times), "steps": args.limb_steps,
            "cutoff": cutoff if method == gbmm.METHOD_WINOGRAD else None, "levels": levels,
            "launches_per_step": int(launches), "equals_crt_result": same,
            "kernels": {k: {"launches": v[0], "ms_total": round(v[1], 3)} for k, v in sorted(prof.items())},
            "roofline": {"kernel": lk, "bound": "int-mul", "achieved": ach, "peak": peak, "unit": "MAC/s",
                         "frac": ach / peak,
                         "note": "32x32-bit limb MACs of the kernel's products / its time; peak: measured rate "
                                 "of the same 96-bit column MAC step on register operands (k_mac_peak)"}}
    best = min(forms, key=lambda f: forms[f]["ms_per_step"])
    return {"ms_per_step": forms[best]["ms_per_step"], "form": best, "forms": forms,
            "roofline": forms[best]["roofline"]}


def gen_jobs(gbmm, W, seed):
    """Seeded uneven jobs of configuration 4 (and 5's rectangular ones), uploaded:
    [(C, A, B, host planes...)], total limb-MACs."""
    rng = np.random.default_rng(seed)
    lu = lambda lo, hi: int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))
    shapes = []
    for _ in range(W["jobs"]):
        shapes.append((lu(16, 512), lu(16, 512), lu(16, 512), lu(64, 16384), lu(64, 16384)))
    for _ in range(W.get("rect", 0)):
        shapes.append((1024, 64, 1024, lu(256, 8192), lu(256, 8192)))
    mats, macs = [], 0
    for K, M, N, ba, bb in shapes:
        Al, As = gen_planes(rng, K * M, ba, W["zero"], 0, 0)
        Bl, Bs = gen_planes(rng, M * N, bb, W["zero"], 0, 0)
        dA, dB = gbmm.DeviceMatrix(K, M, Al.shape[0]), gbmm.DeviceMatrix(M, N, Bl.shape[0])
        dA.upload(Al, As)
        dB.upload(Bl, Bs)
        dC = gbmm.DeviceMatrix(K, N, Al.shape[0] + Bl.shape[0] + 2)
        mats.append((dC, dA, dB, (Al, As, Bl, Bs, K, M, N)))
        macs += limb_macs(K, M, N, As, Bs)
    return mats, macs


def check_jobs(mats, what):
    srng = np.random.default_rng(3)
    for (dC, dA, dB, (Al, As, Bl, Bs, K, M, N)) in mats[:: max(1, len(mats) // 8)]:
        Cl, Cs = dC.download()
        for _ in range(2):
            y, x = int(srng.integers(K)), int(srng.integers(N))
            exp = sum(entry_int(Al, As, y * M + k) * entry_int(Bl, Bs, k * N + x) for k in range(M))
            if entry_int(Cl, Cs, y * N + x) != exp:
                raise SystemExit(f"bench: {what} product differs from the exact product")


def time_batched(h, jobs, args, flush, stream):
    """Warm-up (eager, then capture), then K timed graph replays: mean ms per call."""
    import torch
    for _ in range(max(args.warmup, 0)):
        h.matmul_batched(jobs)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(i)
        ev[i][0].record(stream)
        h.matmul_batched(jobs)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / args.steps


def stream_shapes(rng, njobs, W):
    """Shapes of configuration 5's job stream: (m, k, n, bits_a, bits_b) drawn as
    configuration 4 (dims log-uniform in [16, 512], bits in [64, 16384]), with one
    job in nine a rectangular 1024 x 64 x 1024 product at bits log-uniform in [256, 8192]."""
    lu = lambda lo, hi: int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))
    out = []
    for _ in range(njobs):
        if rng.random() < 1.0 / 9.0:
            out.append((1024, 64, 1024, lu(256, 8192), lu(256, 8192)))
        else:
            out.append((lu(16, 512), lu(16, 512), lu(16, 512), lu(64, 16384), lu(64, 16384)))
    return out


def device_random_matrix(gbmm, torch, rows, cols, bits, zero, gen):
    """rows x cols signed entries of exactly `bits` bits (top bit set), a fraction
    `zero` of exact zeros, random signs; generated on the device."""
    L = (bits + 31) // 32
    n = rows * cols
    m = gbmm.DeviceMatrix(rows, cols, L)
    lv = m.limbs_t.view(L, n)
    lv.copy_(torch.randint(-2 ** 31, 2 ** 31, (L, n), dtype=torch.int64, device="cuda", generator=gen).to(torch.int32))
    top = bits - 32 * (L - 1)
    mask = (1 << top) - 1 if top < 32 else 0xFFFFFFFF
    hi = 1 << (top - 1)
    t = lv[L - 1].to(torch.int64) & mask | hi
    lv[L - 1] = torch.where(t >= 2 ** 31, t - 2 ** 32, t).to(torch.int32)
    z = torch.rand(n, device="cuda", generator=gen) < zero
    lv[:, z] = 0
    sign = torch.where(torch.rand(n, device="cuda", generator=gen) < 0.5, -1, 1).to(torch.int32)
    m.sizes_t.copy_(torch.where(z, 0, sign * L).to(torch.int32))
    return m


def tune_times(gbmm, h, mats, NP):
    """The autotuner's timing of every admissible plan of every job:
    {(m, k, n, la, lb): [ms per plan, NaN where not timed]} and the raw rows."""
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        log = os.path.join(td, "tune.jsonl")
        h.autotune(h.jobs([(c, a, b) for c, a, b, _ in mats]), repeats=1, log_path=log)
        rows = [json.loads(l) for l in open(log)]
    times = {}
    for r in rows:
        times.setdefault((r["m"], r["k"], r["n"], r["la"], r["lb"]), [np.nan] * NP)[r["plan"]] = r["ms"]
    return times, rows


def run_learned(args, W, world, rank, local):
    """Configuration 5: the learned cost model against the plain heuristic.  The
    autotuner times every candidate plan (limb kernel, Winograd at three cutoffs,
    CRT with three tile forms and with a limb-half split) on four seeded streams;
    the MLP trains on those timings with its own CUDA kernels.  Then, on inputs
    drawn separately: (1) a 72-job batch whose every plan is timed too (the summed
    time of each policy's picks), run as one batched call replayed from its CUDA
    graph with the heuristic, the autotuner's table and the model; (2) a stream of
    --stream-jobs jobs (10^4 by default) in batches of 50 with the heuristic and the
    model, the two policies' products compared bit for bit on the device."""
    import torch
    import gbmm
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    NP = gbmm.NPLANS
    ht = gbmm.Handle()
    times, rows = {}, []
    t0 = time.perf_counter()
    for t in range(4):
        train, _ = gen_jobs(gbmm, W, args.seed + 1 + 1000 * t)
        tt, rr = tune_times(gbmm, ht, train, NP)
        times.update(tt)
        rows += rr
        del train
        torch.cuda.empty_cache()
    tune_s = time.perf_counter() - t0
    keys = sorted(times)
    X = np.stack([gbmm.model_features(m, k, n, la, lb) for (m, k, n, la, lb) in keys])
    T = np.log2(np.array([times[k] for k in keys], dtype=np.float64)).astype(np.float32)
    hl = gbmm.Handle()
    hl.model_init(seed=5)
    t0 = time.perf_counter()
    loss = hl.model_train(X, T, epochs=2000, lr=3e-3)
    train_s = time.perf_counter() - t0
    hl.model_use(True)

    # (1) held-out batch: every plan timed, then graph replay of each policy
    evals, macs = gen_jobs(gbmm, W, args.seed)
    he = gbmm.Handle()
    etimes, _ = tune_times(gbmm, he, evals, NP)
    he.close()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device="cuda")
    hh = gbmm.Handle()
    res, picked_ms = {}, {}
    launches = 0
    sampler = ClockSampler(local)
    sampler.start()
    key = lambda c, a, b: (c.rows, a.cols, c.cols, a.nlimbs, b.nlimbs)
    for name, h in (("heuristic", hh), ("autotuned", ht), ("learned", hl)):
        jobs = h.jobs([(c, a, b) for c, a, b, _ in evals])
        chosen = h.matmul_batched(jobs, plans=True)
        torch.cuda.synchronize()
        check_jobs(evals, name)
        picked_ms[name] = float(sum(etimes[key(c, a, b)][q] for (c, a, b, _), (_, q) in zip(evals, chosen)))
        if name == "learned":
            launches0 = gbmm.kernel_launches()
        ms = max_over_ranks(world, time_batched(h, jobs, args, flush, stream))
        if name == "learned":
            launches = gbmm.kernel_launches() - launches0
        res[name] = (ms, {str(p): [q for _, q in chosen].count(p) for p in sorted(set(q for _, q in chosen))})
    picked_ms["best_possible"] = float(sum(np.nanmin(etimes[key(c, a, b)]) for c, a, b, _ in evals))
    n_eval = len(evals)
    del evals
    torch.cuda.empty_cache()

    # (2) the job stream, batches of 50 with inputs made on the device
    srng = np.random.default_rng(args.seed + 7)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(args.seed)
    shapes = stream_shapes(srng, args.stream_jobs, W)
    st_ms = {"heuristic": 0.0, "learned": 0.0}
    st_macs, compared, plans_used = 0, 0, {}
    hh.set_graphs(False)
    hl.set_graphs(False)
    for c0 in range(0, len(shapes), 50):
        mats = []
        for (K, M, N, ba, bb) in shapes[c0:c0 + 50]:
            dA = device_random_matrix(gbmm, torch, K, M, ba, W["zero"], gen)
            dB = device_random_matrix(gbmm, torch, M, N, bb, W["zero"], gen)
            outs = {p: gbmm.DeviceMatrix(K, N, dA.nlimbs + dB.nlimbs + 2) for p in st_ms}
            mats.append((dA, dB, outs))
            st_macs += K * M * N * ((ba + 63) // 64) * ((bb + 63) // 64)
        for name, h in (("heuristic", hh), ("learned", hl)):
            jobs = h.jobs([(o[name], a, b) for a, b, o in mats])
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            chosen = h.matmul_batched(jobs, plans=True)
            e1.record(stream)
            torch.cuda.synchronize()
            st_ms[name] += e0.elapsed_time(e1)
            if name == "learned":
                for _, q in chosen:
                    plans_used[str(q)] = plans_used.get(str(q), 0) + 1
        for a, b, o in mats[::10]:
            if not (torch.equal(o["heuristic"].sizes_t, o["learned"].sizes_t) and
                    torch.equal(o["heuristic"].limbs_t, o["learned"].limbs_t)):
                raise SystemExit("bench: learned and heuristic dispatch gave different products")
            compared += 1
        del mats
    clocks = sampler.stop()
    if rank != 0:
        return 0
    ms = st_ms["learned"]
    line = {
        "metric": "limb-MAC/s", "value": world * st_macs / (ms * 1e-3), "unit": "limb-MAC/s", "n_gpus": world,
        "steps": 1, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16+u32", "data": "synthetic",
        "config": workload_config(W, args.seed),
        "run": {"step": f"one pass over a stream of {len(shapes)} jobs in batches of 50 (learned dispatch)",
                "stream": {"jobs": len(shapes), "limb_macs": st_macs, "ms": st_ms,
                           "learned_vs_heuristic": st_ms["heuristic"] / ms, "plans_used": plans_used,
                           "differential_checks": compared},
                "held_out_batch": {"jobs": n_eval, "ms_per_call": {k: v[0] for k, v in res.items()},
                                   "summed_ms_of_picked_plans": picked_ms,
                                   "plans": {k: v[1] for k, v in res.items()},
                                   "learned_vs_heuristic": res["heuristic"][0] / res["learned"][0],
                                   "limb_macs": macs, "graph": "replayed"},
                "training": {"timings": len(rows), "shapes": len(keys), "autotune_s": tune_s,
                             "train_s": train_s, "final_loss": loss}},
        "gpu_launches": int(launches), "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_limb_kernels(args, W, world, rank, local):
    """Each limb-form kernel through the public API on a batch larger than L2 (so
    every call streams from HBM): mean CUDA-event time per call, algorithmic bytes
    (inputs read once, outputs written once) and GB/s against the measured HBM copy
    peak; the product kernels also report 32x32-bit limb MACs per second.  One JSON
    line with a record per kernel."""
    import torch
    import gbmm
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    dev = "cuda"
    rnd = lambda *shape: torch.randint(-2 ** 31, 2 ** 31 - 1, shape, dtype=torch.int32, device=dev)
    nb, n = 1 << 21, 32                       # operands per batch, limbs per operand
    up, vp, rp = rnd(n, nb), rnd(n, nb), rnd(n, nb)
    vl, cy = rnd(nb), torch.zeros(nb, dtype=torch.int32, device=dev)

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(max(1, args.steps)):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / max(1, args.steps)

    out = {}

    def rec(name, kernel, ms, nbytes, macs=None):
        r = {"kernel": kernel, "ms": ms, "bytes": nbytes, "GB/s": nbytes / (ms * 1e-3) / 1e9,
             "frac_hbm": nbytes / (ms * 1e-3) / 1e9 / hbm}
        if macs:
            r["limb_macs_32"] = macs
            r["MAC/s"] = macs / (ms * 1e-3)
        out[name] = r

    L4 = 4 * n * nb                           # bytes of one operand batch
    rec("mpn_add_n", "k_mpn_addsub_n_serial", timed(lambda: gbmm.mpn_add_n(rp, up, vp, n, nb, nb, cy)),
        3 * L4 + 4 * nb)
    rec("mpn_sub_n", "k_mpn_addsub_n_serial", timed(lambda: gbmm.mpn_sub_n(rp, up, vp, n, nb, nb, cy)),
        3 * L4 + 4 * nb)
    rec("mpn_mul_1", "k_mpn_mul1ops", timed(lambda: gbmm.mpn_mul_1(rp, up, n, vl, nb, nb, cy)),
        2 * L4 + 8 * nb, n * nb)
    rec("mpn_addmul_1", "k_mpn_mul1ops", timed(lambda: gbmm.mpn_addmul_1(rp, up, n, vl, nb, nb, cy)),
        3 * L4 + 8 * nb, n * nb)
    rec("mpn_submul_1", "k_mpn_mul1ops", timed(lambda: gbmm.mpn_submul_1(rp, up, n, vl, nb, nb, cy)),
        3 * L4 + 8 * nb, n * nb)
    del rp
    # products: 2^18 operand pairs of 32 x 32 limbs (basecase), 64 x 64 limbs (basecase and
    # Toom-2.2: the Karatsuba split's gain is the ratio of the two times); MAC counts are
    # schoolbook-equivalent, against the measured rate of the 96-bit column MAC step
    peak = mac_peak(gbmm, stream)
    pb = 1 << 18
    ua, va = rnd(32, pb), rnd(32, pb)
    ra = torch.zeros(64, pb, dtype=torch.int32, device=dev)
    rec("mpn_mul_basecase", "k_mpn_mul_basecase_sm", timed(lambda: gbmm.mpn_mul_basecase(ra, ua, 32, va, 32, pb, pb)),
        4 * pb * (32 + 32 + 64), 32 * 32 * pb)
    ub, vb = rnd(64, pb), rnd(64, pb)
    rb = torch.zeros(128, pb, dtype=torch.int32, device=dev)
    rec("mpn_mul_basecase_64", "k_mpn_mul_basecase_sm",
        timed(lambda: gbmm.mpn_mul_basecase(rb, ub, 64, vb, 64, pb, pb)), 4 * pb * (64 + 64 + 128), 64 * 64 * pb)
    scratch = torch.zeros(int(gbmm.mpn_toom22_mul_itch(64, 64)), pb, dtype=torch.int32, device=dev)
    rec("mpn_toom22_mul", "k_mpn_toom22_sm",
        timed(lambda: gbmm.mpn_toom22_mul(rb, ub, 64, vb, 64, scratch, pb, pb)),
        4 * pb * (64 + 64 + 128), 64 * 64 * pb)
    del ua, va, ra
    # the Karatsuba split against the basecase at longer operands (2^16 pairs)
    qb = 1 << 16
    for L in (128, 192):
        uq, vq = rnd(L, qb), rnd(L, qb)
        rq = torch.zeros(2 * L, qb, dtype=torch.int32, device=dev)
        sq = torch.zeros(int(gbmm.mpn_toom22_mul_itch(L, L)), qb, dtype=torch.int32, device=dev)
        rec(f"mpn_mul_basecase_{L}", "k_mpn_mul_basecase_sm",
            timed(lambda: gbmm.mpn_mul_basecase(rq, uq, L, vq, L, qb, qb)), 4 * qb * 4 * L, L * L * qb)
        rec(f"mpn_toom22_mul_{L}", "k_mpn_toom22_sm",
            timed(lambda: gbmm.mpn_toom22_mul(rq, uq, L, vq, L, sq, qb, qb)), 4 * qb * 4 * L, L * L * qb)
        out[f"mpn_toom22_mul_{L}"]["over_basecase"] = out[f"mpn_mul_basecase_{L}"]["ms"] / out[f"mpn_toom22_mul_{L}"]["ms"]
        del uq, vq, rq, sq
    for k in out:
        if k.startswith("mpn_mul_basecase") or k.startswith("mpn_toom22"):
            out[k]["frac_mac_peak"] = out[k]["MAC/s"] / peak
    out["mpn_toom22_mul"]["over_basecase"] = out["mpn_mul_basecase_64"]["ms"] / out["mpn_toom22_mul"]["ms"]
    del ub, vb, rb, scratch, up, vp
    # signed entries of matrices: 1024 x 2048 entries, 32-limb operands (16 for products)
    rng = np.random.default_rng(args.seed)
    R, Cc = 1024, 2048
    E = R * Cc
    mats = {}
    for key, bits in (("u", 1024), ("v", 1024), ("s", 512), ("t", 512)):
        Lp, Sp = gen_planes(rng, E, bits, 0.0, 0.0, 0)
        m = gbmm.DeviceMatrix(R, Cc, Lp.shape[0])
        m.upload(Lp, Sp)
        mats[key] = m
    w = gbmm.DeviceMatrix(R, Cc, 33)
    rec("mpz_add", "k_mpz_addsub", timed(lambda: gbmm.mpz_add(w, mats["u"], mats["v"])), E * (4 * (32 + 32 + 33) + 12))
    rec("mpz_sub", "k_mpz_addsub", timed(lambda: gbmm.mpz_sub(w, mats["u"], mats["v"])), E * (4 * (32 + 32 + 33) + 12))
    p = gbmm.DeviceMatrix(R, Cc, 33)
    rec("mpz_mul", "k_mpz_mulops", timed(lambda: gbmm.mpz_mul(p, mats["s"], mats["t"])),
        E * (4 * (16 + 16 + 32) + 12), 16 * 16 * E)
    rec("mpz_addmul", "k_mpz_mulops", timed(lambda: gbmm.mpz_addmul(p, mats["s"], mats["t"])),
        E * (4 * (16 + 16 + 33 + 33) + 16), 16 * 16 * E)
    if rank != 0:
        return 0
    line = {
        "metric": "GB/s per limb-form kernel", "value": max(r["GB/s"] for r in out.values()), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": W["label"], "hbm_peak_gbs": hbm, "mac_peak": peak, "operands": nb, "limbs": n,
                   "l2": "every batch is larger than L2"},
        "kernels": out,
    }
    print(json.dumps(line))
    return 0


def run_batched(args, W, world, rank, local):
    """Configuration 4: many uneven products through one gbmm_matmul_batched
    call per step (persistent work-queue kernel, CRT jobs, CUDA-graph replay)."""
    import torch
    import gbmm
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    mats, macs = gen_jobs(gbmm, W, args.seed)
    h = gbmm.Handle()
    jobs = h.jobs([(c, a, b) for c, a, b, _ in mats])
    chosen = h.matmul_batched(jobs)
    torch.cuda.synchronize()
    check_jobs(mats, "batched")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device="cuda")
    for _ in range(max(args.warmup, 0)):
        h.matmul_batched(jobs)
    torch.cuda.synchronize()
    barrier(world)
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = gbmm.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(i)
        ev[i][0].record(stream)
        h.matmul_batched(jobs)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = gbmm.kernel_launches() - launches0
    clocks = sampler.stop()
    ms = max_over_ranks(world, sum(a.elapsed_time(b) for a, b in ev) / args.steps)
    if rank != 0:
        return 0
    npath = {p: chosen.count(p) for p in set(chosen)}
    line = {
        "metric": "limb-MAC/s", "value": world * macs / (ms * 1e-3), "unit": "limb-MAC/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16+u32", "data": "synthetic",
        "config": {"workload": W["label"], "seed": args.seed, "limb_macs_per_step": macs,
                   "paths": {("crt" if p == gbmm.PATH_CRT else "limb"): c for p, c in npath.items()},
                   "graph": "captured on the second call, replayed in the timed steps",
                   "l2": "flushed between timed steps (512 MiB write)"},
        "gpu_launches": int(launches), "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbmm", choices=["gbmm", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--path", default=DEFAULT_PATH, choices=["limb", "crt", "auto"])
    ap.add_argument("--method", default="winograd", choices=["winograd", "naive", "strassen"])
    ap.add_argument("--cutoff", type=int, default=0)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--check", type=int, default=16)
    ap.add_argument("--profile-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=4.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-limb", action="store_true", help="skip the plain limb form's figure")
    ap.add_argument("--limb-cutoff", type=int, default=32)
    ap.add_argument("--limb-steps", type=int, default=2)
    ap.add_argument("--stream-jobs", type=int, default=10000, help="configuration 5: jobs in the evaluated stream")
    ap.add_argument("--jobs", type=int, default=0,
                    help="configuration 4: draw only the first N of its products (small cases for profiling)")
    ap.add_argument("--size", type=int, default=0,
                    help="override K=M=N of a single-product workload (small cases for profiling)")
    ap.add_argument("--bits", type=int, default=0, help="override the entry bit length")
    ap.add_argument("--shape", default="", help="override K,M,N (C is KxN, inner dimension M)")
    args = ap.parse_args()
    W = WORKLOADS[args.workload]
    if args.jobs and args.workload == "cfg4":
        W = dict(W, jobs=min(args.jobs, W["jobs"]),
                 label=f"the first {min(args.jobs, W['jobs'])} of " + W["label"] + " (profiling subset)")
    if (args.size or args.bits or args.shape) and args.workload not in ("cfg4", "cfg5"):
        K = M = N = args.size or W["K"]
        if args.shape:
            K, M, N = (int(x) for x in args.shape.split(","))
        b = args.bits or W["bits"]
        W = dict(W, K=K, M=M, N=N, bits=b, label=f"{K}x{M}x{N} {b}-bit signed (resized {args.workload})")
    world, rank, local = dist_init()
    if args.impl == "reference":
        if args.workload in ("cfg4", "cfg5", "limbkernels"):
            return run_reference(args, WORKLOADS["cfg3"], world, rank)
        return run_reference(args, W, world, rank)
    if args.workload in ("cfg4", "cfg5"):
        # batched calls run on a stream of their own: a handle bound to the legacy
        # default stream runs every batch eagerly, one on a real stream captures its
        # launch sequence into a CUDA graph on the second call and replays it after
        import torch
        torch.cuda.set_device(local)
        with torch.cuda.stream(torch.cuda.Stream()):
            if args.workload == "cfg4":
                return run_batched(args, W, world, rank, local)
            return run_learned(args, W, world, rank, local)
    if args.workload == "limbkernels":
        return run_limb_kernels(args, W, world, rank, local)
    return run_gpu(args, W, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
