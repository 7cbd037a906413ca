#!/usr/bin/env python3
"""bench.py -- exact polynomial-matrix product (and pmbasis) on one GB300.

Headline workload: nmod_poly_mat_mul of two 64x64 polynomial matrices, every
entry of length 4096 (degree < 4096), p = 998244353, coefficients uniform in
[0, p) from a seed (uint64 storage): forward NTT of length 8192, 8192 pointwise
64x64x64 products mod p, inverse NTT.  One "step" = one full product.
`value` is the time of one product with the tensor-core form (FP16 digits on
tcgen05: GB300 has no tcgen05 INT8 kind), inputs resident in HBM (268 MB of
inputs, larger than L2, so no flush is needed).  The INT8 split-limb form
(mma.sync) and the CUDA-core form of the same pipeline are timed beside it;
also reported: pmbasis of a 64x32 matrix at order 8192 (zero shift), the
pointwise contraction alone (4096 batched 64x64 products) and 256 batched
uneven products, each for every form.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl pml|reference]

With N > 1 (torchrun, one rank per GPU) every rank runs an independent
replica (the product does not shard across GPUs here): barrier + max over
ranks, rank 0 prints.  --impl reference times the CPU restatement of the
reference algorithm (the reference itself needs FLINT, which is not
installed) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

P = 998244353
R = K = C = 64
LEN = 4096
PM_M, PM_N, PM_ORDER = 64, 32, 8192
P60 = 576460752303423619   # the reference's 60-bit test prime (testing_collection.h:16-20)
WORKLOAD = "nmod_poly_mat_mul 64x64 . 64x64, len 4096 (deg < 4096), p = 998244353, uniform coefficients"
METRIC = "exact poly_mat_mul & pmbasis time: INT8 split-limb TC vs CUDA-core form, 1 GB300"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["pml", "reference"], default="pml")
    ap.add_argument("--no-pmbasis", action="store_true", help="skip the pmbasis measurement")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the pointwise-batch and batched-uneven measurements")
    ap.add_argument("--profile-case", choices=["product", "pmbasis", "pwbatch", "uneven", "kernel", "layout", "dot",
                                               "pmbasis_word"],
                    default=None,
                    help="run one product per form (or one pmbasis at order 1024, one 4096-product "
                         "pointwise batch per form, one batched-uneven call with the FP16 form, one kernel "
                         "basis of a 64x32 degree-255 matrix, one layout conversion each way at 64x64 x 4096, "
                         "one call of each dot-product kernel on about 256 MB, one pmbasis 64x32 at order 64 "
                         "modulo a 60-bit prime) and exit: the small cases for kernel captures")
    return ap.parse_args()


def run_profile_case(args):
    """One headline product with each form (FP16 digits, INT8, CUDA cores), or one pmbasis 64x32 at
    order 1024: a short, fixed launch sequence for profiler captures."""
    import torch
    import pml_gb300
    ctx = pml_gb300.Context(0)
    if args.profile_case == "product":
        A, B = make_inputs(1)
        dA = torch.from_numpy(A.view(np.int64)).cuda()
        dB = torch.from_numpy(B.view(np.int64)).cuda()
        outs = []
        for form in (pml_gb300.FORM_F16_TC, pml_gb300.FORM_INT8_TC, pml_gb300.FORM_CUDA_CORE):
            ctx.set_form(form)
            outs.append(pml_gb300.nmod_poly_mat_multiply(dA, dB, P, ctx=ctx))
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "product",
                          "forms_agree": all(bool(torch.equal(outs[0], o)) for o in outs),
                          "launches": ctx.launches}))
    elif args.profile_case == "pwbatch":
        forms = (("f16_tc", pml_gb300.FORM_F16_TC), ("int8_tc", pml_gb300.FORM_INT8_TC),
                 ("cuda_core", pml_gb300.FORM_CUDA_CORE))
        r = measure_pointwise_batch(ctx, torch.device("cuda", 0), torch.cuda.current_stream(), forms, 0)
        print(json.dumps({"profile_case": "pwbatch", "forms_agree": r["forms_agree"], "launches": ctx.launches}))
    elif args.profile_case == "uneven":
        ctx.set_form(pml_gb300.FORM_F16_TC)
        r = measure_batched_uneven(ctx, torch.device("cuda", 0), torch.cuda.current_stream(),
                                   (("f16_tc", pml_gb300.FORM_F16_TC),), 0)
        print(json.dumps({"profile_case": "uneven", "ms": r["f16_tc_ms"], "launches": ctx.launches}))
    elif args.profile_case == "kernel":
        rng = np.random.default_rng(21)
        F = torch.from_numpy(rng.integers(0, P, size=(64, 32, 256), dtype=np.uint64).view(np.int64)).cuda()
        ker, piv, rdeg = pml_gb300.nmod_poly_mat_kernel(F, [0] * 64, P, ctx=ctx)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "kernel", "nullity": int(ker.shape[0]), "launches": ctx.launches}))
    elif args.profile_case == "dot":
        import torch
        for name, (a, b, p, nbytes) in _dot_inputs(torch.device("cuda", 0), 61, shift=2).items():
            _dot_call(ctx, name, a, b, p)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "dot", "launches": ctx.launches}))
    elif args.profile_case == "layout":
        rng = np.random.default_rng(31)
        Pm = torch.from_numpy(rng.integers(0, P, size=(64, 64, 4096), dtype=np.uint64).view(np.int64)).cuda()
        M, L = pml_gb300.nmod_mat_poly_set_trunc_from_poly_mat(Pm, 4096, ctx=ctx)
        Q = pml_gb300.nmod_poly_mat_set_trunc_from_mat_poly(M, 4096, ctx=ctx)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "layout", "exact": bool(torch.equal(Pm, Q)), "launches": ctx.launches}))
    elif args.profile_case == "pmbasis_word":
        import oracle
        F = oracle.rand_poly_mat(PM_M, PM_N, 64, P60, 5)
        ab, sh = pml_gb300.nmod_poly_mat_pmbasis(torch.from_numpy(F.view(np.int64)).cuda(), 64, [0] * PM_M, P60,
                                                 ctx=ctx)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "pmbasis_word", "rdeg_sum": int(sum(sh)), "launches": ctx.launches}))
    else:
        rng = np.random.default_rng(7)
        F = rng.integers(0, P, size=(PM_M, PM_N, 1024), dtype=np.uint64)
        ab, sh = pml_gb300.nmod_poly_mat_pmbasis(torch.from_numpy(F.view(np.int64)).cuda(), 1024, [0] * PM_M, P,
                                                 ctx=ctx)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "pmbasis", "rdeg_sum": int(sum(sh)), "launches": ctx.launches}))
    ctx.close()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_inputs(seed: int):
    """Seeded synthetic inputs: uniform in [0, p) (numpy PCG64)."""
    rng = np.random.default_rng(seed)
    A = rng.integers(0, P, size=(R, K, LEN), dtype=np.uint64)
    B = rng.integers(0, P, size=(K, C, LEN), dtype=np.uint64)
    return A, B


def pointwise_batch_inputs(seed: int):
    """The pointwise contraction alone: 4096 pairs of 64x64 matrices, uint32 entries
    uniform in [0, p) (numpy PCG64)."""
    rng = np.random.default_rng(seed)
    A = rng.integers(0, P, size=(4096, 64, 64), dtype=np.uint32)
    B = rng.integers(0, P, size=(4096, 64, 64), dtype=np.uint32)
    return A, B


def pmbasis_input(seed: int):
    """pmbasis input: a 64x32 matrix of length 8192 (the order), coefficients uniform in [0, p)."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, P, size=(PM_M, PM_N, PM_ORDER), dtype=np.uint64)


def uneven_instances(seed: int):
    """The batched uneven workload: 256 products A_i B_i of square m_i x m_i matrices,
    m_i uniform in {4..48}, lengths 2^U(6,12), even i mod p = 998244353, odd i mod a
    seeded random 59-bit prime; coefficients uniform in [0, p_i)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(256):
        m = int(rng.integers(4, 49))
        ln = int(2 ** rng.uniform(6, 12))
        p = P if i % 2 == 0 else random_prime(59, rng)
        A = rng.integers(0, p, size=(m, m, ln), dtype=np.uint64)
        B = rng.integers(0, p, size=(m, m, ln), dtype=np.uint64)
        out.append((A, B, p))
    return out


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


# ---------------------------------------------------------------------------
# CPU legs (oracle port: the reference's algorithm restated in C)
# ---------------------------------------------------------------------------

def cpu_product_ms(nthreads: int, reps: int, warm: int):
    import oracle
    A, B = make_inputs(1)
    t = []
    for i in range(warm + reps):
        t0 = time.perf_counter()
        oracle.poly_mat_mul_ntt(A, B, P, nthreads=nthreads)
        dt = (time.perf_counter() - t0) * 1e3
        if i >= warm:
            t.append(dt)
    return statistics.median(t), t


def _timed(fn):
    t0 = time.perf_counter()
    fn()
    return (time.perf_counter() - t0) * 1e3


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_baselines():
    """The oracle (C restatement of the reference's algorithms; FLINT/PML are not installed)
    on the host cores for every workload of the benchmark set: 1 thread (the reference is
    single-threaded) and all cores, each on a bounded sample stated beside it."""
    import oracle
    nt = os.cpu_count() or 1
    res = {"cores_available": nt, "cpu": cpu_model(), "kind": "port"}
    A1 = oracle.rand_poly_mat(16, 16, 256, P, 101)
    B1 = oracle.rand_poly_mat(16, 16, 256, P, 102)
    res["c1_product_16x16_len256"] = {"ms_1_thread": statistics.median(
        [_timed(lambda: oracle.poly_mat_mul_ntt(A1, B1, P, nthreads=1)) for _ in range(5)]),
        "sample": "full workload, median of 5"}
    A2, B2 = pointwise_batch_inputs(11)
    res["c2_pointwise_batch_4096"] = {
        "ms_1_thread": _timed(lambda: oracle.nmod_mat_mul_batch_u32(A2, B2, P, nthreads=1)),
        "ms_all_cores": _timed(lambda: oracle.nmod_mat_mul_batch_u32(A2, B2, P, nthreads=nt)),
        "sample": "full workload (4096 products 64x64x64 mod p), one call each"}
    A3, B3 = make_inputs(1)
    res["c3_product_64x64_len4096"] = {
        "ms_1_thread": _timed(lambda: oracle.poly_mat_mul_ntt(A3, B3, P, nthreads=1)),
        "ms_all_cores": _timed(lambda: oracle.poly_mat_mul_ntt(A3, B3, P, nthreads=nt)),
        "sample": "full workload, one call each"}
    F = pmbasis_input(7)
    res["c4_pmbasis_64x32_order8192"] = {
        "ms_all_cores": _timed(lambda: oracle.pmbasis(F, PM_ORDER, [0] * PM_M, P, nthreads=nt)),
        "ms_1_thread_order1024": _timed(lambda: oracle.pmbasis(F[:, :, :1024], 1024, [0] * PM_M, P, nthreads=1)),
        "sample": "all cores: the full order-8192 call; 1 thread: the same input truncated to order 1024 "
                  "(the 1-thread full call would take minutes)"}
    Fw = oracle.rand_poly_mat(PM_M, PM_N, 256, P60, 61)
    res["pmbasis_64x32_order256_p60"] = {
        "ms_all_cores": _timed(lambda: oracle.pmbasis(Fw, 256, [0] * PM_M, P60, nthreads=nt)),
        "sample": "pmbasis 64x32 at order 256 modulo the 60-bit prime, all cores, one call"}
    inst = uneven_instances(5)
    sub = inst[:64]
    macs = lambda L: sum(A.shape[0] ** 3 * A.shape[2] for A, _, _ in L)
    res["c5_batched_uneven_256"] = {
        "ms_all_cores_first64": _timed(lambda: [oracle.poly_mat_mul_fast(A, B, p, nthreads=nt) for A, B, p in sub]),
        "sample": f"the first 64 of the 256 instances ({macs(sub) / macs(inst):.3f} of the coefficient MACs), "
                  "all cores; oracle products: single-prime NTT for p = 998244353, multi-prime NTT + CRT otherwise"}
    return res


def rank_barrier(world: int) -> None:
    """Barrier across the replicas (no-op for one process)."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int, device) -> float:
    """Slowest replica's time: the job is done when the last rank is."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return   # the reference arm runs on rank 0 only; the other ranks exit without work
    nthreads = os.cpu_count() or 1
    med, ts = cpu_product_ms(nthreads, max(args.steps, 1), max(args.warmup, 0))
    line = {
        "impl": "reference", "metric": METRIC, "value": med, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": med, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded uniform [0,p))",
        "config": {"workload": WORKLOAD, "implementation": "CPU evaluation/interpolation product (NTT at "
                   "2^13-th roots of unity, one 64x64 matrix product mod p per point), C restatement of "
                   "flint-extras mul_geometric.c; FLINT/PML themselves are not installed",
                   "threads": nthreads},
        "cpu_baseline": {"value": med, "unit": "ms", "cores": nthreads, "kind": "port",
                         "sample": f"full product per step, {nthreads} OpenMP threads"},
        "e2e": {"value": med, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

# DRAM bytes (read + write) per launch of the dominant kernels at the headline workload: constants
# from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of
# `python bench.py --profile-case product`, a cold, single capture, so part of the output is
# still in L2 when the kernel ends
TRAFFIC_SOURCE = ("constant from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of "
                  "`python bench.py --profile-case product`, not measured in this run")
NCU_TRAFFIC = {"ntt_fwd": 216.6e6, "ntt_inv": 347.2e6, "pointwise_f16_tc": 368.2e6,
               "pointwise_int8_tc": 370.8e6, "pointwise_cuda_core": 367.1e6}


def algorithmic_bytes(kernel: str):
    """Algorithmic HBM bytes (or int8 ops) per launch of each kernel at the headline workload."""
    N = 8192
    ent_in = R * K            # = K * C
    if kernel == "ntt_fwd":
        return ("hbm", ent_in * (LEN * 8 + N * 4))          # read uint64 coefficients, write uint32 evaluations
    if kernel == "ntt_inv":
        return ("hbm", R * C * (N * 4 + (2 * LEN - 1) * 8))  # read evaluations, write uint64 coefficients
    if kernel == "pointwise_int8_tc":
        return ("tensor", 2 * 16 * N * R * K * C)           # 16 limb products per MAC, 2 ops per MAC
    if kernel == "pointwise_f16_tc":
        return ("tensor", 2 * 12 * N * R * K * C)           # 12 digit products per MAC on FP16 tensor cores
    if kernel == "pointwise_cuda_core":
        return ("hbm", 3 * N * R * C * 4)
    return ("hbm", None)


def is_prime64(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 2^64 (bases: the first 12 primes)."""
    if n < 2:
        return False
    small = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)
    for q in small:
        if n % q == 0:
            return n == q
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in small:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def random_prime(bits: int, rng) -> int:
    while True:
        n = int(rng.integers(1 << (bits - 1), 1 << bits, dtype=np.uint64)) | 1
        if is_prime64(n):
            return n


def _time_calls(fn, st, reps: int, warm: int):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        out = fn()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, out


def measure_pointwise_batch(ctx, dev, st, forms, rank):
    """4096 independent products 64x64 . 64x64 mod p = 998244353, uint32 storage, one
    pmlg_nmod_mat_mul_batch_u32 call per form (the pointwise contraction alone)."""
    import torch
    import pml_gb300
    nb = 4096
    hA, hB = pointwise_batch_inputs(11 + rank)
    A = torch.from_numpy(hA.view(np.int32)).to(dev)
    B = torch.from_numpy(hB.view(np.int32)).to(dev)
    res, outs = {}, {}
    for name, form in forms:
        ctx.set_form(form)
        ms, out = _time_calls(lambda: pml_gb300.nmod_mat_mul_batch(A, B, P, ctx=ctx), st, 5, 2)
        res[name + "_ms"] = ms
        res[name + "_gmac_per_s"] = nb * 64 ** 3 / ms / 1e6
        outs[name] = out
    ref = outs.get("cuda_core", next(iter(outs.values())))
    res["forms_agree"] = all(bool(torch.equal(ref, o)) for o in outs.values())
    res["config"] = "4096 products 64x64 . 64x64 mod 998244353, uint32 entries uniform in [0, p), batch-major"
    return res


def measure_batched_uneven(ctx, dev, st, forms, rank):
    """256 independent nmod_poly_mat_mul instances in one pmlg_poly_mat_mul_batch call: square
    sizes m uniform in {4..48}, lengths 2^U(6,12), half p = 998244353, half seeded 59-bit primes."""
    import torch
    import pml_gb300
    jobs, macs = [], 0
    for hA, hB, p in uneven_instances(5 + rank):
        m, ln = hA.shape[0], hA.shape[2]
        A = torch.from_numpy(hA.view(np.int64)).to(dev)
        B = torch.from_numpy(hB.view(np.int64)).to(dev)
        jobs.append((A, B, p))
        macs += m ** 3 * ln
    res, outs = {}, {}
    for name, form in forms:
        ctx.set_form(form)
        # outputs allocated once: the repeated batch is replayed from a CUDA graph
        bufs = [torch.empty((A.shape[0], B.shape[1], A.shape[2] + B.shape[2] - 1), dtype=torch.int64, device=dev)
                for A, B, _ in jobs]
        # two warm-up calls: the first launches directly, the second captures the graph
        ms, out = _time_calls(lambda: pml_gb300.nmod_poly_mat_multiply_batch(jobs, ctx=ctx, out=bufs), st, 3, 2)
        res[name + "_ms"] = ms
        outs[name] = out
        if name == "f16_tc":
            ctx.set_batch_graphs(False)
            res[name + "_direct_ms"], _ = _time_calls(
                lambda: pml_gb300.nmod_poly_mat_multiply_batch(jobs, ctx=ctx, out=bufs), st, 3, 1)
            ctx.set_batch_graphs(True)
    ref = outs.get("cuda_core", next(iter(outs.values())))
    res["forms_agree"] = all(all(bool(torch.equal(a, b)) for a, b in zip(ref, o)) for o in outs.values())
    res["config"] = ("256 instances, m uniform in {4..48}, length 2^U(6,12), half p = 998244353, "
                     "half seeded 59-bit primes (CRT over NTT primes), uniform coefficients; "
                     "repeated calls replay a CUDA graph (*_direct_ms: every kernel launched directly)")
    res["coefficient_macs"] = macs
    return res


def measure_kernel_basis(ctx, dev, st, rank):
    """Left kernel basis of a 64x32 polynomial matrix of degree 1023, zero shift
    (nmod_poly_mat_kernel_zls_approx, kernel.c:232; the shape of the reference's
    p-kernel.c profiler): wall clock around one call (it synchronises internally)
    after one warm-up call, and K * F = 0 checked with the GPU product."""
    import time
    import torch
    import pml_gb300
    m, n, ln = 64, 32, 1024
    rng = np.random.default_rng(21 + rank)
    F = torch.from_numpy(rng.integers(0, P, size=(m, n, ln), dtype=np.uint64).view(np.int64)).to(dev)
    pml_gb300.nmod_poly_mat_kernel(F, [0] * m, P, ctx=ctx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ker, piv, rdeg = pml_gb300.nmod_poly_mat_kernel(F, [0] * m, P, ctx=ctx)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    zero = not bool(pml_gb300.nmod_poly_mat_multiply(ker, F, P, ctx=ctx).any().item())
    return {"ms": ms, "nullity": int(ker.shape[0]), "basis_length": int(ker.shape[2]), "kernel_times_F_zero": zero,
            "config": "kernel basis of a 64x32 matrix, degree 1023, zero shift, p = 998244353, uniform coefficients",
            "timing": "wall clock around one call after one warm-up call"}


def _dot_inputs(dev, seed: int, shift: int = 0):
    """About 1 GB >> shift of operands per dot-product kernel (larger than L2 for shift <= 2,
    no flush needed)."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    # entries in [0, hi) drawn as int64; 32-bit operands keep the low 32 bits of each
    rnd = lambda n, dt, hi: torch.randint(0, hi, (n,), dtype=torch.int64, device=dev, generator=g).to(dt)
    p64, p32 = 2 ** 61 - 1, 4294967291
    n64, n32, rows = 1 << (26 - shift), 1 << (27 - shift), 8192 >> shift
    return {
        "dot64": (rnd(n64, torch.int64, p64), rnd(n64, torch.int64, p64), p64, 16 * n64),
        "dot32": (rnd(n32, torch.int32, p32), rnd(n32, torch.int32, p32), p32, 8 * n32),
        "mdot32": (rnd(rows * 32768, torch.int32, p32).view(rows, 32768), rnd(32768, torch.int32, p32), p32,
                   4 * rows * 32768 + 4 * 32768),
        "dot_multi": (rnd(rows // 2, torch.int64, p64), rnd(rows // 2 * 32768, torch.int64, p64).view(rows // 2, 32768),
                      p64, 8 * (rows // 2) * 32768 + 8 * (rows // 2)),
    }


def _dot_call(ctx, name, a, b, p):
    import pml_gb300
    if name == "dot64":
        return pml_gb300.nmod_vec_dot_product(a, b, p, ctx=ctx)
    if name == "dot32":
        return pml_gb300.nmod32_vec_dot_product(a, b, p, ctx=ctx)
    if name == "mdot32":
        return pml_gb300.nmod32_vec_mdot(a, b, p, ctx=ctx)
    return pml_gb300.nmod_vec_dot_product_multi(a, b, p, ctx=ctx)


def measure_dot_products(ctx, dev, st, rank, peak_gbs):
    """The modular dot products (nmod_vec_dot_product_unbalanced, _nmod32_vec_dot_split,
    _nmod32_vec_mdot_split, nmod_vec_dot_product_multi) on about 1 GB of operands each:
    device time of the kernels (CUDA events through the context's profiling), algorithmic
    bytes = every operand entry read once, as a fraction of the measured HBM copy rate."""
    import torch
    res = {}
    for name, (a, b, p, nbytes) in _dot_inputs(dev, 61 + rank).items():
        for _ in range(3):
            _dot_call(ctx, name, a, b, p)
        torch.cuda.synchronize()
        ctx.set_profiling(True)
        for _ in range(10):
            _dot_call(ctx, name, a, b, p)
        torch.cuda.synchronize()
        prof = ctx.profile()
        ctx.set_profiling(False)
        us = sum(v[0] for v in prof.values()) / 10 * 1e3
        gbs = nbytes / us / 1e3
        res[name] = {"us": us, "gbs": gbs, "frac_of_measured_hbm": gbs / peak_gbs if peak_gbs else None,
                     "bytes": nbytes, "kernels": sorted(prof)}
    res["config"] = ("dot64: 2^26 entries mod 2^61-1; dot32: 2^27 entries mod 4294967291; mdot32: 8192 x 32768 "
                     "matrix times vector; dot_multi: 4096-vector times 4096 x 32768 matrix")
    return res


def measure_layout(ctx, dev, st, rank, peak_gbs):
    """Entry-major -> coefficient-major and back for a 64x64 matrix of length 4096
    (nmod_mat_poly_set_trunc_from_poly_mat / nmod_poly_mat_set_trunc_from_mat_poly):
    CUDA events around 10 calls each, 16 bytes of traffic per coefficient (inputs of
    134 MB, larger than L2, so no flush is needed)."""
    import torch
    import pml_gb300
    r = c = 64
    ln = 4096
    rng = np.random.default_rng(31 + rank)
    Pm = torch.from_numpy(rng.integers(0, P, size=(r, c, ln), dtype=np.uint64).view(np.int64)).to(dev)
    M = torch.empty((ln, r, c), dtype=torch.int64, device=dev)
    Q = torch.empty((r, c, ln), dtype=torch.int64, device=dev)
    fwd = lambda: pml_gb300.nmod_mat_poly_set_trunc_from_poly_mat(Pm, ln, ctx=ctx, out=M)
    # the forward call reads the length back (a synchronisation), so time it without
    fwd_nolen = lambda: ctx.check(ctx.lib.pmlg_poly_mat_to_mat_poly(ctx.handle, M.data_ptr(), ln, Pm.data_ptr(), r,
                                                                     c, ln, ln, ln, None, st.cuda_stream))
    bwd = lambda: pml_gb300.nmod_poly_mat_set_trunc_from_mat_poly(M, ln, ctx=ctx, out=Q)
    fwd()
    t_f, _ = _time_calls(fwd_nolen, st, 10, 3)
    t_b, _ = _time_calls(bwd, st, 10, 3)
    ok = bool(torch.equal(Pm, Q))
    nbytes = 2 * r * c * ln * 8
    res = {"to_mat_poly_ms": t_f, "to_poly_mat_ms": t_b, "round_trip_exact": ok,
           "to_mat_poly_gbs": nbytes / t_f / 1e6, "to_poly_mat_gbs": nbytes / t_b / 1e6,
           "config": "64x64 polynomial matrix, length 4096, uint64 coefficients (134 MB each way)"}
    if peak_gbs:
        res["frac_of_measured_hbm"] = max(res["to_mat_poly_gbs"], res["to_poly_mat_gbs"]) / peak_gbs
    return res


def measure_dixon(ctx, dev, st, rank):
    """x-adic Dixon lifting (nmod_poly_mat_dixon.c:92): A 32x32 of degree 63, B 32x32 of
    degree 63, digits of 64 coefficients up to sigma = 4096; wall clock around one call
    (it synchronises) after one warm-up call, and A X = B mod x^sigma checked with the GPU
    product."""
    import time
    import torch
    import pml_gb300
    n, m, ln, order, sigma = 32, 32, 64, 64, 4096
    rng = np.random.default_rng(41 + rank)
    A = torch.from_numpy(rng.integers(0, P, size=(n, n, ln), dtype=np.uint64).view(np.int64)).to(dev)
    B = torch.from_numpy(rng.integers(0, P, size=(n, m, ln), dtype=np.uint64).view(np.int64)).to(dev)
    pml_gb300.nmod_poly_mat_dixon(A, B, order, sigma, P, ctx=ctx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    X, ok = pml_gb300.nmod_poly_mat_dixon(A, B, order, sigma, P, ctx=ctx)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    AX = pml_gb300.nmod_poly_mat_multiply(A, X, P, ctx=ctx)[:, :, :sigma]
    Bs = torch.zeros((n, m, sigma), dtype=torch.int64, device=dev)
    Bs[:, :, :ln] = B
    return {"ms": ms, "invertible": ok, "AX_equals_B_mod_x_sigma": bool(torch.equal(AX, Bs)),
            "config": "Dixon lifting, A and B 32x32 of degree 63, digits of 64, sigma = 4096, p = 998244353",
            "timing": "wall clock around one call after one warm-up call"}


def measure_pmbasis_word(ctx, dev, st, rank):
    """pmbasis of a 64x32 matrix modulo the reference's 60-bit test prime (the 64-bit leaf and
    the products by CRT over NTT primes), zero shift, at orders 256 and 1024; wall clock
    around one call (it synchronises) after one warm-up call."""
    import time
    import torch
    import pml_gb300
    out = {}
    for order in (256, 1024):
        rng = np.random.default_rng(61 + rank)
        F = torch.from_numpy((rng.integers(0, P60, size=(PM_M, PM_N, order), dtype=np.uint64)).view(np.int64)).to(dev)
        pml_gb300.nmod_poly_mat_pmbasis(F, order, [0] * PM_M, P60, ctx=ctx)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ab, sh = pml_gb300.nmod_poly_mat_pmbasis(F, order, [0] * PM_M, P60, ctx=ctx)
        torch.cuda.synchronize()
        out[f"order{order}_ms"] = (time.perf_counter() - t0) * 1e3
        out[f"order{order}_rdeg_sum"] = int(sum(sh))
    out["config"] = f"pmbasis 64x32, zero shift, p = {P60} (60 bits), uniform coefficients"
    out["timing"] = "wall clock around one call after one warm-up call"
    return out


def measure_popov(ctx, dev, st, rank):
    """Shift-Popov approximant basis of a 64x32 matrix at order 1024, zero shift
    (popov_pmbasis: two pmbasis calls and the leading-matrix normalisation); wall clock
    around one call (it synchronises) after one warm-up call."""
    import time
    import torch
    import pml_gb300
    m, n, order = 64, 32, 1024
    rng = np.random.default_rng(51 + rank)
    F = torch.from_numpy(rng.integers(0, P, size=(m, n, order), dtype=np.uint64).view(np.int64)).to(dev)
    pml_gb300.nmod_poly_mat_popov_pmbasis(F, order, [0] * m, P, ctx=ctx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ab, sh = pml_gb300.nmod_poly_mat_popov_pmbasis(F, order, [0] * m, P, ctx=ctx)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    pml_gb300.nmod_poly_mat_pmbasis(F, order, [0] * m, P, ctx=ctx)
    torch.cuda.synchronize()
    ms_pm = (time.perf_counter() - t0) * 1e3
    return {"ms": ms, "pmbasis_ms": ms_pm, "rdeg_sum": int(sum(sh)), "length": int(ab.shape[2]),
            "config": "shift-Popov approximant basis of a 64x32 matrix at order 1024, zero shift, p = 998244353",
            "timing": "wall clock around one call after one warm-up call"}


def run_pml(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import pml_gb300
    from pml_gb300 import _lib

    ctx = pml_gb300.Context(local)
    st = torch.cuda.current_stream(dev)

    A, B = make_inputs(1 + rank)
    dA = torch.from_numpy(A.view(np.int64)).to(dev)
    dB = torch.from_numpy(B.view(np.int64)).to(dev)
    dC = torch.empty((R, C, 2 * LEN - 1), dtype=torch.int64, device=dev)

    def step():
        ctx.check(ctx.lib.pmlg_poly_mat_mul(ctx.handle, dC.data_ptr(), dA.data_ptr(), dB.data_ptr(),
                                            R, K, C, LEN, LEN, P, st.cuda_stream))

    def barrier():
        rank_barrier(world)

    def ranks_max(x: float) -> float:
        return max_over_ranks(x, world, dev)

    def timed(form: int, steps: int, warmup: int, clocks=False):
        ctx.set_form(form)
        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if clocks else None
        if sampler:
            sampler.__enter__()
        l0 = ctx.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            step()
        e1.record(st)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__(None, None, None)
        ms = e0.elapsed_time(e1) / steps
        return ranks_max(ms), ctx.launches - l0, (sampler.summary() if sampler else None)

    FORMS = (("f16_tc", pml_gb300.FORM_F16_TC), ("int8_tc", pml_gb300.FORM_INT8_TC),
             ("cuda_core", pml_gb300.FORM_CUDA_CORE))
    HEAD = pml_gb300.FORM_F16_TC

    # correctness spot-check of this exact workload before timing: all forms equal
    outs_chk = {}
    for name, form in FORMS:
        ctx.set_form(form)
        step()
        outs_chk[name] = dC.clone()
    torch.cuda.synchronize()
    forms_agree = all(bool(torch.equal(outs_chk["cuda_core"], v)) for v in outs_chk.values())
    del outs_chk

    ms = {}
    ms["f16_tc"], launches, clocks = timed(HEAD, args.steps, args.warmup, clocks=True)
    ms["int8_tc"], _, _ = timed(pml_gb300.FORM_INT8_TC, args.steps, args.warmup)
    ms["cuda_core"], _, _ = timed(pml_gb300.FORM_CUDA_CORE, args.steps, args.warmup)

    # per-kernel device times (separate pass, events on the launch stream)
    def kernel_profile(form: int, steps: int):
        ctx.set_form(form)
        step()
        torch.cuda.synchronize()
        ctx.set_profiling(True)
        for _ in range(steps):
            step()
        torch.cuda.synchronize()
        prof = ctx.profile()
        ctx.set_profiling(False)
        return prof

    profs = {name: kernel_profile(form, args.steps) for name, form in FORMS}

    def summarize(prof):
        tot = sum(v[0] for v in prof.values()) or 1.0
        return {k: {"ms_per_launch": v[0] / v[1], "launches": v[1], "share": v[0] / tot} for k, v in prof.items()}

    prof_h = profs["f16_tc"]
    dom = max(prof_h, key=lambda k: prof_h[k][0])
    bound, work = algorithmic_bytes(dom)
    avg_s = prof_h[dom][0] / prof_h[dom][1] / 1e3
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    roofline = None
    if work is not None:
        if bound == "hbm":
            peak = peaks.get("hbm_gbs", 6800.0)
            ach = work / avg_s / 1e9
            roofline = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                        "frac": ach / peak, "traffic": NCU_TRAFFIC.get(dom),
                        "traffic_unit": "bytes per launch (ncu)", "traffic_source": TRAFFIC_SOURCE,
                        "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                        "algorithmic_bytes_per_launch": work}
        else:
            peak = peaks.get("bf16_tflops", 1900.0)
            ach = work / avg_s / 1e12
            roofline = {"bound": "tensor", "kernel": dom, "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                        "frac": ach / peak, "traffic": NCU_TRAFFIC.get(dom),
                        "traffic_unit": "bytes per launch (ncu)", "traffic_source": TRAFFIC_SOURCE,
                        "peak_source": "measured dense bf16 (burst)" if "bf16_tflops" in peaks else "fallback",
                        "algorithmic_ops_per_launch": work}

    # the pointwise kernel beside it, against both of its roofs: FP16 digit-product rate against
    # the dense bf16 peak, and its algorithmic bytes (A and B read, C written, uint32) against HBM
    roofline_pw = None
    if "pointwise_f16_tc" in prof_h:
        pw_s = prof_h["pointwise_f16_tc"][0] / prof_h["pointwise_f16_tc"][1] / 1e3
        flop = algorithmic_bytes("pointwise_f16_tc")[1]
        pw_bytes = 3 * 8192 * R * C * 4
        tpk = peaks.get("bf16_tflops", 1900.0)
        hpk = peaks.get("hbm_gbs", 6800.0)
        roofline_pw = {"kernel": "pointwise_f16_tc", "ms_per_launch": pw_s * 1e3,
                       "tensor": {"achieved": flop / pw_s / 1e12, "peak": tpk, "unit": "TFLOP/s",
                                  "frac": flop / pw_s / 1e12 / tpk,
                                  "ops_per_launch": flop, "ops": "12 FP16 digit products per modular MAC x 2"},
                       "hbm": {"achieved": pw_bytes / pw_s / 1e9, "peak": hpk, "unit": "GB/s",
                               "frac": pw_bytes / pw_s / 1e9 / hpk, "algorithmic_bytes_per_launch": pw_bytes},
                       "traffic": NCU_TRAFFIC.get("pointwise_f16_tc"), "traffic_source": TRAFFIC_SOURCE}

    # end to end through the host-buffer entry point, pinned host memory
    hA = torch.from_numpy(A.view(np.int64)).pin_memory()
    hB = torch.from_numpy(B.view(np.int64)).pin_memory()
    hC = torch.empty((R, C, 2 * LEN - 1), dtype=torch.int64).pin_memory()
    ctx.set_form(HEAD)

    def e2e_step():
        ctx.check(ctx.lib.pmlg_poly_mat_mul_host(ctx.handle, hC.data_ptr(), hA.data_ptr(), hB.data_ptr(),
                                                 R, K, C, LEN, LEN, P, st.cuda_stream))
    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        e2e_step()
    e1.record(st)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = ranks_max(e0.elapsed_time(e1) / args.steps)
    e2e_ok = bool(torch.equal(hC, dC.cpu()))
    h2d = 2 * R * K * LEN * 8
    d2h = R * C * (2 * LEN - 1) * 8

    # pmbasis 64x32, order 8192, every form (one warm-up call, then the median of three timed calls)
    pm = None
    if not args.no_pmbasis:
        F = pmbasis_input(7 + rank)
        dF = torch.from_numpy(F.view(np.int64)).to(dev)
        pm = {}
        outs = {}
        for name, form in FORMS:
            ctx.set_form(form)
            pml_gb300.nmod_poly_mat_pmbasis(dF, PM_ORDER, [0] * PM_M, P, ctx=ctx)
            torch.cuda.synchronize()
            ts = []
            for _ in range(3):
                t0 = time.perf_counter()
                ab, sh = pml_gb300.nmod_poly_mat_pmbasis(dF, PM_ORDER, [0] * PM_M, P, ctx=ctx)
                torch.cuda.synchronize()
                ts.append((time.perf_counter() - t0) * 1e3)
            pm[name + "_ms"] = ranks_max(sorted(ts)[1])
            pm[name + "_ms_min"] = ranks_max(min(ts))
            outs[name] = (ab, sh)
        ctx.set_profiling(True)
        ctx.set_form(HEAD)
        pml_gb300.nmod_poly_mat_pmbasis(dF, PM_ORDER, [0] * PM_M, P, ctx=ctx)
        prof = ctx.profile()
        ctx.set_profiling(False)
        pm["kernels_f16_tc"] = summarize(prof)
        pm["forms_agree"] = all(bool(torch.equal(outs["cuda_core"][0], v[0])) and list(v[1]) == list(outs["cuda_core"][1])
                                for v in outs.values())
        pm["speedup_f16_tc_vs_cuda_core"] = pm["cuda_core_ms"] / pm["f16_tc_ms"]
        pm["speedup_int8_tc_vs_cuda_core"] = pm["cuda_core_ms"] / pm["int8_tc_ms"]
        pm["config"] = "pmbasis 64x32, order 8192, zero shift, p = 998244353, uniform coefficients"
        pm["timing"] = "median of three calls, wall clock around each (it synchronises internally), after one warm-up call"

    # N > 1: the headline product row-sharded over the ranks (pml_gb300.shard): each rank
    # transforms its rows of A and all of B, multiplies and interpolates its rows of C; the
    # blocks of C are all-gathered over NCCL.  Strong scaling: one product in total.
    sharded = None
    if world > 1:
        from pml_gb300.shard import poly_mat_mul_sharded, row_partition
        ctx.set_form(HEAD)
        for _ in range(args.warmup):
            poly_mat_mul_sharded(dA, dB, P, ctx=ctx)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            Cs = poly_mat_mul_sharded(dA, dB, P, ctx=ctx)
        e1.record(st)
        torch.cuda.synchronize()
        barrier()
        sh_ms = ranks_max(e0.elapsed_time(e1) / args.steps)
        e0.record(st)
        for _ in range(args.steps):
            poly_mat_mul_sharded(dA, dB, P, ctx=ctx, gather=False)
        e1.record(st)
        torch.cuda.synchronize()
        barrier()
        sh_ms_nog = ranks_max(e0.elapsed_time(e1) / args.steps)
        step()
        torch.cuda.synchronize()
        sharded = {"ms_with_allgather": sh_ms, "ms_without_allgather": sh_ms_nog,
                   "rows_per_rank": [b_ - a_ for a_, b_ in row_partition(R, world)],
                   "matches_single_gpu": bool(torch.equal(Cs, dC)), "scaling": "strong",
                   "config": "the headline product, rows of A and C split over the ranks, B transformed on "
                             "every rank, C all-gathered (NCCL)"}

    # the two other GPU workloads of the benchmark set: the pointwise contraction alone and the
    # batched uneven products (every form, CUDA events around each call)
    extra = {} if args.no_extra else {
        "pointwise_batch": measure_pointwise_batch(ctx, dev, st, FORMS, rank),
        "batched_uneven": measure_batched_uneven(ctx, dev, st, FORMS + (("auto", pml_gb300.FORM_AUTO),), rank),
        "kernel_basis": measure_kernel_basis(ctx, dev, st, rank),
        "layout_conversion": measure_layout(ctx, dev, st, rank, peaks.get("hbm_gbs")),
        "dot_products": measure_dot_products(ctx, dev, st, rank, peaks.get("hbm_gbs")),
        "dixon": measure_dixon(ctx, dev, st, rank),
        "popov_pmbasis": measure_popov(ctx, dev, st, rank),
        "pmbasis_word_prime": measure_pmbasis_word(ctx, dev, st, rank),
    }

    # CPU baseline (rank 0, N = 1): oracle port, 1 thread (the reference is single-threaded)
    cpu = None
    cpu_all = None
    if rank == 0 and world == 1 and not args.no_cpu:
        med, ts = cpu_product_ms(1, 1, 0)
        cpu = {"value": med, "unit": "ms", "cores": 1, "kind": "port",
               "sample": "one full 64x64 len-4096 product, CPU evaluation/interpolation port (C, 1 thread)"}
        cpu_all = cpu_baselines()

    if rank == 0:
        line = {
            "metric": METRIC, "value": ms["f16_tc"], "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms["f16_tc"], "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded uniform [0,p), numpy PCG64)",
            "config": {"workload": WORKLOAD,
                       "form": "f16_tc: exact split-digit tensor-core form (tcgen05 kind::f16, FP32 accumulate); "
                               "the INT8 split-limb form (mma.sync, GB300's legacy INT8 rate) is timed beside it",
                       "parallelism": f"replicas x{world}", "l2": "inputs 268 MB > 129 MB L2, no flush",
                       "transform": "N = 8192, 2 x 4096 forward + 4096 inverse NTTs"},
            "forms_ms": ms, "forms_agree": forms_agree,
            "speedup_f16_tc_vs_cuda_core": ms["cuda_core"] / ms["f16_tc"],
            "speedup_int8_tc_vs_cuda_core": ms["cuda_core"] / ms["int8_tc"],
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "pmlg_poly_mat_mul_host, pinned host buffers", "matches_device": e2e_ok},
            "gpu_launches": launches,
            "roofline": roofline,
            "roofline_pointwise": roofline_pw,
            "kernels": {name: summarize(pr) for name, pr in profs.items()},
            "clocks": clocks,
            "pmbasis": pm,
            **extra,
            "cpu_baseline": cpu,
            "cpu_baselines": cpu_all,
            "row_sharded": sharded,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.profile_case:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_pml(args)


if __name__ == "__main__":
    main()
