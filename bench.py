#!/usr/bin/env python3
"""Benchmark of the GB300 Magnus engine on the forward + VJP workload.

Workload (default, "config4"): 512 independent trajectories of d=32 matrices
A(t) = C0 + C1 t + C2 t^2 + C3 cos(5t), C_k ~ N(0, 1/d), float32, on [0, 1]
with S = 32769 samples, Boole, order n = 5, op = "sum", cotangent ~ N(0, 1):
one step = the forward (writing the engine's chunk checkpoints, one every
256 samples) plus the VJP that reuses them.  Metric: samples*order/s =
(instances * S * n) / step time.  Inputs (68.7 GB) are far larger than L2,
so no cache flush is needed between steps.

Printed JSON line (rank 0): value (device-resident, mixed precision), the
plain-FP64 throughput and the mixed/plain error on a subset, the dominant
kernel's roofline (CUDA-event timed), the CPU baseline (the C oracle, a
restatement of the reference recursion, on the host cores), the end-to-end
number through the public autograd API with pinned host buffers, and the SM
clocks sampled during the timed region.

``--impl reference`` times the reference algorithm on the host CPU instead
(the oracle port on every host thread), on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "magnus-dp_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "samples·order/s fwd+VJP"
UNIT = "samples·order/s"

CONFIG4 = dict(batch=512, d=32, samples=32769, n=5, integrator="Boole", op="sum", t0=0.0, tf=1.0, K=256)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=CONFIG4["batch"])
    ap.add_argument("--samples", type=int, default=CONFIG4["samples"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "plain"])
    ap.add_argument("--plain-subset", type=int, default=16)
    ap.add_argument("--e2e-batch", type=int, default=0,
                    help="instances of the end-to-end legs (0: the whole batch, if host memory allows)")
    ap.add_argument("--cpu-instances", type=int, default=0, help="0 = one per host thread")
    ap.add_argument("--cpu-samples", type=int, default=4097)
    ap.add_argument("--oracle-instances", type=int, default=4,
                    help="instances of the timed batch whose mixed output and dA are checked against the "
                         "FP64 oracle (full size, in the CPU leg)")
    ap.add_argument("--no-extras", action="store_true", help="skip plain/e2e/cpu legs (quick runs)")
    ap.add_argument("--workload", default="config4", choices=["config4", "config1", "config2", "config3"],
                    help="config4 = the headline fwd+VJP line; the others print their own measurement lines")
    ap.add_argument("--instances", type=int, default=0, help="config3: number of instances (0 = all 10000)")
    ap.add_argument("--dim", type=int, default=64, help="config2: matrix dimension (64 is the configuration; "
                                                         "128 profiles the d = 128 tensor-core kernel)")
    return ap.parse_args()


# ---------------------------------------------------------------- helpers
def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), p.get("sm_max_mhz", 2070.0), "measured"
    return 6800.0, 1900.0, 2070.0, "fallback"


def traffic_from_profiles(kernel, scale=1.0):
    """Per-launch DRAM bytes of `kernel` (full config4 launch) from the committed
    ncu summary profiles/traffic.txt, scaled to the launch being measured."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 2 and not line.startswith("#") and parts[0] == kernel:
                return float(parts[1]) * scale
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.tmp = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.tmp.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.tmp.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- CPU legs
def cpu_sample(instances, samples, threads, repeats=1):
    """The oracle (reference recursion restated in C) on `instances`
    config4-style trajectories with `samples` samples, forward + VJP (the
    VJP rebuilds the reference's carry, as compute_vjp without vjp_data does),
    float32, `threads` host threads.  Returns samples*order/s and seconds."""
    import oracle as O
    from magnus_gb300 import workloads
    c = CONFIG4
    Ck = workloads.config4_coeffs(seed=4, batch=instances, d=c["d"])
    A = workloads.config4_samples_np(Ck, samples=samples, dtype=np.float32)
    cot = workloads.config4_cotangent(batch=instances, d=c["d"])
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        O.batch(A, c["n"], c["t0"], c["tf"], c["op"], c["integrator"], threads=threads)
        O.batch(A, c["n"], c["t0"], c["tf"], c["op"], c["integrator"], cot=cot, threads=threads)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return instances * samples * c["n"] / best, best


def _oracle_instance(job):
    """FP64 forward (op sum) and VJP of one config4 instance by the collapsed
    restatement of the reference recursion (oracle/collapsed.py)."""
    import collapsed as Cl
    A, cot, n, t0, tf = job
    A64 = A.astype(np.float64)
    return Cl.forward(A64, n, t0, tf, "sum", "Boole"), Cl.vjp(A64, cot.astype(np.float64), n, t0, tf, "sum", "Boole")


def oracle_check(A, cot, out, dA, n, t0, tf):
    """Relative Frobenius error of the engine's mixed output and dA (from the
    timed steps) against the FP64 oracle on the same full-size instances;
    one spawned worker per instance."""
    import multiprocessing as mp
    t = time.perf_counter()
    jobs = [(A[i], cot[i], n, t0, tf) for i in range(A.shape[0])]
    saved = os.environ.get("OPENBLAS_NUM_THREADS")
    os.environ["OPENBLAS_NUM_THREADS"] = str(max(1, (os.cpu_count() or 1) // max(1, len(jobs))))
    try:
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            refs = pool.map(_oracle_instance, jobs)
    finally:
        if saved is None:
            os.environ.pop("OPENBLAS_NUM_THREADS", None)
        else:
            os.environ["OPENBLAS_NUM_THREADS"] = saved
    ro = np.stack([r[0] for r in refs])
    rg = np.stack([r[1] for r in refs])
    e_out = float(np.linalg.norm(out.astype(np.float64) - ro) / np.linalg.norm(ro))
    e_dA = float(np.linalg.norm(dA.astype(np.float64) - rg) / np.linalg.norm(rg))
    return {"out": e_out, "dA": e_dA, "instances": len(jobs), "checker": "oracle/collapsed.py (FP64)",
            "seconds": time.perf_counter() - t}


def pinned_host(shape, np_dtype):
    """Page-locked host tensor of exactly its size, from cudaHostAlloc through
    the engine library's CUDA runtime (torch's pinned allocator, the same
    kind of memory, rounds a block up to a power of two: 128 GB for the
    68.7 GB of config4's A; numpy memory registered with cudaHostRegister
    copied at 19-43 GB/s on the GB300 host against 66-211 GB/s).  Returns
    (tensor, release)."""
    import torch
    rt = None
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    if rt is None:
        raise RuntimeError("CUDA runtime library not found")
    count = int(np.prod(shape))
    nbytes = count * np.dtype(np_dtype).itemsize
    ptr = ctypes.c_void_p()
    rc = rt.cudaHostAlloc(ctypes.byref(ptr), ctypes.c_size_t(nbytes), ctypes.c_uint(0))
    if rc != 0:
        raise RuntimeError(f"cudaHostAlloc of {nbytes} bytes failed with CUDA error {rc}")
    buf = (ctypes.c_char * nbytes).from_address(ptr.value)
    arr = np.frombuffer(buf, dtype=np_dtype, count=count).reshape(shape)
    return torch.from_numpy(arr), (lambda: rt.cudaFreeHost(ptr))


def e2e_instances(B, bytes_per_instance):
    """Instances for the end-to-end legs: the whole batch when page-locked
    host buffers for its input and dA (two copies) fit in 70 % of the host's
    available memory, else as many as do."""
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    if avail is None:
        return min(B, 128)
    return max(1, min(B, int(0.7 * avail // (2 * bytes_per_instance))))


def cpu_model():
    """The host CPU's model name (lscpu / /proc/cpuinfo), for the CPU legs."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    inst = args.cpu_instances or threads
    for _ in range(args.warmup):
        cpu_sample(inst, args.cpu_samples, threads)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_sample(inst, args.cpu_samples, threads)
        times.append(dt)
    sec = sum(times) / len(times)
    value = inst * args.cpu_samples * CONFIG4["n"] / sec
    sample = (f"{inst} config4 trajectories (d=32, n=5, Boole, sum, float32) at S={args.cpu_samples} "
              f"(of 32769) per step, forward + VJP without carry")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "config4 fwd+VJP (bounded CPU sample)", "batch": CONFIG4["batch"],
                       "samples": CONFIG4["samples"], "dim": CONFIG4["d"], "n": CONFIG4["n"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- other configurations
def _plan(lib, _lib, probs, A, out, cot=None, dA=None):
    import ctypes as ct
    B = len(probs)
    P = (_lib.Problem * B)(*probs)

    def ptrs(ts):
        return None if ts is None else (ct.c_void_p * B)(*[t.data_ptr() for t in ts])

    plan = ct.c_void_p()
    _lib.check(lib.mgb_plan_create(P, B, ptrs(A), ptrs(out), ptrs(cot), ptrs(dA), ct.byref(plan)))
    return plan


def _describe(lib, plan):
    """The plan's segments: chunk kernel, the launch variant the autotuner
    picked and the per-variant times it measured."""
    import ctypes as ct
    need = lib.mgb_plan_describe(plan, None, 0)
    buf = ct.create_string_buffer(need)
    lib.mgb_plan_describe(plan, buf, need)
    return json.loads(buf.value.decode())["segments"]


def _time_graph(torch, fn, steps, warmup=3):
    fn()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fn()
    for _ in range(warmup):
        g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    del g
    return e0.elapsed_time(e1) / steps


def kernel_roofs(kernels, steps, B, S, d, n, K, plain=False):
    """Roofline of each timed kernel of the config4 step (CUDA-event times
    from the library's launch timing), per launch:

      chunk_local  (n-1) products of 2 d^3 flop per sample; reads A once
      chunk_vjp    3 (n-1) products per sample (forward recomputation,
                   A^T G, G P^T); reads A once, writes dA
      scan, rscan  n(n-1)/2 d x d products per chunk step; read the chunk
                   transfers, write the chunk states (FP64 arrays)
      fin_*        the per-instance FP64 algebra (latency-bound, no roof)

    Mixed-form products on the tensor cores are FP32-accurate emulations:
    three MMAs per product on two scaled FP16 pieces per operand (d = 32) or
    six on three BF16 pieces (d = 64/128), so their roof is the measured
    sustained BF16 rate / 3 (FP16 and BF16 dense rates are equal on this
    part).  The mixed-form scans run double-FP32
    arithmetic on the FP32 pipes (about six FP32 flops per emulated flop):
    roof = nominal FP32 rate (152 SMs x 128 lanes x 2 x max clock) / 6.  The
    plain form's products and scans are rated against the nominal FP64 rate
    (1.25 TFLOP/s; no measured peak).  bound = the roof the kernel is closer
    to; frac = achieved / that roof's peak."""
    hbm_peak, _, sm_max, src = load_peaks()
    fp32_nominal = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    fp64_nominal = 1.25
    m = d * d
    C = -(-(S - 1) // K)
    if plain:
        prod_roof = (fp64_nominal, "fp64", "nominal FP64")
        scan_roof = prod_roof
    else:
        prod_roof = (bf16_sustained_peak() / 3, "tensor", "3 MMAs per product = measured sustained BF16 / 3")
        scan_roof = (fp32_nominal / 6, "fp32", "double-FP32 = nominal FP32 / 6")
    work = {
        "chunk_local": ((n - 1) * 2.0 * d ** 3 * S * B, S * m * 4.0 * B, prod_roof),
        "chunk_vjp": (3 * (n - 1) * 2.0 * d ** 3 * S * B, 2 * S * m * 4.0 * B, prod_roof),
        "scan": (n * (n - 1) / 2 * 2.0 * d ** 3 * C * B, (2 * C + 1) * n * m * 8.0 * B, scan_roof),
        "rscan": (n * (n - 1) / 2 * 2.0 * d ** 3 * C * B, (2 * C) * n * m * 8.0 * B, scan_roof),
    }
    out = {}
    for name, (launches, total_ms, *_) in kernels.items():
        launch_ms = total_ms / max(launches, 1)
        per = launches / steps  # launches per step
        flops, nbytes, (fpeak, fbound, fsrc) = work.get(name, (0.0, 0.0, (None, None, None)))
        flops, nbytes = flops / per, nbytes / per
        t = launch_ms / 1e3
        tf = flops / t / 1e12 if flops else 0.0
        gbs = nbytes / t / 1e9 if nbytes else 0.0
        cfrac = tf / fpeak if fpeak else 0.0
        hfrac = gbs / hbm_peak
        if fpeak and cfrac >= hfrac:
            r = {"bound": fbound, "achieved": tf, "peak": fpeak, "unit": "TFLOP/s", "frac": cfrac, "peak_source": fsrc}
        else:
            r = {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": hfrac,
                 "peak_source": src + " HBM copy"}
        r.update({"ms_per_step": total_ms / steps, "launch_ms": launch_ms, "launches_per_step": per,
                  "compute_frac": cfrac, "hbm_frac": hfrac, "flops_per_launch": flops, "bytes_per_launch": nbytes})
        out[name] = r
    return out


def bf16_sustained_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f).get("bf16_tflops_sustained", 1700.0)
    return 1700.0


def _order_errors(mixed, plain):
    """Per-order relative Frobenius error; orders that vanish (< 1e-6 of the
    largest) are measured against the largest order's norm."""
    mixed = np.asarray(mixed, dtype=np.float64)
    plain = np.asarray(plain, dtype=np.float64)
    scale = max(np.linalg.norm(plain[..., k, :]) for k in range(plain.shape[-2]))
    errs = []
    for k in range(plain.shape[-2]):
        nk = np.linalg.norm(plain[..., k, :])
        den = nk if nk >= 1e-6 * scale else scale
        errs.append(float(np.linalg.norm(mixed[..., k, :] - plain[..., k, :]) / den))
    return errs


def run_config1(args):
    """4096 SpaceCurves, S=65537 on [0,2], Simpson, n=6, op=many, float32,
    forward (mixed) — HBM-bound on the 3-vector samples."""
    import ctypes as ct
    import torch
    from magnus_gb300 import _lib, workloads
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    B, S, n = (args.batch if args.batch != CONFIG4["batch"] else 4096), 65537, 6
    a, b = workloads.config1_coeffs(seed=1, batch=B)
    F = workloads.config1_samples_torch(a, b, samples=S, device=dev)
    out = torch.empty((B, n, 3), dtype=torch.float32, device=dev)
    mk = lambda prec: _lib.make_problem(kind=_lib.KIND_SPACECURVE, dtype_code=_lib.DTYPE_F32, precision=prec,  # noqa
                                        op=_lib.OP_MANY, integrator=1, n=n, samples=S, dim=2, t0=0.0, tf=2.0)
    plan = _plan(lib, _lib, [mk(_lib.PRECISION_MIXED)] * B, [F[i] for i in range(B)], [out[i] for i in range(B)])
    st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    ms = _time_graph(torch, lambda: _lib.check(lib.mgb_plan_forward(plan, ct.c_void_p(torch.cuda.current_stream().cuda_stream))), args.steps)
    lib.mgb_plan_destroy(plan)
    sub = 16
    out_p = torch.empty((sub, n, 3), dtype=torch.float32, device=dev)
    plan_p = _plan(lib, _lib, [mk(_lib.PRECISION_PLAIN)] * sub, [F[i] for i in range(sub)], [out_p[i] for i in range(sub)])
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _lib.check(lib.mgb_plan_forward(plan_p, st))
    e0.record()
    _lib.check(lib.mgb_plan_forward(plan_p, st))
    e1.record()
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    lib.mgb_plan_destroy(plan_p)
    errs = _order_errors(out[:sub].cpu().numpy(), out_p.cpu().numpy())
    bytes_alg = B * S * 3 * 4 + B * n * 3 * 4
    gbs = bytes_alg / (ms / 1e3) / 1e9
    hbm_peak = load_peaks()[0]
    print(json.dumps({"workload": "config1: 4096 SpaceCurves, S=65537, Simpson, n=6, many, float32, forward",
                      "metric": "samples·order/s forward", "value": B * S * n / (ms / 1e3), "ms": ms,
                      "precision": "mixed", "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak,
                                                         "unit": "GB/s", "frac": gbs / hbm_peak},
                      "plain_fp64": {"value": sub * S * n / (plain_ms / 1e3), "instances": sub},
                      "rel_err_per_order_vs_fp64": errs}))


def run_config2(args):
    """256 skew-symmetric d=64 A(t), S=16385, Boole, n=4, op=sum, float32,
    forward (mixed) — FP32-products-bound."""
    import ctypes as ct
    import torch
    from magnus_gb300 import _lib, workloads
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    B, S, n, d = (args.batch if args.batch != CONFIG4["batch"] else 256), 16385, 4, args.dim
    Sk = workloads.config2_coeffs(seed=2, batch=B, d=d)
    A = workloads.config2_samples_torch(Sk, samples=S, device=dev)
    out = torch.empty((B, d, d), dtype=torch.float32, device=dev)
    mk = lambda prec, op: _lib.make_problem(kind=0, dtype_code=_lib.DTYPE_F32, precision=prec, op=op,  # noqa
                                            integrator=0, n=n, samples=S, dim=d, t0=0.0, tf=1.0)
    plan = _plan(lib, _lib, [mk(_lib.PRECISION_MIXED, _lib.OP_SUM)] * B, [A[i] for i in range(B)],
                 [out[i] for i in range(B)])
    autotune = _describe(lib, plan)
    ms = _time_graph(torch, lambda: _lib.check(lib.mgb_plan_forward(plan, ct.c_void_p(torch.cuda.current_stream().cuda_stream))), args.steps)
    lib.mgb_plan_destroy(plan)
    sub = min(4, B)
    st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    res = {}
    for prec in (_lib.PRECISION_MIXED, _lib.PRECISION_PLAIN):
        o = torch.empty((sub, n, d, d), dtype=torch.float32, device=dev)
        pl = _plan(lib, _lib, [mk(prec, _lib.OP_MANY)] * sub, [A[i] for i in range(sub)], [o[i] for i in range(sub)])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        _lib.check(lib.mgb_plan_forward(pl, st))
        e0.record()
        _lib.check(lib.mgb_plan_forward(pl, st))
        e1.record()
        torch.cuda.synchronize()
        res[prec] = (o.cpu().numpy().reshape(sub, n, d * d), e0.elapsed_time(e1))
        lib.mgb_plan_destroy(pl)
    errs = _order_errors(res[_lib.PRECISION_MIXED][0], res[_lib.PRECISION_PLAIN][0])
    flops = (n - 1) * 2.0 * d ** 3 * S * B
    tf = flops / (ms / 1e3) / 1e12
    fp32_peak = 152 * 128 * 2 * load_peaks()[2] * 1e6 / 1e12
    print(json.dumps({"workload": f"config2: {B} x d={d} skew A(t), S=16385, Boole, n=4, sum, float32, forward",
                      "metric": "samples·order/s forward", "value": B * S * n / (ms / 1e3), "ms": ms,
                      "precision": "mixed", "fp32_simt": {"achieved_tflops": tf, "nominal_peak_tflops": fp32_peak,
                                                          "frac": tf / fp32_peak},
                      "plain_fp64": {"value": sub * S * n / (res[_lib.PRECISION_PLAIN][1] / 1e3), "instances": sub},
                      "rel_err_per_order_vs_fp64": errs, "autotune": autotune}))


def run_config3(args):
    """Uneven batch: d in {2..128}, S log-uniform in [257, 65537], n in 2..6,
    A as config0 at each d, float32; fwd+VJP in mixed precision.  The float32
    samples of all 10000 instances (~1.5 TB) exceed HBM, so instances run in
    waves of <= 48 GB; each wave is one plan (instances grouped by dimension,
    segments on concurrent streams) captured in a CUDA graph; sample
    generation between waves is outside the timed regions.  The plain FP64
    path is timed on a per-dimension subset for the mixed/plain ratio."""
    import ctypes as ct
    import torch
    from magnus_gb300 import _lib, workloads
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    ds, Ss, ns, seeds = workloads.config3_instances(seed=3, count=10000)
    count = args.instances or len(ds)
    order = np.arange(count)
    wave_bytes = 48 << 30
    total_ms, total_units = 0.0, 0
    per_d = {}

    def make_inst(i, prec):
        d, S, n = int(ds[i]), int(Ss[i]), int(ns[i])
        C, w = workloads.config0_coeffs(int(seeds[i]), d)
        t = torch.linspace(0.0, 1.0, S, dtype=torch.float64, device=dev)[:, None, None]
        Ct = torch.as_tensor(C, device=dev)
        A = (Ct[0] + Ct[1] * torch.sin(w[0] * t) + Ct[2] * torch.cos(w[1] * t)).to(torch.float32)
        cot = torch.ones((d, d), dtype=torch.float32, device=dev)
        prob = _lib.make_problem(kind=0, dtype_code=_lib.DTYPE_F32, precision=prec, op=_lib.OP_SUM, integrator=0,
                                 n=n, samples=S, dim=d, t0=0.0, tf=1.0)
        return A, cot, prob

    picks = {}  # autotuner picks over the timed waves: "d<d> <kernel> v<variant>" -> segments

    def run_wave(idx, prec, steps, record=False):
        As, cots, probs = [], [], []
        for i in idx:
            A, cot, p = make_inst(i, prec)
            As.append(A); cots.append(cot); probs.append(p)
        outs = [torch.empty((a.shape[1], a.shape[1]), dtype=torch.float32, device=dev) for a in As]
        dAs = [torch.empty_like(a) for a in As]
        plan = _plan(lib, _lib, probs, As, outs, cots, dAs)

        def step():
            s = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
            _lib.check(lib.mgb_plan_forward(plan, s))
            _lib.check(lib.mgb_plan_vjp(plan, s))

        ms = _time_graph(torch, step, steps, warmup=1)
        if record:
            for sg in _describe(lib, plan):
                key = f"d{sg['d']} {sg['kernel']} v{sg['variant']}"
                picks[key] = picks.get(key, 0) + 1
        lib.mgb_plan_destroy(plan)
        del As, dAs, outs
        torch.cuda.empty_cache()
        return ms

    wave, wbytes = [], 0
    for i in order:
        b = int(Ss[i]) * int(ds[i]) ** 2 * 4 * 2
        if wave and wbytes + b > wave_bytes:
            total_ms += run_wave(wave, _lib.PRECISION_MIXED, 1, record=True)
            wave, wbytes = [], 0
        wave.append(int(i))
        wbytes += b
        total_units += int(Ss[i]) * int(ns[i])
    if wave:
        total_ms += run_wave(wave, _lib.PRECISION_MIXED, 1, record=True)
    # Mixed vs plain on the same random subsets of each dimension; both arms
    # are extrapolated to the whole batch with the same work weights, so the
    # ratio compares like with like (the measured mixed total above is the
    # headline value; mixed_estimated checks the extrapolation against it).
    rng = np.random.default_rng(11)
    plain_est_s = mixed_est_s = 0.0
    for d in (2, 4, 8, 16, 32, 64, 128):
        cand = np.nonzero(ds[:count] == d)[0]
        if len(cand) == 0:
            continue
        sel = sorted(int(i) for i in rng.choice(cand, size=min(4, len(cand)), replace=False))
        units = sum(int(Ss[i]) * int(ns[i]) for i in sel)
        mixed_ms = run_wave(sel, _lib.PRECISION_MIXED, 1)
        plain_ms = run_wave(sel, _lib.PRECISION_PLAIN, 1)
        per_d[d] = {"mixed": units / (mixed_ms / 1e3), "plain_fp64": units / (plain_ms / 1e3),
                    "ratio": plain_ms / mixed_ms, "instances": len(sel)}
        work = lambda idx: sum(int(Ss[i]) * int(ns[i]) * d * d * (d + 8) for i in idx)
        scale = work(cand) / max(work(sel), 1)
        plain_est_s += plain_ms / 1e3 * scale
        mixed_est_s += mixed_ms / 1e3 * scale
    value = total_units / (total_ms / 1e3)
    print(json.dumps({"workload": f"config3 uneven batch, {count} instances, fwd+VJP, float32",
                      "metric": "samples·order/s fwd+VJP", "value": value, "ms": total_ms, "precision": "mixed",
                      "plain_fp64_estimated": {"value": total_units / plain_est_s,
                                               "how": "4 random instances per dimension, scaled by S*n*d^2*(d+8)"},
                      "mixed_estimated": total_units / mixed_est_s,
                      "mixed_over_plain": plain_est_s / mixed_est_s, "per_dimension_subsets": per_d,
                      "autotune_picks": picks}))


def config3_subset(torch, lib, _lib, dev, per_d=2):
    """Config3's mixed-over-plain target on a fixed subset: the first `per_d`
    instances of each dimension in the seeded config3 draw (d in 2..128,
    S log-uniform in [257, 65537], n in 2..6, float32 in), forward + VJP
    (op sum) as one plan per form, each timed as a replayed CUDA graph; plus
    the per-order error of the mixed form against the plain FP64 form on the
    same instances (op many; the plain form is pinned to the reference at
    <= 1e-12 by the test suite)."""
    from magnus_gb300 import workloads
    ds, Ss, ns, seeds = workloads.config3_instances(seed=3, count=10000)
    idx = []
    for d in (2, 4, 8, 16, 32, 64, 128):
        idx += [int(i) for i in np.nonzero(ds == d)[0][:per_d]]
    As, cots, units = [], [], 0
    for i in idx:
        d, S = int(ds[i]), int(Ss[i])
        C, w = workloads.config0_coeffs(int(seeds[i]), d)
        t = torch.linspace(0.0, 1.0, S, dtype=torch.float64, device=dev)[:, None, None]
        Ct = torch.as_tensor(C, device=dev)
        As.append((Ct[0] + Ct[1] * torch.sin(w[0] * t) + Ct[2] * torch.cos(w[1] * t)).to(torch.float32))
        cots.append(torch.ones((d, d), dtype=torch.float32, device=dev))
        units += S * int(ns[i])

    def probs(prec, op):
        return [_lib.make_problem(kind=0, dtype_code=_lib.DTYPE_F32, precision=prec, op=op, integrator=0,
                                  n=int(ns[i]), samples=int(Ss[i]), dim=int(ds[i]), t0=0.0, tf=1.0) for i in idx]

    res = {}
    for name, prec in (("mixed", _lib.PRECISION_MIXED), ("plain_fp64", _lib.PRECISION_PLAIN)):
        outs = [torch.empty((a.shape[1], a.shape[1]), dtype=torch.float32, device=dev) for a in As]
        dAs = [torch.empty_like(a) for a in As]
        plan = _plan(lib, _lib, probs(prec, _lib.OP_SUM), As, outs, cots, dAs)

        def step():
            st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            _lib.check(lib.mgb_plan_forward(plan, st))
            _lib.check(lib.mgb_plan_vjp(plan, st))

        ms = _time_graph(torch, step, 2, warmup=1)
        lib.mgb_plan_destroy(plan)
        res[name] = {"value": units / (ms / 1e3), "ms": ms, "dA": [g.cpu().numpy() for g in dAs]}
        # per-order outputs (forward, op many)
        omany = [torch.empty((int(ns[i]), int(ds[i]), int(ds[i])), dtype=torch.float32, device=dev) for i in idx]
        pl = _plan(lib, _lib, probs(prec, _lib.OP_MANY), As, omany)
        _lib.check(lib.mgb_plan_forward(pl, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        lib.mgb_plan_destroy(pl)
        res[name]["orders"] = [o.cpu().numpy() for o in omany]
    per_order = [0.0] * 6
    for om, op_ in zip(res["mixed"]["orders"], res["plain_fp64"]["orders"]):
        for k, e in enumerate(_order_errors(om.reshape(om.shape[0], -1), op_.reshape(op_.shape[0], -1))):
            per_order[k] = max(per_order[k], e)
    e_dA = max(float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))
               for a, b in zip(res["mixed"]["dA"], res["plain_fp64"]["dA"]))
    return {"workload": f"config3 subset: first {per_d} instances of each d in the seeded draw "
                        f"({len(idx)} instances, {units} samples*order), fwd+VJP, float32",
            "instances": [{"d": int(ds[i]), "S": int(Ss[i]), "n": int(ns[i])} for i in idx],
            "mixed": res["mixed"]["value"], "plain_fp64": res["plain_fp64"]["value"],
            "mixed_over_plain": res["mixed"]["value"] / res["plain_fp64"]["value"],
            "ms": {"mixed": res["mixed"]["ms"], "plain_fp64": res["plain_fp64"]["ms"]},
            "rel_err_mixed_vs_fp64_per_order_max": per_order, "rel_err_mixed_vs_fp64_dA_max": e_dA}


# ---------------------------------------------------------------- GPU legs
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "config4":
        {"config1": run_config1, "config2": run_config2, "config3": run_config3}[args.workload](args)
        return

    import torch
    import torch.distributed as dist

    from magnus_gb300 import _lib, workloads
    from magnus_gb300.autograd import magnus

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load()
    c = CONFIG4
    B, S, d, n = args.batch, args.samples, c["d"], c["n"]

    def barrier():
        if world > 1:
            dist.barrier()

    # ---- inputs resident in HBM
    Ck = workloads.config4_coeffs(seed=4 + rank, batch=B, d=d)
    A = workloads.config4_samples_torch(Ck, samples=S, device=dev)
    cot = torch.tensor(workloads.config4_cotangent(batch=B, d=d), device=dev)
    out = torch.empty((B, d, d), dtype=torch.float32, device=dev)
    dA = torch.empty_like(A)
    prec = _lib.PRECISION_CODES[args.precision]
    prob = _lib.make_problem(kind=_lib.KIND_MATRIX, dtype_code=_lib.DTYPE_F32, precision=prec, op=_lib.OP_SUM,
                             integrator=_lib.INTEGRATOR_CODES[c["integrator"]], n=n, samples=S, dim=d, t0=c["t0"],
                             tf=c["tf"], checkpoint_K=c["K"])
    probs = (_lib.Problem * B)(*([prob] * B))

    def ptrs(t):
        return (ctypes.c_void_p * B)(*[t[i].data_ptr() for i in range(B)])

    # One plan binds the batch's buffers (and holds the chunk checkpoints);
    # a step = plan forward + plan VJP, captured once into a CUDA graph.
    plan = ctypes.c_void_p()
    _lib.check(lib.mgb_plan_create(probs, B, ptrs(A), ptrs(out), ptrs(cot), ptrs(dA), ctypes.byref(plan)))
    autotune = _describe(lib, plan)
    stream = torch.cuda.current_stream(dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def step_eager():
        _lib.check(lib.mgb_plan_forward(plan, sptr))
        _lib.check(lib.mgb_plan_vjp(plan, sptr))

    step_eager()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        gs = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        _lib.check(lib.mgb_plan_forward(plan, gs))
        _lib.check(lib.mgb_plan_vjp(plan, gs))
    for _ in range(max(args.warmup, 3)):
        graph.replay()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms_t = torch.tensor([ms], device=dev)
    if world > 1:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms = float(ms_t.item())
    value = world * B * S * n / (ms / 1e3)

    # per-kernel CUDA-event times: the same steps run eagerly with the
    # library's launch timing enabled (events bracket every kernel launch)
    lib.mgb_profile_enable(1)
    _lib.profile_read(reset=True)
    for _ in range(args.steps):
        step_eager()
    torch.cuda.synchronize()
    lib.mgb_profile_enable(0)
    kernels = _lib.profile_read(reset=True)
    launches = sum(v[0] for v in kernels.values()) // args.steps * args.steps

    # ---- roofline of every timed kernel, and of the dominant one
    roofs = kernel_roofs(kernels, args.steps, B, S, d, n, c["K"], plain=args.precision == "plain")
    dom_name = max(roofs, key=lambda k: roofs[k]["ms_per_step"])
    dom = roofs[dom_name]
    units_scale = (B * S) / (CONFIG4["batch"] * CONFIG4["samples"])
    roof = {"bound": dom["bound"], "achieved": dom["achieved"], "peak": dom["peak"], "unit": dom["unit"],
            "frac": dom["frac"], "traffic": traffic_from_profiles(dom_name, units_scale), "kernel": dom_name,
            "peak_source": dom["peak_source"], "launch_ms": dom["launch_ms"],
            "algorithmic_flops_per_launch": dom["flops_per_launch"],
            "algorithmic_bytes_per_launch": dom["bytes_per_launch"],
            "per_kernel": {k: {kk: v[kk] for kk in ("ms_per_step", "bound", "frac", "achieved", "unit", "peak",
                                                    "peak_source", "compute_frac", "hbm_frac")}
                           for k, v in roofs.items()}}

    result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
              "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
              "config": {"workload": f"config4: {B} x d={d} A(t)=C0+C1 t+C2 t^2+C3 cos5t, S={S}, Boole, n={n}, "
                                     f"sum, float32 in, fwd+VJP, checkpoints every {c['K']} samples",
                         "precision": args.precision, "global_batch": B * world,
                         "cache": "inputs 68.7 GB >> L2 (no flush needed)",
                         "execution": "mgb_plan forward+VJP captured in one CUDA graph, replayed per step",
                         "autotune": autotune},
              "roofline": roof, "gpu_launches": launches, "clocks": clk,
              "kernels_ms_per_step": {k: v[1] / args.steps for k, v in kernels.items()}}

    if rank == 0 and not args.no_extras:
        # the timed steps' outputs of the first instances, for the check
        # against the FP64 oracle in the CPU leg below
        nck = min(args.oracle_instances, B)
        ck_in = (A[:nck].cpu().numpy(), cot[:nck].cpu().numpy(), out[:nck].cpu().numpy(), dA[:nck].cpu().numpy())

        try:
            # ---- plain FP64 path and mixed-vs-FP64 error on a subset
            sub = min(args.plain_subset, B)
            prob_p = _lib.make_problem(kind=_lib.KIND_MATRIX, dtype_code=_lib.DTYPE_F32, precision=_lib.PRECISION_PLAIN,
                                       op=_lib.OP_SUM, integrator=0, n=n, samples=S, dim=d, t0=c["t0"], tf=c["tf"],
                                       checkpoint_K=c["K"])
            probs_p = (_lib.Problem * sub)(*([prob_p] * sub))
            Ap = A[:sub]
            out_p = torch.empty((sub, d, d), dtype=torch.float32, device=dev)
            dA_p = torch.empty_like(Ap)

            def sp(t):
                return (ctypes.c_void_p * sub)(*[t[i].data_ptr() for i in range(sub)])

            # a plan like the mixed arm's (its creation and autotuning outside
            # the timed region); one untimed forward + VJP, then one timed
            plan_p = ctypes.c_void_p()
            _lib.check(lib.mgb_plan_create(probs_p, sub, sp(Ap), sp(out_p), sp(cot[:sub]), sp(dA_p),
                                           ctypes.byref(plan_p)))
            _lib.check(lib.mgb_plan_forward(plan_p, sptr))
            _lib.check(lib.mgb_plan_vjp(plan_p, sptr))
            torch.cuda.synchronize()
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            _lib.check(lib.mgb_plan_forward(plan_p, sptr))
            _lib.check(lib.mgb_plan_vjp(plan_p, sptr))
            f1.record(stream)
            torch.cuda.synchronize()
            _lib.check(lib.mgb_plan_destroy(plan_p))
            plain_ms = f0.elapsed_time(f1)
            plain_value = sub * S * n / (plain_ms / 1e3)
            # mixed (already computed in the timed steps for these instances) vs FP64
            e_out = float(torch.linalg.norm((out[:sub] - out_p).double()) / torch.linalg.norm(out_p.double()))
            e_dA = float(torch.linalg.norm((dA[:sub] - dA_p).double()) / torch.linalg.norm(dA_p.double()))
            result["plain_fp64"] = {"value": plain_value, "unit": UNIT, "instances": sub, "ms": plain_ms,
                                    "mixed_speedup": value / world / plain_value}
            result["rel_err_mixed_vs_fp64"] = {"out": e_out, "dA": e_dA, "instances": sub}
            del out_p, dA_p
        except Exception as exc:  # a failed extra leg must not cost the contract line
            msg = f"{type(exc).__name__}: {exc}"[:400]
            result['plain_fp64'] = {"error": msg}

        try:
            # ---- config3's mixed-over-plain target on a fixed subset
            result["config3_subset"] = config3_subset(torch, lib, _lib, dev)
        except Exception as exc:  # a failed extra leg must not cost the contract line
            msg = f"{type(exc).__name__}: {exc}"[:400]
            result['config3_subset'] = {"error": msg}

        # the timed step's graph, plan and dA give their memory to the e2e legs
        del graph
        _lib.check(lib.mgb_plan_destroy(plan))
        plan = None
        del dA
        torch.cuda.empty_cache()

        try:
            # ---- end to end through the public autograd API, pinned host buffers
            eb = min(args.e2e_batch, B) if args.e2e_batch > 0 else e2e_instances(B, S * d * d * 4)
            # page-locked host buffers; fewer instances if the host cannot lock them
            while True:
                try:
                    A_host, free_A_host = pinned_host((eb, S, d, d), np.float32)
                except RuntimeError:
                    if eb == 1:
                        raise
                    eb = max(1, eb // 2)
                    continue
                try:
                    dA_host, free_dA_host = pinned_host((eb, S, d, d), np.float32)
                except RuntimeError:
                    del A_host
                    free_A_host()
                    if eb == 1:
                        raise
                    eb = max(1, eb // 2)
                    continue
                break
            A_host.copy_(A[:eb])
            cot_host = cot[:eb].cpu().pin_memory()
            out_host = torch.empty((eb, d, d), dtype=torch.float32).pin_memory()
            A_dev = torch.empty((eb, S, d, d), dtype=torch.float32, device=dev)

            marks = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

            def e2e_step():
                marks[0].record(stream)
                A_dev.copy_(A_host, non_blocking=True)
                x = A_dev.detach().requires_grad_(True)
                g = cot_host.to(dev, non_blocking=True)
                marks[1].record(stream)
                o = magnus(x, n, c["t0"], c["tf"], op="sum", integrator="Boole", precision=args.precision,
                           checkpoint_K=c["K"])
                o.backward(g)
                marks[2].record(stream)
                out_host.copy_(o.detach(), non_blocking=True)
                dA_host.copy_(x.grad, non_blocking=True)
                marks[3].record(stream)

            e2e_step()
            torch.cuda.synchronize()
            g0 = torch.cuda.Event(enable_timing=True)
            g1 = torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            e2e_steps = max(1, min(args.steps, 2))
            for _ in range(e2e_steps):
                e2e_step()
            g1.record(stream)
            torch.cuda.synchronize()
            e2e_ms = g0.elapsed_time(g1) / e2e_steps
            h2d = A_host.numel() * 4 + cot_host.numel() * 4
            d2h = dA_host.numel() * 4 + out_host.numel() * 4
            split = [marks[i].elapsed_time(marks[i + 1]) for i in range(3)]  # last step
            result["e2e_autograd"] = {"value": eb * S * n / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                                      "d2h_bytes_per_step": d2h, "instances": eb, "ms_per_step": e2e_ms,
                                      "api": "magnus_gb300.autograd.magnus forward + backward, copies on one stream",
                                      "last_step_ms": {"h2d": split[0], "compute": split[1], "d2h": split[2]}}
            del A_dev
            torch.cuda.empty_cache()

            # ---- end to end through the C ABI's host entry point (the call the
            # reference's module binds), pinned host buffers, copies pipelined
            probs_e = (_lib.Problem * eb)(*([prob] * eb))
            hp = lambda t: (ctypes.c_void_p * eb)(*[t[i].data_ptr() for i in range(eb)])  # noqa: E731

            def host_step():
                _lib.check(lib.mgb_fwd_vjp_host_batched(probs_e, eb, hp(A_host), hp(cot_host), hp(out_host), hp(dA_host)))

            host_step()  # warm-up (also allocates the library's staging slots)
            host_ms_all = []
            for _ in range(5):
                t0h = time.perf_counter()
                host_step()
                host_ms_all.append((time.perf_counter() - t0h) * 1e3)
            host_ms = statistics.median(host_ms_all)
            # one more call with the library's launch timing on: per-stage device
            # time (copies in, kernels, copies out) against the wall clock, to
            # show how far the stages overlap
            lib.mgb_profile_enable(1)
            _lib.profile_read(reset=True)
            t0h = time.perf_counter()
            host_step()
            prof_wall = (time.perf_counter() - t0h) * 1e3
            lib.mgb_profile_enable(0)
            stages = _lib.profile_read(reset=True)
            def stage_sum(prefix):
                return sum(v[1] for k, v in stages.items() if k.startswith(prefix + "."))

            stage_ms = {"h2d": stage_sum("h2d"), "d2h": stage_sum("d2h"),
                        "kernels": sum(v[1] for k, v in stages.items() if "." not in k), "wall": prof_wall}
            # per sub-batch: [start, end] of its copies in, kernels and copies out
            # (ms after the first copy started)
            subs = sorted(int(k.split(".")[1]) for k in stages if k.startswith("comp."))
            t_first = min((v[2] for k, v in stages.items() if "." in k), default=0.0)
            timeline = [{st: [round(stages[f"{st}.{b}"][2] - t_first, 2), round(stages[f"{st}.{b}"][3] - t_first, 2)]
                         for st in ("h2d", "comp", "d2h") if f"{st}.{b}" in stages} for b in subs]
            result["e2e"] = {"value": eb * S * n / (host_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                             "d2h_bytes_per_step": d2h, "instances": eb, "ms_per_step": host_ms,
                             "ms_per_step_min_max": [min(host_ms_all), max(host_ms_all)], "steps": len(host_ms_all),
                             "api": "mgb_fwd_vjp_host_batched (C ABI, host buffers, synchronous; wall clock, median "
                                    "of 5 calls: host-to-device copy rates on this machine vary between calls)",
                             "stage_ms_one_call": stage_ms, "sub_batches_ms": timeline,
                             "link_gbs": {"h2d": h2d / (stage_ms["h2d"] / 1e3) / 1e9 if stage_ms["h2d"] else None,
                                          "d2h": d2h / (stage_ms["d2h"] / 1e3) / 1e9 if stage_ms["d2h"] else None}}
            del A_host, dA_host
            free_A_host()
            free_dA_host()
        except Exception as exc:  # a failed extra leg must not cost the contract line
            msg = f"{type(exc).__name__}: {exc}"[:400]
            result['e2e'] = {"error": msg}

        try:
            # ---- CPU baseline (oracle port on the host cores, bounded sample)
            threads = os.cpu_count() or 1
            inst = args.cpu_instances or threads
            cpu_value, cpu_s = cpu_sample(inst, args.cpu_samples, threads)
            result["cpu_baseline"] = {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": "port",
                                      "sample": f"{inst} config4 trajectories at S={args.cpu_samples} (of 32769), "
                                                f"fwd + VJP, float32, {cpu_s:.1f} s", "cpu_model": cpu_model()}
        except Exception as exc:  # a failed extra leg must not cost the contract line
            msg = f"{type(exc).__name__}: {exc}"[:400]
            result['cpu_baseline'] = {"error": msg}

        try:
            if nck:
                result["rel_err_mixed_vs_oracle"] = oracle_check(*ck_in, n=n, t0=c["t0"], tf=c["tf"])
        except Exception as exc:  # a failed extra leg must not cost the contract line
            msg = f"{type(exc).__name__}: {exc}"[:400]
            result['rel_err_mixed_vs_oracle'] = {"error": msg}
    if plan is not None and plan.value:
        _lib.check(lib.mgb_plan_destroy(plan))
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
