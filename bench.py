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
    ap.add_argument("--e2e-batch", type=int, default=128)
    ap.add_argument("--cpu-instances", type=int, default=0, help="0 = one per host thread")
    ap.add_argument("--cpu-samples", type=int, default=4097)
    ap.add_argument("--no-extras", action="store_true", help="skip plain/e2e/cpu legs (quick runs)")
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
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU legs
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
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

    # ---- roofline of the dominant kernel
    hbm_peak, bf16_peak, sm_max, peak_src = load_peaks()
    dom = max(kernels.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms_total) = dom
    dom_ms = dom_ms_total / dom_launches
    m = d * d
    prods = {"chunk_local": (n - 1), "chunk_vjp": 3 * (n - 1)}.get(dom_name, 0)
    flops = prods * 2.0 * d ** 3 * S * B
    bytes_alg = {"chunk_local": S * m * 4 * B, "chunk_vjp": 2 * S * m * 4 * B}.get(dom_name, S * m * 4 * B)
    tflops = flops / (dom_ms / 1e3) / 1e12
    gbs = bytes_alg / (dom_ms / 1e3) / 1e9
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    if tflops / bf16_peak >= gbs / hbm_peak:
        roof = {"bound": "tensor", "achieved": tflops, "peak": bf16_peak, "unit": "TFLOP/s", "frac": tflops / bf16_peak}
    else:
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak}
    units_scale = (B * S) / (CONFIG4["batch"] * CONFIG4["samples"])
    roof.update({"kernel": dom_name, "traffic": traffic_from_profiles(dom_name, units_scale), "peak_source": peak_src,
                 "launch_ms": dom_ms, "algorithmic_flops_per_launch": flops, "algorithmic_bytes_per_launch": bytes_alg,
                 "fp32_simt": {"achieved_tflops": tflops, "nominal_peak_tflops": fp32_peak,
                               "frac": tflops / fp32_peak}})

    result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
              "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
              "config": {"workload": f"config4: {B} x d={d} A(t)=C0+C1 t+C2 t^2+C3 cos5t, S={S}, Boole, n={n}, "
                                     f"sum, float32 in, fwd+VJP, checkpoints every {c['K']} samples",
                         "precision": args.precision, "global_batch": B * world,
                         "cache": "inputs 68.7 GB >> L2 (no flush needed)",
                         "execution": "mgb_plan forward+VJP captured in one CUDA graph, replayed per step"},
              "roofline": roof, "gpu_launches": launches, "clocks": clk,
              "kernels_ms_per_step": {k: v[1] / args.steps for k, v in kernels.items()}}

    if rank == 0 and not args.no_extras:
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

        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        _lib.check(lib.mgb_forward_batched(probs_p, sub, sp(Ap), sp(out_p), None, sptr))
        _lib.check(lib.mgb_vjp_batched(probs_p, sub, sp(Ap), sp(cot[:sub]), None, sp(dA_p), sptr))
        f1.record(stream)
        torch.cuda.synchronize()
        plain_ms = f0.elapsed_time(f1)
        plain_value = sub * S * n / (plain_ms / 1e3)
        # mixed (already computed in the timed steps for these instances) vs FP64
        e_out = float(torch.linalg.norm((out[:sub] - out_p).double()) / torch.linalg.norm(out_p.double()))
        e_dA = float(torch.linalg.norm((dA[:sub] - dA_p).double()) / torch.linalg.norm(dA_p.double()))
        result["plain_fp64"] = {"value": plain_value, "unit": UNIT, "instances": sub, "ms": plain_ms,
                                "mixed_speedup": value / world / plain_value}
        result["rel_err_mixed_vs_fp64"] = {"out": e_out, "dA": e_dA, "instances": sub}
        del out_p, dA_p

        # ---- end to end through the public autograd API, pinned host buffers
        eb = min(args.e2e_batch, B)
        A_host = torch.empty((eb, S, d, d), dtype=torch.float32, pin_memory=True)
        A_host.copy_(A[:eb])
        cot_host = cot[:eb].cpu().pin_memory()
        dA_host = torch.empty_like(A_host).pin_memory()
        out_host = torch.empty((eb, d, d), dtype=torch.float32).pin_memory()
        del graph
        _lib.check(lib.mgb_plan_destroy(plan))
        plan = None
        del dA
        torch.cuda.empty_cache()
        A_dev = torch.empty((eb, S, d, d), dtype=torch.float32, device=dev)

        def e2e_step():
            A_dev.copy_(A_host, non_blocking=True)
            x = A_dev.detach().requires_grad_(True)
            g = cot_host.to(dev, non_blocking=True)
            o = magnus(x, n, c["t0"], c["tf"], op="sum", integrator="Boole", precision=args.precision,
                       checkpoint_K=c["K"])
            o.backward(g)
            out_host.copy_(o.detach(), non_blocking=True)
            dA_host.copy_(x.grad, non_blocking=True)

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
        result["e2e"] = {"value": eb * S * n / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h, "instances": eb, "ms_per_step": e2e_ms,
                         "api": "magnus_gb300.autograd.magnus forward + backward"}

        # ---- CPU baseline (oracle port on the host cores, bounded sample)
        threads = os.cpu_count() or 1
        inst = args.cpu_instances or threads
        cpu_value, cpu_s = cpu_sample(inst, args.cpu_samples, threads)
        result["cpu_baseline"] = {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": "port",
                                  "sample": f"{inst} config4 trajectories at S={args.cpu_samples} (of 32769), "
                                            f"fwd + VJP, float32, {cpu_s:.1f} s"}
    if plan is not None and plan.value:
        _lib.check(lib.mgb_plan_destroy(plan))
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
