"""bench.py's reference arm (the CPU baseline; it needs no GPU) prints one
JSON line with the contract's keys, and the rank-nonzero processes of a
torchrun launch print nothing."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def _run(env_extra=None, *args):
    env = dict(os.environ)
    env.update(env_extra or {})
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--cpu-samples", "257", "--cpu-instances", "2", *args],
                         capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    return [ln for ln in out.stdout.splitlines() if ln.strip()]


def test_reference_arm_json_line():
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["cpu_model"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]


def test_reference_arm_other_ranks_are_silent():
    assert _run({"RANK": "1"}) == []


def test_kernel_roofs_from_profile_records():
    """The per-kernel roofline of the JSON line from the library's timing
    records ({name: (launches, total_ms, first_start_ms, last_end_ms)}): the
    config4 chunk kernels are rated against the tensor roof, the mixed-form
    scans against double-FP32, and every fraction is achieved / peak."""
    sys.path.insert(0, ROOT)
    import bench
    rec = {"chunk_local": (3, 420.0, 0.0, 1.0), "chunk_vjp": (3, 1170.0, 0.0, 1.0), "scan": (3, 39.7, 0.0, 1.0),
           "rscan": (3, 39.8, 0.0, 1.0), "fin_fwd": (3, 9.6, 0.0, 1.0)}
    roofs = bench.kernel_roofs(rec, 3, 512, 32769, 32, 5, 256)
    vjp = roofs["chunk_vjp"]
    assert vjp["bound"] == "tensor" and abs(vjp["launch_ms"] - 390.0) < 1e-9
    assert abs(vjp["achieved"] - 3 * 4 * 2 * 32 ** 3 * 32769 * 512 / 0.39 / 1e12) < 1e-6
    assert abs(vjp["frac"] - vjp["achieved"] / vjp["peak"]) < 1e-12
    assert roofs["scan"]["bound"] == "fp32" and roofs["fin_fwd"]["bound"] == "hbm"
