"""The reference's own `_core.compute` / `compute_vjp` with
matrix_backend="GB300" (the module oracle/build_ref.sh builds into
oracle/_ref/gb300/) against the reference's golden outputs: forward, recorded
carry and VJP, plain FP64 engine path, every rule and op of the small cases.

Needs a host that has both a CUDA GPU and the reference module built for its
own architecture; elsewhere it is skipped (test_ref_binding_cpu.py covers the
binding without a GPU).
"""
import glob
import json
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, ROOT

GB300_REF = os.path.join(ROOT, "oracle", "_ref", "gb300")

CODE = f"""
import json, sys
import numpy as np
sys.path.insert(0, {GB300_REF!r})
import magnus
core = magnus._core
g = np.load({os.path.join(GOLDEN, 'small.npz')!r})
cases = {{}}
for f in g.files:
    k, fld = f.split('/', 1)
    cases.setdefault(k, {{}})[fld] = g[f]
rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
worst = {{'out': 0.0, 'dA': 0.0, 'carry': 0.0, 'cases': 0}}
for k, c in cases.items():
    if str(c['kind']) != 'matrix':
        continue
    n, A, op, integ = int(c['n']), c['A'], str(c['op']), str(c['integrator'])
    t0, tf = float(c['t0']), float(c['tf'])
    out = core.compute(n, A, t0, tf, op=op, matrix_backend='GB300', integrator=integ)
    dA = core.compute_vjp(n, A, c['cot'], t0=t0, tf=tf, op=op, matrix_backend='GB300', integrator=integ)
    worst['out'] = max(worst['out'], rel(out, c['out']))
    worst['dA'] = max(worst['dA'], rel(dA, c['dA']))
    if 'carry' in c:
        _, carry = core.compute(n, A, t0, tf, op=op, matrix_backend='GB300', integrator=integ, record_vjp=True)
        worst['carry'] = max(worst['carry'], rel(carry, c['carry']))
        dA2 = core.compute_vjp(n, A, c['cot'], vjp_data=carry, t0=t0, tf=tf, op=op, matrix_backend='GB300',
                               integrator=integ)
        worst['dA'] = max(worst['dA'], rel(dA2, c['dA']))
    worst['cases'] += 1
print(json.dumps(worst))
"""


def _module_loads():
    if not glob.glob(os.path.join(GB300_REF, "magnus", "_core*.so")):
        return False
    r = subprocess.run([sys.executable, "-c", f"import sys; sys.path.insert(0, {GB300_REF!r}); import magnus"],
                       capture_output=True, timeout=120)
    return r.returncode == 0


@pytest.mark.gpu
def test_reference_module_with_gb300_backend_matches_golden(cuda):
    if not _module_loads():
        pytest.skip("the reference module with the GB300 backend is not built for this host")
    r = subprocess.run([sys.executable, "-c", CODE], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    worst = json.loads(r.stdout.strip().splitlines()[-1])
    assert worst["cases"] > 0
    assert worst["out"] <= 1e-12 and worst["dA"] <= 1e-12 and worst["carry"] <= 1e-12, worst
