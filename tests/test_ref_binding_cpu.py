"""The reference's own pybind11 module with the "GB300" matrix backend bound in
(oracle/build_ref.sh builds it into oracle/_ref/gb300/ from the reference's
sources plus oracle/ref_gb300/): the binding compiles, links against
libmagnus_gb300.so, advertises the backend, leaves the reference's own
backends untouched, keeps the reference's argument checks in front of the
engine, and routes "GB300" to the engine (which, with no GPU, answers with
its CUDA error as a RuntimeError).  Each check runs in a child process,
since the module is named `magnus` like the unmodified reference's.

The same calls on a GPU are in test_ref_binding_gpu.py.
"""
import glob
import json
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, ROOT

GB300_REF = os.path.join(ROOT, "oracle", "_ref", "gb300")

pytestmark = pytest.mark.skipif(
    not glob.glob(os.path.join(GB300_REF, "magnus", "_core*.so")),
    reason="reference module with the GB300 backend not built here (oracle/build_ref.sh needs the reference sources)")

PRELUDE = f"""
import json, sys
import numpy as np
sys.path.insert(0, {GB300_REF!r})
import magnus
core = magnus._core
g = np.load({os.path.join(GOLDEN, 'small.npz')!r})
case = lambda k: {{f.split('/', 1)[1]: g[f] for f in g.files if f.startswith(k + '/')}}
def err(fn):
    try:
        fn()
    except Exception as e:
        return [type(e).__name__, str(e)]
    return None
"""


def run(code):
    r = subprocess.run([sys.executable, "-c", PRELUDE + code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_backend_is_listed_after_the_references_own():
    names = run("print(json.dumps(list(magnus.matrix_backends())))")
    assert names[-1] == "GB300"
    assert {"Fixed2", "Manual", "Auto"} <= set(names[:-1])


def test_reference_backends_still_match_golden():
    res = run("""
c = case('m000')
n, A = int(c['n']), c['A']
out = core.compute(n, A, float(c['t0']), float(c['tf']), op=str(c['op']), matrix_backend='Fixed2',
                   integrator=str(c['integrator']), gl_backend='serial')
print(json.dumps(float(np.linalg.norm(out - c['out']) / np.linalg.norm(c['out']))))
""")
    assert res <= 1e-13


def test_gb300_backend_reaches_the_engine():
    # with no CUDA device the engine's own error comes back; with one (a GPU
    # host) the call succeeds and test_ref_binding_gpu.py checks the values
    res = run("""
c = case('m000')
print(json.dumps(err(lambda: core.compute(int(c['n']), c['A'], 0.0, 1.3, op=str(c['op']), matrix_backend='GB300',
                                          integrator=str(c['integrator'])))))
""")
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        assert res is None
    else:
        assert res is not None and res[0] == "RuntimeError" and res[1].startswith("GB300 backend:"), res


def test_reference_checks_run_before_the_engine():
    res = run("""
A = np.zeros((17, 2, 2))
out = [
    err(lambda: core.compute(3, A, 0.0, 1.0, op='bogus', matrix_backend='GB300', integrator='Boole')),
    err(lambda: core.compute(3, A, 0.0, 1.0, op='sum', matrix_backend='GB300', integrator='Nope')),
    err(lambda: core.compute(3, np.zeros((17, 2, 3)), 0.0, 1.0, op='sum', matrix_backend='GB300',
                             integrator='Boole')),
    err(lambda: core.compute_vjp(3, A, np.zeros((3, 2, 2)), t0=0.0, tf=1.0, op='sum', matrix_backend='GB300',
                                 integrator='Boole')),
    err(lambda: core.compute(3, A.astype(np.int8).astype(object), 0.0, 1.0, op='sum', matrix_backend='GB300',
                             integrator='Boole')),
]
print(json.dumps(out))
""")
    bad_op, bad_integ, bad_shape, bad_cot, bad_dtype = res
    assert bad_op[0] == "ValueError" and "op_from_str" in bad_op[1]
    assert bad_integ == ["ValueError", "Could not resolve dispatch name option"]
    assert bad_shape[0] == "ValueError"
    assert bad_cot[0] == "ValueError"
    assert bad_dtype[0] == "TypeError"
