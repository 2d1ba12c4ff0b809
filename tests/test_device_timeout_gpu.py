"""The bounded device-side wait and its error path, exercised without a GPU
fault: a kernel waits (1 ms) on a barrier that nothing arrives at, gives up
the way the engine's tensor-core and bulk-copy kernels do, and raises the
time-out flag.  The host reads it as MGB_ERR_DEVICE_TIMEOUT (a status, as the
reference's JAX handlers return errors, src/api/jax_ffi.cpp:280-284), the
flag is cleared by that read, and the context stays usable."""
import ctypes

import pytest

import oracle as O
from conftest import rel
from magnus_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu
MGB_OK, MGB_ERR_INVALID_ARGUMENT, MGB_ERR_DEVICE_TIMEOUT = 0, 1, 5


def test_bounded_wait_times_out_and_context_survives(cuda):
    import torch
    lib = _lib.load()
    assert lib.mgb_device_check() == MGB_OK  # nothing pending
    assert lib.mgb_selftest_bounded_wait(1_000_000, None) == MGB_OK
    assert lib.mgb_device_check() == MGB_ERR_DEVICE_TIMEOUT
    assert b"timed out" in lib.mgb_last_error()
    assert lib.mgb_device_check() == MGB_OK  # the flag was cleared by the read
    # the context still computes: a small forward against the oracle
    A = workloads.config0_samples(seed=9, d=2, samples=257)
    At = torch.tensor(A, device=cuda)
    out = torch.empty((2, 2), dtype=torch.float64, device=cuda)
    prob = _lib.make_problem(kind=_lib.KIND_MATRIX, dtype_code=_lib.DTYPE_F64, precision=_lib.PRECISION_PLAIN,
                             op=_lib.OP_SUM, integrator=0, n=4, samples=257, dim=2, t0=0.0, tf=1.0)
    _lib.check(lib.mgb_forward(ctypes.byref(prob), At.data_ptr(), out.data_ptr(), None, None, None))
    assert lib.mgb_device_check() == MGB_OK
    assert rel(out.cpu().numpy(), O.forward(A, 4, 0.0, 1.0, "sum", "Boole")) <= 1e-12


def test_bounded_wait_limit_is_checked(cuda):
    lib = _lib.load()
    assert lib.mgb_selftest_bounded_wait(0, None) == MGB_ERR_INVALID_ARGUMENT
    assert lib.mgb_selftest_bounded_wait(3_000_000_000, None) == MGB_ERR_INVALID_ARGUMENT
    assert lib.mgb_device_check() == MGB_OK
