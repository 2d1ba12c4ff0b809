"""Device-side sampling (magnus_gb300.device): the same function sampled on
the GPU gives the host path's result, and the propagator exp(Omega) of a
Magnus sum tracks a reference ODE solution."""
import numpy as np
import pytest

import magnus_gb300 as magnus
from conftest import rel

pytestmark = pytest.mark.gpu


def test_compute_device_matches_host_path(cuda):
    import torch
    from magnus_gb300 import device
    C = np.random.default_rng(2).standard_normal((3, 4, 4)) / 2

    def f_np(t):
        t = np.asarray(t)[:, None, None]
        return C[0] + C[1] * np.sin(2 * t) + C[2] * t * t

    Ct = torch.tensor(C, device=cuda)

    def f_t(t):
        t = t[:, None, None]
        return Ct[0] + Ct[1] * torch.sin(2 * t) + Ct[2] * t * t

    host = magnus.compute(5, f_np, 0.0, 1.0, 257, op="many", integrator="Boole", precision="plain")
    dev = device.compute_device(5, f_t, 0.0, 1.0, 257, op="many", integrator="Boole", precision="plain",
                                dtype=torch.float64)
    assert rel(dev.cpu().numpy(), host) <= 1e-14


def test_propagator_tracks_ode_solution(cuda):
    import torch
    from scipy.integrate import solve_ivp
    from magnus_gb300 import device
    C = np.random.default_rng(4).standard_normal((2, 3, 3)) / 5  # inside the fast-converging regime

    def A_np(t):
        return C[0] + C[1] * np.cos(3 * t)

    sol = solve_ivp(lambda t, y: (A_np(t) @ y.reshape(3, 3)).ravel(), (0.0, 1.0), np.eye(3).ravel(), rtol=1e-12,
                    atol=1e-14)
    Y1 = sol.y[:, -1].reshape(3, 3)
    Ct = torch.tensor(C, device=cuda)
    omega = device.compute_device(10, lambda t: Ct[0] + Ct[1] * torch.cos(3 * t)[:, None, None], 0.0, 1.0, 4097,
                                  op="sum", integrator="Boole", precision="plain", dtype=torch.float64)
    U = device.expm(omega).cpu().numpy()
    assert rel(U, Y1) <= 1e-8
