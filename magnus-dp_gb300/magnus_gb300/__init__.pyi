import numpy as np
from typing import Any, Callable, Literal, overload

from ._generated_typing import (GLBackendName, IntegratorName, KernelOpName, MatrixBackendName, NumericBackendName,
                                PrecisionName)

def max_order() -> int:
    """Largest Gauss-Legendre order in the active table."""

def numeric_backends() -> tuple[NumericBackendName, ...]: ...

def matrix_backends() -> tuple[MatrixBackendName, ...]: ...

def integrators() -> tuple[IntegratorName, ...]: ...

def gl_backends() -> tuple[GLBackendName, ...]: ...

def ops() -> tuple[KernelOpName, ...]: ...

def replace_gl_table(max_order: int) -> None:
    """Generate and install a new Gauss-Legendre table through max_order."""

@overload
def compute(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    matrix_backend: MatrixBackendName = "Auto",
    integrator: IntegratorName = "Auto",
    gl_backend: GLBackendName = "Auto",
    record_vjp: Literal[False] = False,
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> np.ndarray:
    """Magnus operation of a sampled R -> matrix function on the GB300."""

@overload
def compute(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    matrix_backend: MatrixBackendName = "Auto",
    integrator: IntegratorName = "Auto",
    gl_backend: GLBackendName = "Auto",
    record_vjp: Literal[True],
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> tuple[np.ndarray, np.ndarray]: ...

@overload
def compute(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    matrix_backend: MatrixBackendName = "Auto",
    integrator: IntegratorName = "Auto",
    gl_backend: GLBackendName = "Auto",
    record_vjp: bool,
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> np.ndarray | tuple[np.ndarray, np.ndarray]: ...

@overload
def compute_sc(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    integrator: IntegratorName = "Auto",
    gl_backend: GLBackendName = "Auto",
    record_vjp: Literal[False] = False,
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> np.ndarray:
    """Magnus operation of a sampled R -> R^3 SpaceCurve on the GB300."""

@overload
def compute_sc(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    integrator: IntegratorName = "Auto",
    gl_backend: GLBackendName = "Auto",
    record_vjp: Literal[True],
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> tuple[np.ndarray, np.ndarray]: ...

@overload
def compute_sc(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    integrator: IntegratorName = "Auto",
    gl_backend: GLBackendName = "Auto",
    record_vjp: bool,
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> np.ndarray | tuple[np.ndarray, np.ndarray]: ...

def compute_vjp(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    cotangent: np.ndarray,
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    matrix_backend: MatrixBackendName = "Auto",
    integrator: IntegratorName = "Auto",
    vjp_data: np.ndarray | None = None,
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> np.ndarray:
    """Gradient with respect to the sampled matrices, given the output's cotangent."""

def compute_sc_vjp(
    n: int,
    f: Callable[[np.ndarray], np.ndarray],
    cotangent: np.ndarray,
    t0: float,
    tf: float,
    samples: int,
    *,
    op: KernelOpName = "sum",
    dtype: Any = None,
    vectorized: bool = True,
    integrator: IntegratorName = "Auto",
    vjp_data: np.ndarray | None = None,
    precision: PrecisionName = "plain",
    checkpoint_K: int = 0,
) -> np.ndarray:
    """Gradient with respect to the sampled SpaceCurve, given the output's cotangent."""
