"""Public Python API of magnus_gb300 mirrors the reference `magnus` package:
exports, dispatch metadata and the error contract
(tests/test_python_api.py:234-283, 766-871 of the reference).  All of these
fail during validation, before any GPU work."""
import numpy as np
import pytest

import magnus_gb300 as magnus


def matrix_values(t, dtype=np.float64):
    t = np.asarray(t)
    out = np.empty((t.size, 2, 2), dtype=dtype)
    out[:, 0, 0] = 1.0 + t
    out[:, 0, 1] = t * t
    out[:, 1, 0] = -0.5 * t
    out[:, 1, 1] = 2.0 - t
    return out


def spacecurve_values(t, dtype=np.float64):
    t = np.asarray(t)
    out = np.empty((t.size, 3), dtype=dtype)
    out[:, 0] = np.sin(1.3 * t) + 0.2 * t
    out[:, 1] = np.cos(0.7 * t) - 0.1
    out[:, 2] = 0.4 + t * t
    return out


def test_public_api_exports_only_compute_entrypoints():
    assert set(magnus.__all__) == {"max_order", "numeric_backends", "matrix_backends", "integrators", "gl_backends",
                                   "ops", "replace_gl_table", "compute", "compute_sc", "compute_vjp",
                                   "compute_sc_vjp"}
    for removed in ["one_s", "many_s", "sum_s", "one", "many", "sum", "one_sc", "many_sc", "sum_sc"]:
        assert not hasattr(magnus, removed)


def test_dispatch_metadata_is_discoverable():
    assert magnus.ops() == ("one", "many", "sum")
    for name in ("Manual", "SpaceCurve", "Auto", "GB300"):
        assert name in magnus.matrix_backends()
    assert "Riemann" in magnus.integrators() and "Auto" in magnus.integrators()
    for name in ("serial", "openmp", "threadpool", "Auto"):
        assert name in magnus.gl_backends()
    assert "float" in magnus.numeric_backends() and "double" in magnus.numeric_backends()
    assert "Auto" not in magnus.numeric_backends()


def test_dispatch_kwargs_are_forwarded():
    def f(t):
        return np.zeros((np.asarray(t).size, 3, 3), dtype=np.float64)

    with pytest.raises(ValueError, match="invalid dispatch option"):
        magnus.compute(1, f, 0.0, 1.0, 9, op="one", matrix_backend="Fixed2")
    with pytest.raises(ValueError, match="dispatch name"):
        magnus.compute(1, f, 0.0, 1.0, 9, op="one", matrix_backend="Missing")
    with pytest.raises(ValueError, match="dispatch name"):
        magnus.compute(1, f, 0.0, 1.0, 9, op="one", integrator="Missing")
    with pytest.raises(ValueError, match="dispatch name"):
        magnus.compute(1, f, 0.0, 1.0, 9, op="one", gl_backend="Missing")
    with pytest.raises(ValueError, match="deduce kernel op"):
        magnus.compute(1, f, 0.0, 1.0, 9, op="missing")
    with pytest.raises(ValueError, match="invalid dispatch option"):
        magnus.compute(1, f, 0.0, 1.0, 9, gl_backend="threadpool")


def test_sample_count_is_validated_by_core_after_sampling():
    called = []

    def f(t):
        called.append(True)
        return matrix_values(t)

    with pytest.raises(ValueError, match="at least two samples"):
        magnus.compute(1, f, 0.0, 1.0, 1)
    assert called
    with pytest.raises(ValueError, match="at least two samples"):
        magnus.compute_sc(1, lambda t: spacecurve_values(t), 0.0, 1.0, 1)


@pytest.mark.parametrize("bad", [np.zeros((9, 2)), np.zeros((8, 2, 2)), np.zeros((9, 2, 3))])
def test_callable_output_shape_is_validated(bad):
    with pytest.raises(ValueError):
        magnus.compute(1, lambda t: bad, 0.0, 1.0, 9)


@pytest.mark.parametrize("bad", [np.zeros((9, 2)), np.zeros((8, 3)), np.zeros((9, 3, 1))])
def test_spacecurve_callable_output_shape_is_validated(bad):
    with pytest.raises(ValueError):
        magnus.compute_sc(1, lambda t: bad, 0.0, 1.0, 9)


def test_core_inputs_are_validated_through_public_compute():
    with pytest.raises(ValueError, match="n must be at least 1"):
        magnus.compute(0, matrix_values, 0.0, 1.0, 9)
    with pytest.raises(TypeError, match="supports dtypes"):
        magnus.compute(1, lambda t: matrix_values(t).astype(np.int64), 0.0, 1.0, 9)
    with pytest.raises(ValueError, match="n must be at least 1"):
        magnus.compute_sc(0, spacecurve_values, 0.0, 1.0, 9)
    with pytest.raises(TypeError, match="supports dtypes"):
        magnus.compute_sc(1, lambda t: spacecurve_values(t).astype(np.int64), 0.0, 1.0, 9)
    with pytest.raises(ValueError, match="shape"):
        magnus.compute_sc(1, lambda t: np.zeros((np.asarray(t).size, 4)), 0.0, 1.0, 9)


def test_vjp_shapes_are_validated():
    with pytest.raises(ValueError, match="one/sum output must have shape"):
        magnus.compute_vjp(4, matrix_values, np.zeros((3, 3)), 0.0, 1.0, 9)
    with pytest.raises(ValueError, match="many output must have shape"):
        magnus.compute_vjp(4, matrix_values, np.zeros((2, 2)), 0.0, 1.0, 9, op="many")
    with pytest.raises(ValueError, match="VJP data has an invalid shape"):
        magnus.compute_vjp(4, matrix_values, np.zeros((2, 2)), 0.0, 1.0, 9, vjp_data=np.zeros((3, 3, 9, 2, 1)))
    with pytest.raises(ValueError, match="spacecurve output must have shape"):
        magnus.compute_sc_vjp(4, spacecurve_values, np.zeros((2,)), 0.0, 1.0, 9)


def test_divisibility_and_gl_order_errors():
    with pytest.raises(ValueError, match="divisibility"):
        magnus.compute(4, matrix_values, 0.0, 1.0, 10, integrator="Boole")
    with pytest.raises(ValueError, match="divisibility"):
        magnus.compute(4, matrix_values, 0.0, 1.0, 10)  # Auto resolves to Boole
    with pytest.raises(ValueError, match="exceeds GL table"):
        magnus.compute(130, matrix_values, 0.0, 1.0, 9)


def test_complex_inputs_are_validated_before_device_work():
    """Complex data take the same validation path (shape errors surface as
    the reference's ValueError before any device work)."""
    with pytest.raises(ValueError, match="shape"):
        magnus.compute_sc(2, lambda t: np.ones((len(t), 4)) + 0j, 0.0, 1.0, 9)
    with pytest.raises(ValueError, match="divisibility"):
        magnus.compute(2, lambda t: matrix_values(t) + 0j, 0.0, 1.0, 10, integrator="Boole")


def test_precision_keyword_is_checked():
    with pytest.raises(ValueError, match="precision"):
        magnus.compute(1, matrix_values, 0.0, 1.0, 9, precision="bf16")


def test_generated_typing_matches_the_name_lists():
    """The committed Literal aliases are what the generator writes from the
    package's dispatch-name lists (src/api/typing_gen.cpp:43-50 in the
    reference), and each alias lists exactly the metadata function's names."""
    import inspect
    import typing

    from magnus_gb300 import _generated_typing as gt
    from magnus_gb300 import _typing_gen
    assert inspect.getsource(gt) == _typing_gen.typing_source()
    assert typing.get_args(gt.MatrixBackendName) == magnus.matrix_backends()
    assert typing.get_args(gt.IntegratorName) == magnus.integrators()
    assert typing.get_args(gt.GLBackendName) == magnus.gl_backends()
    assert typing.get_args(gt.NumericBackendName) == magnus.numeric_backends()
    assert typing.get_args(gt.KernelOpName) == magnus.ops()


def test_stub_declares_every_public_name():
    import ast
    import os
    stub = os.path.join(os.path.dirname(magnus.__file__), "__init__.pyi")
    with open(stub, encoding="utf-8") as f:
        tree = ast.parse(f.read())
    declared = {node.name for node in tree.body if isinstance(node, ast.FunctionDef)}
    assert set(magnus.__all__) <= declared
    assert os.path.exists(os.path.join(os.path.dirname(magnus.__file__), "py.typed"))
