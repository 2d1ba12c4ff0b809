"""Writes ``_generated_typing.py``: ``Literal`` aliases of the dispatch-name
lists, so that type checkers see the backend, integrator and op names of this
build (``"GB300"`` among the matrix backends).  Same aliases as the
reference's build-time generator (src/api/typing_gen.cpp:43-50); here the
names live in this package, so the generator reads them from it.

    python -m magnus_gb300._typing_gen [output-file]
"""
from __future__ import annotations

import json
import os
import sys


def typing_source() -> str:
    from . import _GL_BACKENDS, _INTEGRATORS, _MATRIX_BACKENDS, _NUMERIC, _OPS

    def alias(name, names, with_auto=False):
        items = list(names) + (["Auto"] if with_auto else [])
        return f"{name} = Literal[{', '.join(json.dumps(x) for x in items)}]\n"

    return ("from typing import Literal\n\n"
            + alias("NumericBackendName", _NUMERIC)
            + alias("MatrixBackendName", _MATRIX_BACKENDS, True)
            + alias("IntegratorName", _INTEGRATORS, True)
            + alias("GLBackendName", _GL_BACKENDS, True)
            + alias("KernelOpName", _OPS)
            + alias("PrecisionName", ("plain", "mixed")))


def default_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_generated_typing.py")


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) > 1:
        raise SystemExit("usage: python -m magnus_gb300._typing_gen [output-file]")
    path = argv[0] if argv else default_path()
    with open(path, "w", encoding="utf-8") as f:
        f.write(typing_source())
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
