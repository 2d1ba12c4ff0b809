"""Writes gl_table.inc: the default Gauss-Legendre table compiled into the
library (orders 1..64, nodes x = (xi + 1) / 2 and weights w / 2 on [0, 1],
from numpy.polynomial.legendre.leggauss, i.e. the same values the reference
bakes into its binary table in src/util/gen_nodes.py:11-47 and that
magnus.replace_gl_table recomputes in src/api/magnus/__init__.py:38-55).

Layout: order q occupies entries [q(q-1)/2, q(q-1)/2 + q) of both arrays,
the reference's offset scheme (src/api/pybind.cpp:77-88).  Values are
emitted as C99 hex-float literals so the table is bit-exact.
"""
import sys

import numpy as np

MAX_ORDER = 64


def main(out_path: str) -> None:
    nodes, weights = [], []
    for q in range(1, MAX_ORDER + 1):
        x, w = np.polynomial.legendre.leggauss(q)
        nodes.extend(float(v) for v in 0.5 * (x + 1.0))
        weights.extend(float(v) for v in 0.5 * w)
    with open(out_path, "w") as f:
        f.write("// generated by gen_gl_table.py; do not edit\n")
        f.write(f"#define MGB_GL_DEFAULT_MAX_ORDER {MAX_ORDER}\n")
        f.write("static const double mgb_gl_default_nodes[] = {\n")
        f.write(",\n".join(v.hex() for v in nodes))
        f.write("\n};\nstatic const double mgb_gl_default_weights[] = {\n")
        f.write(",\n".join(v.hex() for v in weights))
        f.write("\n};\n")


if __name__ == "__main__":
    main(sys.argv[1])
