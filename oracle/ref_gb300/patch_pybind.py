"""Write a copy of the reference's src/api/pybind.cpp with the "GB300" matrix
backend routed to the engine: the lines a maintainer adds to bind the engine
into the reference's own pybind11 module.

Test infrastructure (run by oracle/build_ref.sh; the output goes to
oracle/_ref/gb300/, git-ignored).  The inserted lines are this project's own;
each insertion point is found by a short anchor in the reference source and the
script fails loudly when one is missing.

    python patch_pybind.py <reference pybind.cpp> <output .cpp>

Insertions:
  * after `#include <pybind11/pybind11.h>`: the backend header
    (gb300_backend.hpp beside this script);
  * run_typed (src/api/pybind.cpp:146-192): before the block that calls
    run_raw_impl, `if (matrix_backend == "GB300")` -> gb300_backend::forward;
  * run_vjp_typed (src/api/pybind.cpp:239-298): before the block that calls
    run_vjp_raw_impl, the same -> gb300_backend::vjp;
  * the `matrix_backends` module function lists "GB300" after the
    reference's own names.
"""
import sys

FORWARD_HOOK = """    if (matrix_backend == "GB300") {
        gb300_backend::forward<NumT>(n, in, out_data, vjp_data, input_shape.samples, input_shape.dim, t0, tf, op,
                                     integrator);
        if (record_vjp) return py::make_tuple(out, vjp);
        return out;
    }

"""

VJP_HOOK = """    if (matrix_backend == "GB300") {
        gb300_backend::vjp<NumT>(n, static_cast<NumT*>(in_info.ptr), static_cast<NumT*>(cotangent_info.ptr),
                                 static_cast<NumT*>(out_info.ptr), input_shape.samples, input_shape.dim, t0, tf, op,
                                 integrator);
        return out;
    }

"""

BACKENDS_DEF = ("[]() { py::list names(Magnus::detail::matrix_backends()); names.append(\"GB300\"); "
                "return py::tuple(names); },")


def _find(src, anchor, start=0):
    i = src.find(anchor, start)
    if i < 0:
        raise SystemExit(f"patch_pybind: anchor not found: {anchor!r}")
    return i


def _insert_before_block(src, func_anchor, call_anchor, hook):
    """Insert `hook` before the `{` line that opens the block holding the
    first `call_anchor` after `func_anchor`."""
    f = _find(src, func_anchor)
    c = _find(src, call_anchor, f)
    blk = src.rfind("\n    {\n", f, c)
    if blk < 0:
        raise SystemExit(f"patch_pybind: no block opening before {call_anchor!r}")
    at = blk + 1
    return src[:at] + hook + src[at:]


def patch(src):
    inc = "#include <pybind11/pybind11.h>\n"
    i = _find(src, inc) + len(inc)
    src = src[:i] + '\n#include "gb300_backend.hpp"\n' + src[i:]
    src = _insert_before_block(src, "py::object run_typed(", "run_raw_impl(", FORWARD_HOOK)
    src = _insert_before_block(src, "py::array run_vjp_typed(", "run_vjp_raw_impl(", VJP_HOOK)
    anchor = "&Magnus::detail::matrix_backends,"
    i = _find(src, anchor)
    src = src[:i] + BACKENDS_DEF + src[i + len(anchor):]
    return src


def main(argv):
    if len(argv) != 3:
        raise SystemExit(__doc__)
    with open(argv[1]) as f:
        src = f.read()
    with open(argv[2], "w") as f:
        f.write(patch(src))


if __name__ == "__main__":
    main(sys.argv)
