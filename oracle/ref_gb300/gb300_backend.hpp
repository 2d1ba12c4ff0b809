// The "GB300" matrix backend as the reference's own pybind11 module would
// carry it: the bodies behind the two lines that route run_typed and
// run_vjp_typed (src/api/pybind.cpp:146-192, :239-298) to the engine's C ABI
// (include/magnus_gb300.h) before the reference resolves its CPU backends.
//
// Test infrastructure: compiled only into the reference module that
// oracle/build_ref.sh builds under oracle/_ref/gb300/ (git-ignored), next to
// the unmodified one.  The routing lines themselves are inserted into a copy
// of pybind.cpp by oracle/ref_gb300/patch_pybind.py; the reference's input
// and cotangent shape checks run before them, exactly as for its own
// backends.
//
// Mapping: the element type picks MGB_DTYPE_*; the precision is PLAIN (the
// reference's arithmetic); op names go through the reference's own
// Dispatch::op_from_str (ONE/MANY/SUM = 0/1/2 in both); integrator "Auto"
// resolves to Boole as the reference's type list does
// (src/integration/backends.hpp:53-58).  The GL backend selects how the
// reference runs its node lanes and does not change results; the engine
// collapses the nodes, so it is accepted and not used.  A recorded carry
// passed to compute_vjp is shape-checked by the reference and then not read:
// the engine replays from its own checkpoints (equal for any carry that
// compute(record_vjp=True) produced).
//
// Errors: MGB_ERR_TYPE -> TypeError, MGB_ERR_INVALID_ARGUMENT ->
// std::invalid_argument (ValueError), anything else (no CUDA device, a CUDA
// failure, a device-side time-out) -> RuntimeError with the engine's message.
#pragma once

#include <complex>
#include <stdexcept>
#include <string>
#include <string_view>
#include <type_traits>

#include <pybind11/pybind11.h>

#include "magnus_gb300.h"

namespace gb300_backend {

template <class NumT>
constexpr int32_t dtype_code() {
    if constexpr (std::is_same_v<NumT, float>) return MGB_DTYPE_F32;
    else if constexpr (std::is_same_v<NumT, double>) return MGB_DTYPE_F64;
    else if constexpr (std::is_same_v<NumT, std::complex<float>>) return MGB_DTYPE_C64;
    else return MGB_DTYPE_C128;
}

inline int32_t integrator_code(std::string_view s) {
    if (s == "Auto" || s == "Boole") return MGB_INTEGRATOR_BOOLE;
    if (s == "Simpson") return MGB_INTEGRATOR_SIMPSON;
    if (s == "Trapezoid") return MGB_INTEGRATOR_TRAPEZOID;
    if (s == "Riemann") return MGB_INTEGRATOR_RIEMANN;
    throw std::invalid_argument("Could not resolve dispatch name option");
}

inline void raise_for(mgb_status st) {
    if (st == MGB_OK) return;
    const std::string msg = mgb_last_error();
    if (st == MGB_ERR_TYPE) throw pybind11::type_error(msg);
    if (st == MGB_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
    throw std::runtime_error("GB300 backend: " + msg);
}

template <class NumT>
mgb_problem problem(size_t n, size_t samples, size_t dim, double t0, double tf, std::string_view op,
                    std::string_view integrator) {
    mgb_problem p{};
    p.kind = MGB_KIND_MATRIX;
    p.dtype = dtype_code<NumT>();
    p.precision = MGB_PRECISION_PLAIN;
    p.op = (int32_t)Magnus::Dispatch::op_from_str(op);
    p.integrator = integrator_code(integrator);
    p.n = n;
    p.samples = samples;
    p.dim = dim;
    p.t0 = t0;
    p.tf = tf;
    return p;
}

// Forward: out (and, when recorded, the carry in the reference's layout).
template <class NumT>
void forward(size_t n, const NumT* in, NumT* out, NumT* carry, size_t samples, size_t dim, double t0, double tf,
             std::string_view op, std::string_view integrator) {
    const mgb_problem p = problem<NumT>(n, samples, dim, t0, tf, op, integrator);
    mgb_status st;
    {
        pybind11::gil_scoped_release release;
        st = mgb_forward_host(&p, in, out, carry);
    }
    raise_for(st);
}

// VJP: dA (S, d, d) from the cotangent on the forward's output.
template <class NumT>
void vjp(size_t n, const NumT* in, const NumT* cot, NumT* dA, size_t samples, size_t dim, double t0, double tf,
         std::string_view op, std::string_view integrator) {
    const mgb_problem p = problem<NumT>(n, samples, dim, t0, tf, op, integrator);
    mgb_status st;
    {
        pybind11::gil_scoped_release release;
        st = mgb_vjp_host(&p, in, cot, dA);
    }
    raise_for(st);
}

}  // namespace gb300_backend
