// Host-visible launch interface of the engine kernels (no torch types).
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "mgb_common.cuh"

namespace mgb {

enum ChunkMode : int { MODE_LOCAL = 0, MODE_CARRY = 1, MODE_VJP = 2 };
enum SmallKernel : int { SMALL_SCAN = 0, SMALL_FIN_FWD = 1, SMALL_FIN_VJP = 2, SMALL_RSCAN = 3 };

struct LaunchArgs {
    const InstDev* insts;
    const ChunkRef* work;
    int64_t nwork;
    void* scratch;        // grid * slot_elems elements of the compute type
    int64_t slot_elems;
    int64_t grid;
    int f64io;            // problem dtype is float64
    cudaStream_t stream;
};

// Generic level-major chunk kernel (any d, SpaceCurve).  Slot size in
// elements: (n + 4) * (K + 1) * m for the largest instance.
cudaError_t launch_generic_chunk(bool fp64, int kind, int rule, int mode, const LaunchArgs& a);

// Per-instance small math: one CTA per instance, or one warp per instance
// (eight to a CTA) when every instance has n d^2 <= 256 (nm_max: the largest
// n d^2 of the instances).
cudaError_t launch_small(bool fp64, int kind, int which, const InstDev* insts, int count, int f64io, int write_out,
                         int64_t nm_max, cudaStream_t st);

// Chunk scans spread over the GPU (mgb_scan.cu), for matrix instances with
// d a multiple of 16.  `insts` are `count` instances of one dimension sorted
// by chunk count (descending); active[c] = number of them with C > c.  The
// forward pass writes pi^0..pi^C; the reverse pass rho^{C-1}..rho^0 (from
// tau) and zeroes the dA rows shared by two chunks.
// Complex matrix problems as real 2d x 2d problems (mgb_complex.cu): count
// complex d x d matrices (interleaved re, im; float or double parts) to
// [[X, -Y], [Y, X]] (cot: the cotangent form [[Re C, Im C], [-Im C, Re C]] / 2),
// and back (grad: the bilinear gradient (dR11 + dR22) + i (dR12 - dR21)).
cudaError_t launch_cplx_embed(bool f64, const void* Z, void* out, int64_t count, int d, bool cot, cudaStream_t st);
cudaError_t launch_cplx_extract(bool f64, const void* in, void* Z, int64_t count, int d, bool grad, cudaStream_t st);

// Complex SpaceCurve data as the real 8 x 8 matrix problem (op many) on the
// embedding of rho(0, f) (mgb_complex.cu).  count: samples (SC_EMBED,
// SC_GRAD, SC_CARRY), unused for SC_COT / SC_OUT (n orders, op of the call).
enum { SC_EMBED = 0, SC_COT = 1, SC_OUT = 2, SC_GRAD = 3, SC_CARRY = 4 };
cudaError_t launch_sc_complex(int what, bool f64, const void* src, void* dst, int64_t count, int n, int op,
                              cudaStream_t st);

// The small FP64 algebra after the scans, spread over the GPU (mgb_fin.cu),
// for the same segments as the tiled scans.  vjp = false: D^(q), E, Omega
// (and the op output when write_out); vjp = true: tau (after the former).
cudaError_t launch_fin_tiled(const InstDev* insts, int count, int d, int nmax, bool vjp, int write_out, int f64io,
                             cudaStream_t st);

bool scan_tiled_ok(int kind, int d);
// Mixed-form chunk scans in double-FP32 arithmetic, one CTA per instance and
// one launch per direction (mgb_scan_df.cu), for d = 16 / 32 matrices whose
// state and transfers (4 n d^2 floats) fit in 200 KB of shared memory.
bool scan_df_ok(int kind, int d, int nmax);
cudaError_t launch_scan_df(const InstDev* insts, int count, int d, int nmax, bool reverse, int f64io,
                           cudaStream_t st, bool prepare_only = false);
cudaError_t launch_scan_tiled(const InstDev* insts, int count, int d, int nmax, const std::vector<int32_t>& active,
                              bool reverse, int f64io, cudaStream_t st);

}  // namespace mgb
