// Host-visible launch interface of the engine kernels (no torch types).
#pragma once

#include <cstdint>
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

// Per-instance small math, one CTA per instance.
cudaError_t launch_small(bool fp64, int kind, int which, const InstDev* insts, int count, int f64io, int write_out,
                         cudaStream_t st);

}  // namespace mgb
