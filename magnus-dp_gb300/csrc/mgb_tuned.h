// Selection of the shape-specialised chunk kernels with fallback to the
// generic level-major kernel, and their launch variants (the autotuner in
// mgb_api.cu times the variants of a segment's kernel and keeps the fastest).
#pragma once

#include <vector>

#include "mgb_kernels.h"

namespace mgb {

struct TunedChoice {
    bool use = false;
    int family = 0;  // 1: thread-per-chunk registers (d = 2, SpaceCurve); 2: group-tiled CTA kernel (mixed, d = 16 / 32); 3: tensor-core level-major (mixed, d = 64 / 128)
    int D = 0;
    int nmax = 0;
    int ctas_per_sm = 1;
    int variant = 0;    // launch variant of the family's kernel
    int nvariants = 1;  // variants the autotuner may choose from
};

// Scratch geometry of a segment: per-slot elements (compute type) and the
// number of slots (CTAs, or threads for the thread-per-chunk family).
struct SegSizing {
    int64_t slot_elems = 0;
    int64_t grid = 0;
};
SegSizing size_segment(bool plain, int kind, int rule, bool f64io, const std::vector<InstDev>& hi, int64_t nwork,
                       int sms, size_t budget_bytes);
cudaError_t launch_small_family(bool plain, int kind, int rule, int mode, const LaunchArgs& a);
int small_family_max_levels();

TunedChoice choose_tuned(bool plain, int kind, int rule, int mode, bool f64io, const std::vector<InstDev>& hi,
                         int variant);
// Tensor-core chunk kernel (mgb_bigtc.cu) for the mixed form at d = 64 / 128.
// Variants: d = 64: k-block 32 or 64 x 2 or 1 CTAs per SM; d = 128: k-block
// 32 or 64.  The grid is min(a.grid, sms x CTAs per SM).
cudaError_t launch_big(int D, int rule, int mode, const LaunchArgs& a, int sms, int variant, bool prepare_only);
int big_variants(int D);
int big_ctas_per_sm(int D, int variant);
// Group-tiled kernel (mgb_tuned.cu), variant 0: 2 CTAs per SM, 1: one;
// at d = 32 variant 2: the tcgen05 forward local pass (mgb_tiletc.cu) with
// the warp-MMA VJP, variant 3: the warp-MMA kernel for both.
cudaError_t launch_tile(int D, int rule, int mode, const LaunchArgs& a, int grid, int variant, bool prepare_only);
cudaError_t launch_tiletc(int rule, const LaunchArgs& a, int grid, bool prepare_only);
// Warp-MMA kernel at d = 32 (mgb_mma32.cu), forward local pass and VJP; two
// CTAs per SM.
cudaError_t launch_mma32(int rule, int mode, const LaunchArgs& a, int grid, bool prepare_only);
// Device address of the time-out flag the tensor-core kernels raise.
int* device_timeout_ptr();
// One CTA waits (limit_ns) on an mbarrier nothing arrives at and raises the
// time-out flag (mgb_selftest.cu).
cudaError_t launch_wait_selftest(uint64_t limit_ns, cudaStream_t st);
// Generic kernel variants: 8, 4 or 2 CTAs per SM.
constexpr int GENERIC_VARIANTS = 3;
int generic_ctas_per_sm(int variant);
// 1 if a kernel gave up a bounded device-side wait since the last call.
int read_clear_device_timeout();
cudaError_t prepare_tuned(const TunedChoice& tc, int rule, int mode);
cudaError_t launch_tuned(const TunedChoice& tc, bool plain, int kind, int rule, int mode, const LaunchArgs& a, int sms);
cudaError_t launch_chunk_any(bool plain, int kind, int rule, int mode, const LaunchArgs& a,
                             const std::vector<InstDev>& hi, int sms, int variant);

}  // namespace mgb
