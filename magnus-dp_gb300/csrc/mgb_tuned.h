// Selection of the shape-specialised chunk kernels with fallback to the
// generic level-major kernel.
#pragma once

#include <vector>

#include "mgb_kernels.h"

namespace mgb {

struct TunedChoice {
    bool use = false;
    int family = 0;  // 2: group-tiled CTA kernel (mixed, d = 16 / 32); 3: level-major tiled (mixed, d = 64 / 128)
    int D = 0;
    int nmax = 0;
    int ctas_per_sm = 1;
};

TunedChoice choose_tuned(bool plain, int kind, int rule, int mode, bool f64io, const std::vector<InstDev>& hi);
cudaError_t launch_big(int D, int rule, int mode, const LaunchArgs& a, int sms, bool prepare_only);
cudaError_t prepare_tuned(const TunedChoice& tc, int rule, int mode);
cudaError_t launch_tuned(const TunedChoice& tc, bool plain, int kind, int rule, int mode, const LaunchArgs& a, int sms);
cudaError_t launch_chunk_any(bool plain, int kind, int rule, int mode, const LaunchArgs& a,
                             const std::vector<InstDev>& hi, int sms);

}  // namespace mgb
