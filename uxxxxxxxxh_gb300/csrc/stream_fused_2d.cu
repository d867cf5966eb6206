// Temporal fusion of rank-2 star and box stencils (the kernel:
// stream_fused.cuh), compiled apart from the rank-3 variants.
#include "stream_fused.cuh"

namespace uhs {

cudaError_t launch_fused_2d(const StreamCall &c, int K) { return fused::launch_fused_rank<kStar2, kBox2>(c, K); }

}  // namespace uhs
