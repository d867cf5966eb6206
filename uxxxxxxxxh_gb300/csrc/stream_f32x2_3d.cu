// Streaming-kernel variants for one storage/arithmetic pair and rank
// (instantiated in their own translation unit so builds run in parallel).
#include "stream_launch.cuh"

namespace uhs {
cudaError_t launch_stream_f32x2_3d(const StreamCall &c) { return dispatch_shape<kStF32x2, kArDf32, false>(c); }
}  // namespace uhs
