// lgpu_advance_stash.cu - the batched advance in the stash launch shape
// (warp_loop_stash: pending collisions parked in shared memory while the
// lanes keep flying).
#include "lgpu_advance.cuh"

namespace lgpu {

int launch_batch_advance_stash(const BatchArgs& b, int sm_count, unsigned parts, cudaStream_t s) {
  return launch_batch_advance_shape<kFirstStashShape>(b, sm_count, parts, s);
}

cudaError_t prepare_advance_stash() { return prepare_batch_advance_shape<kFirstStashShape>(); }

}  // namespace lgpu
