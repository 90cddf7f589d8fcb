// lgpu_advance_stash.cu - the batched advance in the stash launch shapes
// (warp_loop_stash: pending collisions parked in shared memory while the
// lanes keep flying), 256 threads x 4 blocks and 512 x 2 per SM.
#include "lgpu_advance.cuh"

namespace lgpu {

int launch_batch_advance_stash(const BatchArgs& b, int sm_count, unsigned parts, int shape, cudaStream_t s) {
  return shape == 5 ? launch_batch_advance_shape<5>(b, sm_count, parts, s)
                    : launch_batch_advance_shape<4>(b, sm_count, parts, s);
}

cudaError_t prepare_advance_stash() {
  cudaError_t e = prepare_batch_advance_shape<4>();
  return e == cudaSuccess ? prepare_batch_advance_shape<5>() : e;
}

}  // namespace lgpu
