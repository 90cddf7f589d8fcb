// lgpu_advance_batch.cu - the batched advance in the warp-turn launch shapes
// and the dispatch over all shapes; the stash shape compiles in
// lgpu_advance_stash.cu (the two translation units build in parallel).
#include "lgpu_advance.cuh"

namespace lgpu {

int launch_batch_advance(const BatchArgs& b, int sm_count, unsigned parts, int shape, cudaStream_t s) {
  switch (shape) {
    case 1: return launch_batch_advance_shape<1>(b, sm_count, parts, s);
    case 2: return launch_batch_advance_shape<2>(b, sm_count, parts, s);
    case 3: return launch_batch_advance_shape<3>(b, sm_count, parts, s);
    case 4:
    case 5: return launch_batch_advance_stash(b, sm_count, parts, shape, s);
    default: return launch_batch_advance_shape<0>(b, sm_count, parts, s);
  }
}

void advance_shape(int shape, int* threads, int* blocks_per_sm, int* chunk, int* stash) {
  switch (shape) {
    case 1: return shape_of<1>(threads, blocks_per_sm, chunk, stash);
    case 2: return shape_of<2>(threads, blocks_per_sm, chunk, stash);
    case 3: return shape_of<3>(threads, blocks_per_sm, chunk, stash);
    case 4: return shape_of<4>(threads, blocks_per_sm, chunk, stash);
    case 5: return shape_of<5>(threads, blocks_per_sm, chunk, stash);
    default: return shape_of<0>(threads, blocks_per_sm, chunk, stash);
  }
}

}  // namespace lgpu
