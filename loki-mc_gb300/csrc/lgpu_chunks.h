// lgpu_chunks.h - how the batched passes cut many conditions into chunks.
//
// The moment and distribution passes of a batch list each condition's full
// chunks first (an exclusive prefix over the conditions) and then one
// remainder chunk per condition, largest first. Their blocks take the list in
// snake order - rounds of one chunk per block, every other round in reverse
// block order - so over a list sorted by size the blocks' totals differ by
// about one remainder. The host builds the list (layout_pass); the kernels
// map a chunk index back to (condition, first electron) (pass_chunk). Both
// halves are here, usable from host C++ and device code alike.
#pragma once

#if defined(__CUDACC__)
#define LGPU_HD __host__ __device__ __forceinline__
#else
#define LGPU_HD inline
#endif

#if !defined(__CUDA_ARCH__)
#include <algorithm>
#include <utility>
#include <vector>
#endif

namespace lgpu {

// largest s < n_slots with prefix[s] <= c, for 0 <= c < prefix[n_slots]
LGPU_HD int slot_of_chunk(const int* prefix, int n_slots, int c) {
  int lo = 0, hi = n_slots;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= c) lo = mid;
    else hi = mid;
  }
  return lo;
}

struct ChunkRef {
  int slot, first;
};

// chunk c of a pass: its condition and first electron (the chunk ends at
// first + chunk or at the condition's last electron)
LGPU_HD ChunkRef pass_chunk(const int* full_prefix, const int* part_slot, int n_slots, int n_full, int chunk, int c) {
  ChunkRef r;
  if (c < n_full) {
    r.slot = slot_of_chunk(full_prefix, n_slots, c);
    r.first = (c - full_prefix[r.slot]) * chunk;
  } else {
    r.slot = part_slot[c - n_full];
    r.first = (full_prefix[r.slot + 1] - full_prefix[r.slot]) * chunk;
  }
  return r;
}

// the chunk block b of G takes in round r
LGPU_HD int snake_index(int r, int G, int b) { return r * G + ((r & 1) ? G - 1 - b : b); }

#if !defined(__CUDA_ARCH__)
// The pass over the conditions s < n_slots with take[s]: full_prefix[0..n_slots]
// gets the exclusive prefix of their full chunks, part_slot the conditions
// with a remainder, largest remainder first (ties in condition order).
// Returns {full chunks, remainder chunks}; `rem` is scratch.
inline std::pair<int, int> layout_pass(int n_slots, const int* n, const unsigned char* take, int chunk,
                                       int* full_prefix, int* part_slot, std::vector<std::pair<int, int>>& rem) {
  rem.clear();
  int full = 0;
  for (int s = 0; s < n_slots; ++s) {
    full_prefix[s] = full;
    if (!take[s]) continue;
    full += n[s] / chunk;
    if (n[s] % chunk) rem.emplace_back(n[s] % chunk, s);
  }
  full_prefix[n_slots] = full;
  std::stable_sort(rem.begin(), rem.end(),
                   [](const std::pair<int, int>& x, const std::pair<int, int>& y) { return x.first > y.first; });
  for (size_t k = 0; k < rem.size(); ++k) part_slot[k] = rem[k].second;
  return {full, (int)rem.size()};
}
#endif

}  // namespace lgpu
