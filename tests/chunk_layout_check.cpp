// Host check of lgpu_chunks.h (compiled with g++ by test_chunk_layout.py).
//
// For random sets of conditions, chunk sizes and grid sizes: the layout the
// batch stages (layout_pass) walked in the order the kernels take it
// (snake_index over the blocks, pass_chunk per chunk index) visits every chunk
// once and covers every electron of every included condition exactly once and
// no electron of an excluded one. On sweep-like sets of conditions (64,
// log-uniform 1e4..2e6 electrons, 65535-electron chunks, 152 blocks) the
// busiest block takes at most one chunk more than the mean (a round-robin in
// condition order exceeds that on such sets).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <utility>
#include <vector>

#include "lgpu_chunks.h"

static int failures = 0;
#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      std::printf("FAIL: " __VA_ARGS__); \
      std::printf("\n");                 \
      ++failures;                        \
    }                                    \
  } while (0)

// electrons each block takes; checks coverage on the way
static std::vector<long long> walk(const std::vector<int>& n, const std::vector<unsigned char>& take, int chunk,
                                   int G, bool per_electron) {
  const int ns = (int)n.size();
  std::vector<int> prefix(ns + 1), part(ns);
  std::vector<std::pair<int, int>> rem;
  const auto lay = lgpu::layout_pass(ns, n.data(), take.data(), chunk, prefix.data(), part.data(), rem);
  const int total = lay.first + lay.second;
  std::vector<char> seen(total, 0);
  std::vector<long long> covered(ns, 0), block(G, 0);
  std::vector<std::vector<unsigned char>> cover(ns);
  if (per_electron)
    for (int s = 0; s < ns; ++s) cover[s].assign(n[s], 0);
  for (int b = 0; b < G; ++b) {
    for (int r = 0; r * G < total; ++r) {
      const int c = lgpu::snake_index(r, G, b);
      if (c >= total) continue;
      CHECK(!seen[c], "chunk %d visited twice", c);
      seen[c] = 1;
      const lgpu::ChunkRef k = lgpu::pass_chunk(prefix.data(), part.data(), ns, lay.first, chunk, c);
      CHECK(k.slot >= 0 && k.slot < ns, "chunk %d: slot %d out of range", c, k.slot);
      if (k.slot < 0 || k.slot >= ns) continue;
      CHECK(take[k.slot], "chunk %d in an excluded condition %d", c, k.slot);
      CHECK(k.first >= 0 && k.first < n[k.slot], "chunk %d: first %d outside %d electrons", c, k.first, n[k.slot]);
      const int last = std::min(k.first + chunk, n[k.slot]);
      covered[k.slot] += last - k.first;
      block[b] += last - k.first;
      if (per_electron)
        for (int i = k.first; i < last; ++i) cover[k.slot][i]++;
    }
  }
  for (int c = 0; c < total; ++c) CHECK(seen[c], "chunk %d never visited", c);
  for (int s = 0; s < ns; ++s) {
    CHECK(covered[s] == (take[s] ? n[s] : 0), "condition %d: %lld of %d electrons covered", s, covered[s], n[s]);
    if (per_electron && take[s])
      for (int i = 0; i < n[s]; ++i) CHECK(cover[s][i] == 1, "condition %d electron %d covered %d times", s, i, cover[s][i]);
  }
  return block;
}

int main() {
  std::mt19937 rng(20261204u);
  const int chunks[] = {7, 100, 4096, 65535};
  for (int trial = 0; trial < 400 && failures < 20; ++trial) {
    const int ns = 1 + (int)(rng() % 70);
    const int chunk = chunks[rng() % 4];
    std::vector<int> n(ns);
    std::vector<unsigned char> take(ns);
    for (int s = 0; s < ns; ++s) {
      n[s] = 1 + (int)(rng() % (5u * (unsigned)chunk));
      take[s] = (rng() % 4) != 0;
    }
    const int G = 1 + (int)(rng() % 400);
    walk(n, take, chunk, G, chunk < 1000);
  }
  // balance on sweep-like sets
  for (int trial = 0; trial < 50 && failures < 20; ++trial) {
    std::vector<int> n(64);
    std::vector<unsigned char> take(64, 1);
    std::uniform_real_distribution<double> u(std::log(1e4), std::log(2e6));
    long long sum = 0;
    for (int s = 0; s < 64; ++s) {
      n[s] = (int)std::exp(u(rng));
      sum += n[s];
    }
    const std::vector<long long> block = walk(n, take, 65535, 152, false);
    const double mean = (double)sum / 152.0;
    const double peak = (double)*std::max_element(block.begin(), block.end());
    CHECK(peak <= mean + 65535.0, "busiest block %.0f electrons against a mean of %.0f", peak, mean);
  }
  if (failures == 0) std::printf("ok\n");
  return failures ? 1 : 0;
}
