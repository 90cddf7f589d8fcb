// lgpu_kernels.cu - sm_103a kernels of the electron Monte Carlo path.
//
//   k_advance       free flights + collisions of every electron up to the
//                   synchronisation time (BoltzmannMC.C:617-688, 804-1280)
//   k_init          Maxwellian start ensemble (BoltzmannMC.C:491-508)
//   k_build_tables  FP64 interpolated tables -> FP32 row pairs
//                   (BoltzmannMC.C:561-615)
//   k_sample        ensemble moments and maximum energy (BoltzmannMC.C:1410-1446)
//   k_hist          EEDF / EADF / EVDF tallies (BoltzmannMC.C:1550-1571)
//   k_pop_*         population control after ionization and attachment
//                   (BoltzmannMC.C:1282-1408)
//   k_replay_*      the same device functions on given inputs (parity tests)
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "lgpu_advance.cuh"
#include "lgpu_device.cuh"
#include "lgpu_kernels.cuh"

namespace lgpu {

namespace {

// the main pass over the ensemble and the drain of left-over secondaries
// carry different names so that profiles can tell them apart
template <int MODE>
__global__ void __launch_bounds__(kAdvanceThreads, kAdvanceBlocksPerSM) k_advance(AdvanceArgs a) {
  __shared__ AdvShared sh;
  advance_body<MODE>(a, sh);
}
template <int MODE>
__global__ void __launch_bounds__(32) k_advance_drain(AdvanceArgs a) {
  __shared__ AdvShared sh;
  // the warps took their own queues during the advance: only spilled
  // secondaries are left (the count is final: the advance launch came first)
  if (*(volatile const int*)a.spill_count == 0) return;
  advance_body<MODE>(a, sh);
}

// the drain of every slot's spilled secondaries: one warp per slot
__global__ void __launch_bounds__(32) k_advance_drain_batch(BatchArgs b) {
  __shared__ AdvShared sh;
  __shared__ AdvanceArgs s_a;
  const int slot = blockIdx.x;
  if (slot >= b.hdr->n_slots || !(b.slots[slot].flags & kSlotIonAtt)) return;
  // the warps took their own queues during the advance: only spilled
  // secondaries are left (the count is final: the advance launches came first)
  if (*(volatile const int*)b.slots[slot].adv.spill_count == 0) return;
  load_slot_args(&b.slots[slot].adv, &s_a);
  __syncthreads();
  if (threadIdx.x == 0) {
    s_a.queue_only = 1;
    s_a.salt = 2;
  }
  __syncthreads();
  advance_body<-1>(s_a, sh);
}

// ------------------------------------------------------------------ init
__global__ void k_init(InitArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.0f;
  if (i < a.n) {
    PhiloxStream rng;
    rng.init((uint32_t)i, 0xFFFFFFFFFFFFull, a.seed, 0x7u);
    // three normals from four uniforms (Box-Muller, MathFunctions.C:54-59)
    const float r1 = rng.oc(), r2 = rng.oc(), r3 = rng.oc(), r4 = rng.oc();
    const float aa = sqrtf(-2.0f * logf(r1));
    float sb, cb;
    sincosf(kTwoPiF * r2, &sb, &cb);
    const float3 v = make_float3(aa * cb * a.sd, aa * sb * a.sd, sqrtf(-2.0f * logf(r3)) * cosf(kTwoPiF * r4) * a.sd);
    a.state[2 * i] = make_float4(0.f, 0.f, 0.f, -1.0f);
    a.state[2 * i + 1] = make_float4(v.x, v.y, v.z, 0.0f);
    e = energy_of(v, a.half_me_over_e);
  }
  e = warp_max(e);
  if ((threadIdx.x & 31) == 0 && e > 0.0f) atomic_max_energy(a.max_energy_bits, e);
}

// --------------------------------------------------------------- tables
// Linear interpolation of the raw table (the bracketing index by bisection,
// largest i with x_i <= x clamped to n-2, then y_i + (x-x_i)/(x_{i+1}-x_i)*(y_{i+1}-y_i)),
// with explicit round-to-nearest operations so no FMA contraction happens.
__device__ double interp_raw(const double* xs, const double* ys, int n, double x) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (hi + lo) >> 1;
    if (xs[mid] > x) hi = mid; else lo = mid;
  }
  const double dx = __dsub_rn(xs[lo + 1], xs[lo]);
  return __dadd_rn(ys[lo], __dmul_rn(__ddiv_rn(__dsub_rn(x, xs[lo]), dx), __dsub_rn(ys[lo + 1], ys[lo])));
}

// sigma*n of process p at `energy` (a superelastic process reads its
// inelastic partner's raw table at energy + threshold)
__device__ double table_value(const TableBuildArgs& a, int p, double energy) {
  if (a.is_super[p]) {
    if (energy > a.emin[p] && energy <= a.emax[p]) {
      const double thr = a.emin[p - 1];
      const double sg = interp_raw(a.raw_e + a.raw_off[p - 1], a.raw_v + a.raw_off[p - 1], a.raw_len[p - 1],
                                   __dadd_rn(energy, thr));
      return __dmul_rn(__dmul_rn(__dmul_rn(a.superw[p], __dadd_rn(1.0, __ddiv_rn(thr, energy))), sg), a.rel_dens[p]);
    }
  } else if (energy >= a.emin[p] && energy <= a.emax[p]) {
    return __dmul_rn(interp_raw(a.raw_e + a.raw_off[p], a.raw_v + a.raw_off[p], a.raw_len[p], energy), a.rel_dens[p]);
  }
  return 0.0;
}

// One warp per energy row: the lanes interpolate the processes of the row in
// parallel, then the cumulative row is summed in process order (the order
// fixes the FP64 rounding) and written as FP32 row pairs.
constexpr int kTableWarps = 4;

__global__ void __launch_bounds__(32 * kTableWarps) k_build_tables(TableBuildArgs a) {
  __shared__ double s_val[kTableWarps][kMaxProcesses];
  __shared__ double s_cum[kTableWarps][kMaxProcesses];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * kTableWarps + w;
  if (i >= a.M) return;  // whole warps
  const int P = a.P;
  const double energy = __dmul_rn((double)i, a.step);
  for (int p = lane; p < P; p += 32) s_val[w][p] = table_value(a, p, energy);
  __syncwarp();
  if (lane == 0) {
    double cur = 0.0;
    for (int p = 0; p < P; ++p) {
      cur = __dadd_rn(cur, s_val[w][p]);
      s_cum[w][p] = cur;
    }
  }
  __syncwarp();
  for (int p = lane; p < a.stride; p += 32) {
    const size_t k = (size_t)i * a.stride + p;
    if (p < P) {
      const double value = s_val[w][p], cur = s_cum[w][p];
      if (a.sig64) a.sig64[(size_t)i * P + p] = value;
      if (a.cum64) a.cum64[(size_t)i * P + p] = cur;
      const float vf = (float)value, cf = (float)cur;
      a.sig_pair[k].x = vf;
      a.cum_pair[k].x = cf;
      if (i > 0) {
        a.sig_pair[k - a.stride].y = vf;
        a.cum_pair[k - a.stride].y = cf;
      }
      if (i == a.M - 1) {
        a.sig_pair[k].y = vf;
        a.cum_pair[k].y = cf;
      }
    } else {
      // row padding: a cumulative value no random number reaches, zero rate
      a.cum_pair[k] = make_float2(3.0e38f, 3.0e38f);
      a.sig_pair[k] = make_float2(0.0f, 0.0f);
    }
  }
  if (lane == 0) {
    const double cur = s_cum[w][P - 1];
    const double kq = 1.6021766208e-19, km = 9.10938356e-31;
    const double nu = __dmul_rn(cur, __dmul_rn(a.N, __dsqrt_rn(__ddiv_rn(__dmul_rn(__dmul_rn(energy, 2.0), kq), km))));
    a.nu_tot[i] = nu;
    a.nu_pair[i].x = (float)nu;
    if (i > 0) a.nu_pair[i - 1].y = (float)nu;
    if (i == a.M - 1) a.nu_pair[i].y = (float)nu;
  }
}

// running maximum of nu_tot (one block of 1024 threads, tiles of 1024 rows;
// max is exact in any order)
constexpr int kPrefixThreads = 1024;

__global__ void __launch_bounds__(kPrefixThreads) k_prefix_max(const double* nu_tot, double* nu_max, int M) {
  __shared__ double s_w[kPrefixThreads / 32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  double carry = 0.0;
  for (int base = 0; base < M; base += kPrefixThreads) {
    const int i = base + t;
    double v = i < M ? nu_tot[i] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v = fmax(v, u);
    }
    if (lane == 31) s_w[w] = v;
    __syncthreads();
    if (w == 0) {
      double x = s_w[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = fmax(x, u);
      }
      s_w[lane] = x;
    }
    __syncthreads();
    double r = fmax(carry, v);
    if (w > 0) r = fmax(r, s_w[w - 1]);
    if (i < M) nu_max[i] = r;
    carry = fmax(carry, s_w[kPrefixThreads / 32 - 1]);
    __syncthreads();
  }
}

// block bounds of the total frequency for the coarse null test: the largest
// FP32 value of rows [b R, (b+1) R] (row pairs cover the next row), raised
// by 2^-20 relative against the rounding of the interpolation
__global__ void k_coarse_max(const float2* nu_pair, int M, int shift, float* coarse, int n_coarse) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_coarse) return;
  const int i0 = b << shift, i1 = min((b + 1) << shift, M);
  float m = 0.0f;
  for (int i = i0; i < i1; ++i) {
    const float2 v = nu_pair[i];
    m = fmaxf(m, fmaxf(v.x, v.y));
  }
  coarse[b] = m * (1.0f + 9.5367431640625e-7f);
}

// ---------------------------------------------------------------- sample
constexpr int kSampleThreads = 256;

// Moment sums of electrons begin, begin+step, ... < end into a.moments: per
// thread in FP32 (a handful of electrons each), FP64 from the warp reduction on.
// Every thread of the block calls this; s_m is the block's scratch.
struct NoExtra {
  __device__ __forceinline__ void operator()(float4) const {}
};

// `extra` sees every electron's (vx, vy, vz, flag) in the same pass (the
// batched kernel counts the EVDF with it)
template <class Extra = NoExtra>
__device__ __forceinline__ void sample_range(const SampleArgs& a, int begin, int end, int step,
                                             double (*s_m)[kMoments], Extra extra = Extra()) {
  float m[kMoments];
#pragma unroll
  for (int k = 0; k < kMoments; ++k) m[k] = 0.0f;
  float e_max = 0.0f;
  auto add = [&](float4 A, float4 B) {
    extra(B);
    const float e = energy_of(make_float3(B.x, B.y, B.z), a.half_me_over_e);
    e_max = fmaxf(e_max, e);
    const float x = A.x, y = A.y, z = A.z, vx = B.x, vy = B.y, vz = B.z;
    m[0] += e;
    m[1] += x; m[2] += y; m[3] += z;
    m[4] += vx; m[5] += vy; m[6] += vz;
    m[7] += x * x; m[8] += x * y; m[9] += x * z; m[10] += y * y; m[11] += y * z; m[12] += z * z;
    m[13] += x * vx; m[14] += x * vy; m[15] += x * vz;
    m[16] += y * vx; m[17] += y * vy; m[18] += y * vz;
    m[19] += z * vx; m[20] += z * vy; m[21] += z * vz;
  };
  // four electrons' loads in flight before their sums (memory-level parallelism)
  int i = begin;
  for (; i + 3 * step < end; i += 4 * step) {
    float4 A[4], B[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) load_record(a.state + 2 * (i + u * step), A[u], B[u]);
#pragma unroll
    for (int u = 0; u < 4; ++u) add(A[u], B[u]);
  }
  for (; i < end; i += step) {
    float4 A, B;
    load_record(a.state + 2 * i, A, B);
    add(A, B);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // FP32 tree reduction inside the warp (32 partials), FP64 across warps and blocks
#pragma unroll
  for (int k = 0; k < kMoments; ++k) {
    float w = m[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (lane == 0) s_m[wid][k] = (double)w;
  }
  e_max = warp_max(e_max);
  if (lane == 0 && e_max > 0.0f) atomic_max_energy(a.max_energy_bits, e_max);
  __syncthreads();
  if (threadIdx.x < kMoments) {
    double sum = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += s_m[w][threadIdx.x];
    atomicAdd(&a.moments[threadIdx.x], sum);
  }
}

__global__ void __launch_bounds__(kSampleThreads) k_sample(SampleArgs a) {
  __shared__ double s_m[kSampleThreads / 32][kMoments];
  sample_range(a, blockIdx.x * blockDim.x + threadIdx.x, a.n, gridDim.x * blockDim.x, s_m);
}

// ------------------------------------------------------------- histograms
// The tallies of one sample in two passes over the electrons' velocities,
// each in blocks of up to kHistChunk electrons that count in shared memory and
// then add one atomic per occupied cell to the FP64 tallies:
//   pass A: EEDF counts (32-bit) and EADF counts (16-bit, two per word),
//   pass B: EVDF counts (16-bit, two per word), cylindrical conditions only.
// A block's chunk is below 2^16 electrons, so no 16-bit count can carry into
// its neighbour. A condition whose grid is larger than the block's shared
// memory counts that tally with global atomics instead.
constexpr int kHistChunk = kBatchHistChunk;  // below 2^16: 16-bit counts cannot carry
constexpr int kHistAThreads = 1024;
constexpr int kHistBThreads = 512;
constexpr int kHistASmem = 224 * 1024;  // one block per SM
constexpr int kHistBSmem = 96 * 1024;   // two blocks per SM

__device__ __forceinline__ float radial_speed(float v2xy) { return v2xy > 0.0f ? v2xy * rsqrtf(v2xy) : 0.0f; }

__device__ __forceinline__ void hist_cells(const HistArgs& a, float4 B, int& c, int& cy, int& rx, int& ry) {
  // MathFunctions.C:61-81 (energy) and 106-127 (energy x cos, radial x axial velocity)
  const float v2xy = __fmaf_rn(B.y, B.y, __fmul_rn(B.x, B.x));
  const float v2 = __fmaf_rn(B.z, B.z, v2xy);
  const float e = __fmul_rn(v2, a.half_me_over_e);  // energy_of's rounding
  c = (int)(e * a.inv_e_step);
  cy = rx = ry = -1;
  if (a.cylindrical) {
    // cos and radial speed from the hardware reciprocal square root: a cell
    // edge moves by a few 1e-7 relative, far below the statistical resolution
    // of any cell (a zero speed has no angle and stays outside the cos cells)
    const float cosang = v2 > 0.0f ? B.z * rsqrtf(v2) : 2.0f;
    cy = (int)((cosang + 1.0f) * (0.5f * (float)a.n_cos));
    rx = (int)(radial_speed(v2xy) * a.inv_rad_step);
    ry = (int)((B.z + a.max_speed) * a.inv_ax_step);
  }
}

// Below this many electrons a chunk counts EADF and EVDF with global atomics:
// clearing and scanning the whole shared-memory grid would cost more.
constexpr int kHistSharedMin = 16384;

// pass A over electrons [first, last) of one condition
__device__ __forceinline__ void hist_chunk_a(const HistArgs& a, int first, int last, unsigned int* sm, int sm_words) {
  const int nE = a.n_e_cells;
  const int nA = a.cylindrical ? nE * a.n_cos : 0;
  const int nAw = (nA + 1) >> 1;
  const bool a_shared = a.cylindrical && last - first >= kHistSharedMin && nE + nAw <= sm_words;
  unsigned int* hE = sm;
  unsigned int* hA = sm + nE;
  const int zero_words = nE + (a_shared ? nAw : 0);
  for (int w = threadIdx.x; w < zero_words; w += blockDim.x) sm[w] = 0u;
  __syncthreads();
  // With the EADF in shared memory the EEDF count of a cell is its EADF row
  // sum, so only electrons outside the cos cells (cos rounding to 1, zero
  // speed) are counted into hE: one shared-memory atomic per electron.
  auto bin = [&](float4 B) {
    int c, cy, rx, ry;
    hist_cells(a, B, c, cy, rx, ry);
    if (c >= 0 && c < nE) {
      if (a.cylindrical && cy < a.n_cos && cy >= 0) {
        const int idx = c * a.n_cos + cy;
        if (a_shared) {
          atomicAdd(&hA[idx >> 1], 1u << ((idx & 1) << 4));
        } else {
          atomicAdd(&hE[c], 1u);
          atomicAdd(&a.eadf[idx], 1.0);
        }
      } else {
        atomicAdd(&hE[c], 1u);
      }
    }
  };
  // four electrons' loads in flight per thread before their counts; each
  // warp bulk-prefetches into L2 its 128 records of the block's pass two
  // rounds ahead
  const int st = blockDim.x;
  auto prefetch_round = [&](int base) {
    const int e0 = base + (int)(threadIdx.x >> 5) * 128;
    if ((threadIdx.x & 31) == 0 && e0 < last) prefetch_l2(a.state + 2 * e0, (uint32_t)min(128, last - e0) * 32u);
  };
  prefetch_round(first);
  prefetch_round(first + 4 * st);
  int i = first + threadIdx.x;
  for (; i + 3 * st < last; i += 4 * st) {
    prefetch_round(i - (int)threadIdx.x + 8 * st);
    const float4 B0 = a.state[2 * i + 1], B1 = a.state[2 * (i + st) + 1];
    const float4 B2 = a.state[2 * (i + 2 * st) + 1], B3 = a.state[2 * (i + 3 * st) + 1];
    bin(B0);
    bin(B1);
    bin(B2);
    bin(B3);
  }
  for (; i < last; i += st) bin(a.state[2 * i + 1]);
  __syncthreads();
  for (int c = threadIdx.x; c < nE; c += blockDim.x) {
    unsigned int h = hE[c];
    if (a_shared) {
      for (int k = 0; k < a.n_cos; ++k) {
        const int idx = c * a.n_cos + k;
        h += (hA[idx >> 1] >> ((idx & 1) << 4)) & 0xFFFFu;
      }
    }
    if (h) {
      atomicAdd(&a.eedf[c], (double)h);
      if (a.eedf_periodic_row) atomicAdd(&a.eedf_periodic_row[c], (double)h);
    }
  }
  if (a_shared) {
    for (int w = threadIdx.x; w < nAw; w += blockDim.x) {
      const unsigned int h = hA[w];
      if (h & 0xFFFFu) atomicAdd(&a.eadf[2 * w], (double)(h & 0xFFFFu));
      if ((h >> 16) && 2 * w + 1 < nA) atomicAdd(&a.eadf[2 * w + 1], (double)(h >> 16));
    }
  }
  __syncthreads();
}

// pass B over electrons [first, last) of one cylindrical condition
__device__ __forceinline__ void hist_chunk_b(const HistArgs& a, int first, int last, unsigned int* sm, int sm_words) {
  const int nV = a.n_rad * a.n_ax;
  const int nVw = (nV + 1) >> 1;
  const bool v_shared = last - first >= kHistSharedMin && nVw <= sm_words;
  if (v_shared)
    for (int w = threadIdx.x; w < nVw; w += blockDim.x) sm[w] = 0u;
  __syncthreads();
  for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
    int c, cy, rx, ry;
    hist_cells(a, a.state[2 * i + 1], c, cy, rx, ry);
    if (rx < a.n_rad && rx >= 0 && ry < a.n_ax && ry >= 0) {
      const int idx = rx * a.n_ax + ry;
      if (v_shared) atomicAdd(&sm[idx >> 1], 1u << ((idx & 1) << 4));
      else atomicAdd(&a.evdf[idx], 1.0);
    }
  }
  __syncthreads();
  if (v_shared) {
    for (int w = threadIdx.x; w < nVw; w += blockDim.x) {
      const unsigned int h = sm[w];
      if (h & 0xFFFFu) atomicAdd(&a.evdf[2 * w], (double)(h & 0xFFFFu));
      if ((h >> 16) && 2 * w + 1 < nV) atomicAdd(&a.evdf[2 * w + 1], (double)(h >> 16));
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kHistAThreads) k_hist_a(HistArgs a) {
  extern __shared__ unsigned int sm_hist[];
  const int chunks = (a.n + kHistChunk - 1) / kHistChunk;
  for (int c = blockIdx.x; c < chunks; c += gridDim.x)
    hist_chunk_a(a, c * kHistChunk, min(a.n, (c + 1) * kHistChunk), sm_hist, kHistASmem / 4);
}

__global__ void __launch_bounds__(kHistBThreads) k_hist_b(HistArgs a) {
  extern __shared__ unsigned int sm_hist[];
  const int chunks = (a.n + kHistChunk - 1) / kHistChunk;
  for (int c = blockIdx.x; c < chunks; c += gridDim.x)
    hist_chunk_b(a, c * kHistChunk, min(a.n, (c + 1) * kHistChunk), sm_hist, kHistBSmem / 4);
}

// ------------------------------------------------------- population control
__device__ __forceinline__ uint32_t pop_word(uint32_t idx, uint64_t interval, uint64_t seed, uint32_t salt,
                                             uint32_t draw) {
  Philox ph;
  ph.ctr = make_uint4(idx, (uint32_t)interval, (uint32_t)(interval >> 32) ^ (salt << 16), 0x80000000u | draw);
  ph.key = make_uint2((uint32_t)(seed ^ 0xA5A5A5A5u), (uint32_t)(seed >> 32));
  return ph.next().x;
}

// uniform integer in [0, n) from a 32-bit word (n < 2^31)
__device__ __forceinline__ int uniform_index(uint32_t w, int n) {
  return (int)(((unsigned long long)w * (unsigned long long)n) >> 32);
}

// adds a per-thread energy to the growth accumulator with one atomic per warp
__device__ __forceinline__ void add_growth(double* growth, double e) {
  cg::coalesced_group g = cg::coalesced_threads();
  const double tot = cg::reduce(g, e, cg::plus<double>());
  if (g.thread_rank() == 0) atomicAdd(growth, tot);
}

__device__ __forceinline__ float energy4(float4 B, float hme) { return energy_of(make_float3(B.x, B.y, B.z), hme); }

// Population control (BoltzmannMC.C:1282-1408), when all electrons and
// secondaries are at the synchronisation time. Five launches, each a grid of
// blocks over one or many slots (blockIdx.y) whose threads stride over the
// slot's items:
//  (0) the secondaries that did not attach are listed (alive);
//  (1) attached slots take secondaries, one per slot (:1344-1359); the slots
//      that stay attached are marked in the claim bitmap, so that no clone is
//      made from another clone;
//  (2) the slots still attached clone a random non-attached electron, whose
//      energy enters the growth term (:1360-1376); or, when secondaries are
//      left over, a uniformly random subset of size m is drawn from the pool of
//      N slots + m unplaced secondaries - the outcome of the reference's
//      sequential uniform removal (:1379-1407) - by claiming pool bits;
//  (3) clone marks are cleared; the removed ensemble slots and the unremoved
//      secondaries are listed, removed energies leave the growth term;
//  (4) the listed secondaries move into the removed slots; removal marks are
//      cleared, so the bitmap is zero again.
constexpr int kPopThreads = 256;
constexpr int kPopBlocks = 64;           // blocks, single condition
constexpr int kPopBlocksPerSM = 2;       // blocks per SM, batches

// one condition, arguments by value
struct PopOne {
  PopArgs a;
  __device__ int count() const { return 1; }
  __device__ const PopArgs* get(int s) const { return s == 0 ? &a : nullptr; }
};
// the slots of a batch that ionize or attach
struct PopBatch {
  const BatchHeader* hdr;
  const BatchSlot* slots;
  __device__ int count() const { return hdr->n_slots; }
  __device__ const PopArgs* get(int s) const {
    return (s < hdr->n_slots && (slots[s].flags & kSlotIonAtt)) ? &slots[s].pop : nullptr;
  }
};

__device__ __forceinline__ int pop_sec_total(const PopArgs& a) { return min(*a.sec_count, a.sec_cap); }
__device__ __forceinline__ bool claimed(const unsigned int* claim, int i) { return (claim[i >> 5] >> (i & 31)) & 1u; }

// Each phase is a list of items per slot (its length from the slot's counts
// as the previous phases left them). The grid works through all slots' items
// in 32-item warp chunks, so a warp's lanes always belong to one slot (the
// warp-aggregated appends and growth sums stay within it).
struct PopPlan {
  int pre[kBatchMaxSlots + 1];  // exclusive prefix of the slots' chunk counts
  int items[kBatchMaxSlots];
  int warp[kPopThreads / 32];
};

// exclusive block-wide prefix sum of v (every thread calls it); *total = the sum
__device__ __forceinline__ int block_exclusive_sum(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) s_warp[lane] = w;
  }
  __syncthreads();
  const int off = wid ? s_warp[wid - 1] : 0;
  *total = s_warp[nw - 1];
  __syncthreads();
  return off + x - v;
}

// the phase's item counts and chunk prefix in shared memory; returns the chunks
template <class Src, class Items>
__device__ __forceinline__ int pop_plan(const Src& src, int n, Items items, PopPlan& pl) {
  int carry = 0;
  for (int base = 0; base < n; base += blockDim.x) {
    const int s = base + threadIdx.x;
    int k = 0;
    if (s < n) {
      const PopArgs* ap = src.get(s);
      k = ap ? max(items(*ap), 0) : 0;
      pl.items[s] = k;
    }
    int tot = 0;
    const int ex = block_exclusive_sum((k + 31) >> 5, pl.warp, &tot);
    if (s < n) pl.pre[s] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) pl.pre[n] = carry;
  __syncthreads();
  return carry;
}

// body(a, i) for every item i of every slot
template <class Src, class Items, class Body>
__device__ __forceinline__ void pop_phase(const Src& src, Items items, Body body) {
  __shared__ PopPlan pl;
  const int n = src.count();
  const int total = pop_plan(src, n, items, pl);
  const int lane = threadIdx.x & 31;
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), GW = (int)((gridDim.x * blockDim.x) >> 5);
  for (int c = gw; c < total; c += GW) {
    int lo = 0, hi = n;  // largest s with pre[s] <= c
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (pl.pre[mid] <= c) lo = mid;
      else hi = mid;
    }
    const int i = ((c - pl.pre[lo]) << 5) + lane;
    if (i < pl.items[lo]) body(*src.get(lo), i);
  }
}

template <class Src>
__global__ void __launch_bounds__(kPopThreads) k_pop_list(Src src) {
  pop_phase(
      src, [](const PopArgs& a) { return pop_sec_total(a); },
      [](const PopArgs& a, int j) {
        if (a.sec[2 * j + 1].w == 0.0f) a.alive[append_slot(&a.counts[0])] = j;
      });
}

// items: every attached slot; the first min(n_att, n_sec) take secondaries,
// the rest are marked for clones
template <class Src>
__global__ void __launch_bounds__(kPopThreads) k_pop_fill(Src src) {
  pop_phase(
      src, [](const PopArgs& a) { return *a.att_count; },
      [](const PopArgs& a, int j) {
        const int n_att = *a.att_count, n_sec = a.counts[0];
        const int k = min(n_att, n_sec);
        if (j < k) {
          const int slot = a.att_list[j];
          const int sidx = a.alive[n_sec - 1 - j];
          a.state[2 * slot] = a.sec[2 * sidx];
          a.state[2 * slot + 1] = a.sec[2 * sidx + 1];
        } else {
          const int dest = a.att_list[j];
          atomicOr(&a.claim[dest >> 5], 1u << (dest & 31));
        }
      });
}

// items: the clones (n_att > n_sec) or the removal draws (n_sec > n_att)
template <class Src>
__global__ void __launch_bounds__(kPopThreads) k_pop_draw(Src src) {
  pop_phase(
      src, [](const PopArgs& a) { return abs(*a.att_count - a.counts[0]); },
      [](const PopArgs& a, int item) {
        const int n_att = *a.att_count, n_sec = a.counts[0];
        const uint64_t interval = a.ctl->interval;
        if (n_att > n_sec) {
          const int j = n_sec + item;
          const int dest = a.att_list[j];
          int src_slot = -1;
          for (uint32_t d = 0; d < 4096u; ++d) {
            const int r = uniform_index(pop_word((uint32_t)j, interval, a.seed, 1u, d), a.n_electrons);
            if (!claimed(a.claim, r) && a.state[2 * r + 1].w == 0.0f) {
              src_slot = r;
              break;
            }
          }
          if (src_slot < 0) {
            atomicExch(a.error_flag, 4);
            return;
          }
          const float4 A = a.state[2 * src_slot], B = a.state[2 * src_slot + 1];
          a.state[2 * dest] = A;
          a.state[2 * dest + 1] = B;
          add_growth(a.growth, (double)energy4(B, a.half_me_over_e));
        } else {
          const int j = item;
          const int pool = a.n_electrons + (n_sec - n_att);
          int got = -1;
          for (uint32_t d = 0; d < 4096u; ++d) {
            const int r = uniform_index(pop_word((uint32_t)j, interval, a.seed, 2u, d), pool);
            const unsigned int bit = 1u << (r & 31);
            const unsigned int old = atomicOr(&a.claim[r >> 5], bit);
            if (!(old & bit)) {
              got = r;
              break;
            }
          }
          a.removed[j] = got;
          if (got < 0) atomicExch(a.error_flag, 5);
        }
      });
}

// items: the clone marks to clear (n_att > n_sec) or the removal outcomes to
// list (n_sec > n_att)
template <class Src>
__global__ void __launch_bounds__(kPopThreads) k_pop_sort(Src src) {
  pop_phase(
      src, [](const PopArgs& a) { return abs(*a.att_count - a.counts[0]); },
      [](const PopArgs& a, int item) {
        const int n_att = *a.att_count, n_sec = a.counts[0];
        if (n_att > n_sec) {
          const int dest = a.att_list[n_sec + item];
          atomicAnd(&a.claim[dest >> 5], ~(1u << (dest & 31)));
          return;
        }
        const int j = item;
        const int r = a.removed[j];
        if (r >= 0 && r < a.n_electrons) {
          a.pair_slot[append_slot(&a.counts[1])] = r;
          add_growth(a.growth, -(double)energy4(a.state[2 * r + 1], a.half_me_over_e));
        } else if (r >= a.n_electrons) {
          add_growth(a.growth, -(double)energy4(a.sec[2 * a.alive[r - a.n_electrons] + 1], a.half_me_over_e));
        }
        if (!claimed(a.claim, a.n_electrons + j)) a.pair_sec[append_slot(&a.counts[2])] = a.alive[j];
      });
}

// items: the (removed slot, surviving secondary) pairs, then the removal
// marks to clear
template <class Src>
__global__ void __launch_bounds__(kPopThreads) k_pop_place(Src src) {
  pop_phase(
      src,
      [](const PopArgs& a) {
        return min(a.counts[1], a.counts[2]) + max(a.counts[0] - *a.att_count, 0);
      },
      [](const PopArgs& a, int item) {
        const int np = min(a.counts[1], a.counts[2]);
        if (item < np) {
          const int slot = a.pair_slot[item];
          const int sidx = a.pair_sec[item];
          a.state[2 * slot] = a.sec[2 * sidx];
          a.state[2 * slot + 1] = a.sec[2 * sidx + 1];
        } else {
          const int r = a.removed[item - np];
          if (r >= 0) atomicAnd(&a.claim[r >> 5], ~(1u << (r & 31)));
        }
      });
}

template <class Src>
void launch_pop_phases(const Src& src, int grid, cudaStream_t s) {
  k_pop_list<<<grid, kPopThreads, 0, s>>>(src);
  k_pop_fill<<<grid, kPopThreads, 0, s>>>(src);
  k_pop_draw<<<grid, kPopThreads, 0, s>>>(src);
  k_pop_sort<<<grid, kPopThreads, 0, s>>>(src);
  k_pop_place<<<grid, kPopThreads, 0, s>>>(src);
}

// ---------------------------------------------------------- batch helpers
// Before the advance: each slot's interval values to its control block, the
// per-interval scalars cleared (and the moment sums of sampling slots), the
// advance counter reset. One warp per slot.
__global__ void k_batch_prep(BatchArgs b) {
  const int n = b.hdr->n_slots;
  const int lane = threadIdx.x & 31;
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= n) return;
  const BatchSlot& sl = b.slots[s];
  DevScalars* sc = sl.sc;
  if (lane == 0) {
    *sl.ctl_dst = sl.ctl;
    sc->sec_count = 0;
    sc->att_count = 0;
    sc->spill_count = 0;
    sc->error_flag = 0;
    sc->max_energy_bits = 0u;
    sc->work_counter = 0;
    sc->pop_counts[0] = sc->pop_counts[1] = sc->pop_counts[2] = 0;
  }
  if (sl.flags & kSlotSample) {
    if (lane < kMoments) sc->moments[lane] = 0.0;
    if (lane == 0) sc->sample_max_bits = 0u;
  }
}

// distribution tallies of the slots that sample them this interval
// the chunk this block takes in round r (snake order, lgpu_chunks.h)
__device__ __forceinline__ int snake_chunk(int r) { return snake_index(r, gridDim.x, blockIdx.x); }

__global__ void __launch_bounds__(kHistAThreads) k_hist_a_batch(BatchArgs b) {
  extern __shared__ unsigned int sm_hist[];
  const int n_slots = b.hdr->n_slots, total = b.hdr->hist_chunks, n_full = b.hdr->hist_full;
  for (int r = 0; r * (int)gridDim.x < total; ++r) {
    const int c = snake_chunk(r);
    if (c >= total) continue;
    const ChunkRef k = pass_chunk(b.hist_prefix, b.hist_part, n_slots, n_full, kHistChunk, c);
    const HistArgs& a = b.slots[k.slot].hist;
    hist_chunk_a(a, k.first, min(k.first + kHistChunk, a.n), sm_hist, kHistASmem / 4);
  }
}

__global__ void __launch_bounds__(kHistBThreads) k_hist_b_batch(BatchArgs b) {
  extern __shared__ unsigned int sm_hist[];
  const int n_slots = b.hdr->n_slots, total = b.hdr->hist2_chunks, n_full = b.hdr->hist2_full;
  for (int r = 0; r * (int)gridDim.x < total; ++r) {
    const int c = snake_chunk(r);
    if (c >= total) continue;
    const ChunkRef k = pass_chunk(b.hist2_prefix, b.hist2_part, n_slots, n_full, kHistChunk, c);
    const HistArgs& a = b.slots[k.slot].hist;
    hist_chunk_b(a, k.first, min(k.first + kHistChunk, a.n), sm_hist, kHistBSmem / 4);
  }
}

// Ensemble moments of the sampling slots; for the slots whose sample records
// distributions (kSlotEvdf) the same pass counts the EVDF (BoltzmannMC.C:
// 1550-1571; 16-bit counts in shared memory per chunk, global atomics for
// small chunks), saving its separate pass over the velocities.
constexpr int kSampleBatchThreads = 512;
constexpr int kSampleBatchSmem = 80 * 1024;  // EVDF counts, two blocks per SM

__global__ void __launch_bounds__(kSampleBatchThreads, 2) k_sample_batch(BatchArgs b) {
  __shared__ double s_m[kSampleBatchThreads / 32][kMoments];
  extern __shared__ unsigned int sm_evdf[];
  const int n_slots = b.hdr->n_slots, total = b.hdr->smp_chunks, n_full = b.hdr->smp_full;
  for (int r = 0; r * (int)gridDim.x < total; ++r) {
    const int c = snake_chunk(r);
    if (c >= total) continue;
    const ChunkRef k = pass_chunk(b.smp_prefix, b.smp_part, n_slots, n_full, kBatchSampleChunk, c);
    const BatchSlot& sl = b.slots[k.slot];
    const SampleArgs& a = sl.smp;
    const int first = k.first;
    const int last = min(first + kBatchSampleChunk, a.n);
    const bool evdf = (sl.flags & kSlotEvdf) != 0;
    const HistArgs& h = sl.vhist;
    const int nV = evdf ? h.n_rad * h.n_ax : 0;
    const int nVw = (nV + 1) >> 1;
    const bool v_shared = evdf && last - first >= kHistSharedMin && nVw <= kSampleBatchSmem / 4;
    if (v_shared)
      for (int w = threadIdx.x; w < nVw; w += blockDim.x) sm_evdf[w] = 0u;
    __syncthreads();
    if (evdf) {
      auto bin = [&](float4 B) {
        const float v2xy = __fmaf_rn(B.y, B.y, __fmul_rn(B.x, B.x));
        const int rx = (int)(radial_speed(v2xy) * h.inv_rad_step);
        const int ry = (int)((B.z + h.max_speed) * h.inv_ax_step);
        if (rx < h.n_rad && rx >= 0 && ry < h.n_ax && ry >= 0) {
          const int idx = rx * h.n_ax + ry;
          if (v_shared) atomicAdd(&sm_evdf[idx >> 1], 1u << ((idx & 1) << 4));
          else atomicAdd(&h.evdf[idx], 1.0);
        }
      };
      sample_range(a, first + threadIdx.x, last, blockDim.x, s_m, bin);
    } else {
      sample_range(a, first + threadIdx.x, last, blockDim.x, s_m);
    }
    __syncthreads();
    if (v_shared) {
      for (int w = threadIdx.x; w < nVw; w += blockDim.x) {
        const unsigned int v = sm_evdf[w];
        if (v & 0xFFFFu) atomicAdd(&h.evdf[2 * w], (double)(v & 0xFFFFu));
        if ((v >> 16) && 2 * w + 1 < nV) atomicAdd(&h.evdf[2 * w + 1], (double)(v >> 16));
      }
      __syncthreads();
    }
  }
}

// every slot's scalars into one contiguous array for a single read-back
__global__ void k_batch_gather(BatchArgs b) {
  const int n = b.hdr->n_slots;
  constexpr int kWords = (int)(sizeof(DevScalars) / sizeof(int));
  for (int s = blockIdx.x; s < n; s += gridDim.x) {
    const int* src = reinterpret_cast<const int*>(b.slots[s].sc);
    int* dst = reinterpret_cast<int*>(&b.gather[s]);
    for (int k = threadIdx.x; k < kWords; k += blockDim.x) dst[k] = src[k];
  }
}

// --------------------------------------------------------------- replay
__global__ void k_replay_flight(ReplayFlightArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  float3 p = make_float3((float)a.pos[3 * i], (float)a.pos[3 * i + 1], (float)a.pos[3 * i + 2]);
  float3 v = make_float3((float)a.vel[3 * i], (float)a.vel[3 * i + 1], (float)a.vel[3 * i + 2]);
  const float e0 = energy_of(v, a.half_me_over_e);
  free_flight(a.field, (float)a.phi0[i], (float)a.dt[i], p, v);
  const float e1 = energy_of(v, a.half_me_over_e);
  a.pos_out[3 * i] = p.x;
  a.pos_out[3 * i + 1] = p.y;
  a.pos_out[3 * i + 2] = p.z;
  a.vel_out[3 * i] = v.x;
  a.vel_out[3 * i + 1] = v.y;
  a.vel_out[3 * i + 2] = v.z;
  a.energy_out[i] = e1;
  a.gain_out[i] = e1 - e0;
}

__global__ void k_replay_collide(ReplayCollArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  ReplayStream rng;
  rng.u = a.u + (size_t)i * a.u_stride;
  rng.n = a.u_stride;
  rng.pos = 0;
  float3 v = make_float3((float)a.vel[3 * i], (float)a.vel[3 * i + 1], (float)a.vel[3 * i + 2]);
  float energy = (float)a.energy[i];
  CollResult cr;
  cr.ej_v = make_float3(0.f, 0.f, 0.f);
  if (a.coarse) {
    // the advance kernels' event: the null test tries the block bound of the
    // total frequency first (lane_flight), then the rest of the collision
    // (lane_real)
    float r = 0.0f;
    const float nu = (float)a.nu[i];
    if (is_thermal(a.c, energy) || cold_real(a.t, nu, energy, rng, r, a.t.nu_coarse)) {
      collide_pending(a.c, a.t, a.procs, a.gases, nu, r, v, energy, rng, cr);
    } else {
      cr.chosen = -1;
      cr.dE = 0.0f;
      cr.ionized = 0;
    }
  } else {
    collide(a.c, a.t, a.procs, a.gases, (float)a.nu[i], v, energy, rng, cr);
  }
  double* o = a.out + (size_t)i * 11;
  o[0] = cr.chosen;
  o[1] = v.x;
  o[2] = v.y;
  o[3] = v.z;
  o[4] = energy;
  o[5] = cr.chosen >= 0 ? cr.dE : 0.0;
  o[6] = cr.chosen >= 0 ? (double)cr.dE / a.energy[i] : 0.0;
  const bool ion = cr.chosen >= 0 && cr.ionized;
  o[7] = ion ? cr.ej_v.x : 0.0;
  o[8] = ion ? cr.ej_v.y : 0.0;
  o[9] = ion ? cr.ej_v.z : 0.0;
  o[10] = ion ? (double)energy_of(cr.ej_v, a.c.half_me_over_e) : 0.0;
  a.used[i] = rng.pos;
}

inline int blocks_for(int n, int threads) { return (n + threads - 1) / threads; }

}  // namespace

void launch_advance(const AdvanceArgs& a, cudaStream_t s) {
#define LGPU_ADVANCE(K, G, B)                                  \
  switch (a.field.mode) {                                      \
    case kFieldDC: K<kFieldDC><<<G, B, 0, s>>>(a); break;      \
    case kFieldAC: K<kFieldAC><<<G, B, 0, s>>>(a); break;      \
    case kFieldB: K<kFieldB><<<G, B, 0, s>>>(a); break;        \
    case kFieldECR: K<kFieldECR><<<G, B, 0, s>>>(a); break;    \
    default: K<kFieldACB><<<G, B, 0, s>>>(a); break;           \
  }
  if (a.queue_only) {
    LGPU_ADVANCE(k_advance_drain, 1, 32)
  } else {
    // persistent grid: at most kAdvanceBlocksPerSM blocks per SM, fewer when
    // the electrons do not fill them (one chunk per warp)
    const int warps_needed = (a.n + AdvShape<0>::kChunk - 1) / AdvShape<0>::kChunk;
    const int grid = max(1, min(a.sm_count * kAdvanceBlocksPerSM, (warps_needed + 7) / 8));
    LGPU_ADVANCE(k_advance, grid, kAdvanceThreads)
  }
#undef LGPU_ADVANCE
}

void launch_init(const InitArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  k_init<<<blocks_for(a.n, 256), 256, 0, s>>>(a);
}

void launch_build_tables(const TableBuildArgs& a, cudaStream_t s) {
  k_build_tables<<<blocks_for(a.M, kTableWarps), 32 * kTableWarps, 0, s>>>(a);
  k_prefix_max<<<1, kPrefixThreads, 0, s>>>(a.nu_tot, a.nu_max, a.M);
  if (a.nu_coarse) k_coarse_max<<<1, kMaxCoarse, 0, s>>>(a.nu_pair, a.M, a.coarse_shift, a.nu_coarse, a.n_coarse);
}

void launch_sample(const SampleArgs& a, int sm_count, cudaStream_t s) {
  if (a.n <= 0) return;
  const int grid = min(blocks_for(a.n, kSampleThreads), max(1, sm_count) * 4);
  k_sample<<<grid, kSampleThreads, 0, s>>>(a);
}

void launch_hist(const HistArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  const int chunks = (a.n + kHistChunk - 1) / kHistChunk;
  k_hist_a<<<chunks, kHistAThreads, kHistASmem, s>>>(a);
  if (a.cylindrical && !a.evdf_done) k_hist_b<<<chunks, kHistBThreads, kHistBSmem, s>>>(a);
}

void launch_pop_control(const PopArgs& a, cudaStream_t s) {
  PopOne one;
  one.a = a;
  launch_pop_phases(one, kPopBlocks, s);
}

cudaError_t prepare_kernels() {
  cudaError_t e = cudaFuncSetAttribute(k_hist_a, cudaFuncAttributeMaxDynamicSharedMemorySize, kHistASmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hist_b, cudaFuncAttributeMaxDynamicSharedMemorySize, kHistBSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_hist_a_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, kHistASmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_hist_b_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, kHistBSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sample_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, kSampleBatchSmem);
  if (e == cudaSuccess) e = prepare_advance_stash();
  return e;
}

size_t batch_prefix_offset() { return (sizeof(BatchHeader) + 15) / 16 * 16; }
size_t batch_slots_offset() {
  return (batch_prefix_offset() + (4 * (kBatchMaxSlots + 1) + 3 * kBatchMaxSlots) * sizeof(int) + 255) / 256 * 256;
}

int launch_batch_pre(const BatchArgs& b, int sm_count, int max_slots, unsigned parts, cudaStream_t s) {
  const int slots = max(1, min(max_slots, kBatchMaxSlots));
  k_batch_prep<<<(slots + 7) / 8, 256, 0, s>>>(b);
  return 1;
}

int launch_batch_hist(const BatchArgs& b, int sm_count, unsigned parts, cudaStream_t s) {
  int n = 0;
  if (parts & kPartHistA) {
    k_hist_a_batch<<<sm_count, kHistAThreads, kHistASmem, s>>>(b);
    ++n;
  }
  if (parts & kPartHistB) {
    k_hist_b_batch<<<sm_count * 2, kHistBThreads, kHistBSmem, s>>>(b);
    ++n;
  }
  return n;
}

int launch_batch_post(const BatchArgs& b, int sm_count, int max_slots, unsigned parts, cudaStream_t s) {
  const int slots = max(1, min(max_slots, kBatchMaxSlots));
  int n = 1;
  if (parts & kPartIonAtt) {
    k_advance_drain_batch<<<slots, 32, 0, s>>>(b);
    PopBatch pb;
    pb.hdr = b.hdr;
    pb.slots = b.slots;
    launch_pop_phases(pb, sm_count * kPopBlocksPerSM, s);
    n += 1 + kPopLaunches;
  }
  if (parts & kPartSample) {
    k_sample_batch<<<sm_count * 2, kSampleBatchThreads, kSampleBatchSmem, s>>>(b);
    ++n;
  }
  k_batch_gather<<<min(slots, 64), 64, 0, s>>>(b);
  return n;
}

void launch_replay_flight(const ReplayFlightArgs& a, cudaStream_t s) {
  if (a.n > 0) k_replay_flight<<<blocks_for(a.n, 128), 128, 0, s>>>(a);
}

void launch_replay_collide(const ReplayCollArgs& a, cudaStream_t s) {
  if (a.n > 0) k_replay_collide<<<blocks_for(a.n, 128), 128, 0, s>>>(a);
}

}  // namespace lgpu
