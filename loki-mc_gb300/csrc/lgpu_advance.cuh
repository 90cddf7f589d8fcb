// lgpu_advance.cuh - device code of the advance: free flights and collisions
// of every electron up to the synchronisation time (BoltzmannMC.C:617-688,
// 804-1280). Included by the translation units that instantiate its kernels:
// lgpu_kernels.cu (one condition per launch, drains) and
// lgpu_advance_batch.cu / lgpu_advance_stash.cu (the batched advance in its
// launch shapes), which compile in parallel.
#pragma once

#include <cooperative_groups.h>

#include "lgpu_device.cuh"
#include "lgpu_kernels.cuh"

namespace cg = cooperative_groups;

namespace lgpu {

namespace {

__device__ __forceinline__ void atomic_max_energy(unsigned int* bits, float e) {
  // energies are >= 0, so the IEEE bit pattern orders like the value
  atomicMax(bits, __float_as_uint(fmaxf(e, 0.0f)));
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp-aggregated append: one atomic per warp for the lanes that call it.
__device__ __forceinline__ int append_slot(int* counter) {
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, (int)g.size());
  base = g.shfl(base, 0);
  return base + (int)g.thread_rank();
}

// Launch shapes of the advance: threads per block, blocks per SM (which fix
// the register budget: 65536 / (threads x blocks)), the electrons a warp
// takes from the work counter at a time (its chunk: chunk/32 electrons per
// lane) and the records of a warp's collision stash (0: none, the warp waits
// for its collision turn with the pending electrons in their lanes; see
// warp_loop_stash). The single-condition kernels use shape 0; the batched
// kernel is built in every shape and the batch's tuner picks one per mixture.
template <int S>
struct AdvShape;
template <>
struct AdvShape<0> { static constexpr int kThreads = 256, kBlocksPerSM = 4, kChunk = 128, kStash = 0; };
template <>
struct AdvShape<1> { static constexpr int kThreads = 512, kBlocksPerSM = 2, kChunk = 128, kStash = 0; };
template <>
struct AdvShape<2> { static constexpr int kThreads = 256, kBlocksPerSM = 4, kChunk = 64, kStash = 0; };
template <>
struct AdvShape<3> { static constexpr int kThreads = 256, kBlocksPerSM = 4, kChunk = 256, kStash = 0; };
template <>
struct AdvShape<4> { static constexpr int kThreads = 256, kBlocksPerSM = 4, kChunk = 128, kStash = 64; };
template <>
struct AdvShape<5> { static constexpr int kThreads = 512, kBlocksPerSM = 2, kChunk = 128, kStash = 64; };
static_assert(kAdvShapes == 6, "one AdvShape per tuner candidate");
static_assert(AdvShape<kFirstStashShape>::kStash > 0 && AdvShape<kFirstStashShape - 1>::kStash == 0,
              "stash shapes come last");

// dynamic shared memory of a shape's stashes (bytes per block)
template <int S>
constexpr int adv_stash_bytes() {
  return AdvShape<S>::kThreads / 32 * AdvShape<S>::kStash * 4 * (int)sizeof(float4);
}

constexpr int kAdvanceThreads = AdvShape<0>::kThreads;
constexpr int kAdvanceBlocksPerSM = AdvShape<0>::kBlocksPerSM;
constexpr int kAdvanceWarps = kAdvanceThreads / 32;

// ---------------------------------------------------------------- advance
// Every electron is flown and collided until the synchronisation time
// (BoltzmannMC.C:617-688). Work distribution: a persistent grid; each warp
// takes chunks of electrons from a global counter and every lane holds one
// electron. A lane whose electron reaches the synchronisation time (or is
// attached) writes it back and takes the next electron of the warp's chunk,
// so the lanes of a warp stay busy although the number of collisions per
// electron and interval is random. A secondary created by a lane goes on its
// warp's own queue (shared memory) and an idle lane of the same warp pushes it
// from its creation time to the end of the interval: the creating lane keeps
// the warp alive, so no warp ever waits on another. A warp whose queue is full
// spills to a global buffer that the one-warp drain launch works off after.
constexpr int kLocalQ = 32;

// Shared memory of an advance block: constants and per-process tallies of the
// block's current condition, the warps' secondary queues, reduction scratch.
// Stash shapes read the process constants from global memory (they are read
// once per real collision) to leave room for the stashes.
template <int WARPS, int CHUNK, int STASH = 0>
struct AdvSharedT {
  static constexpr int kWarps = WARPS, kChunk = CHUNK, kStash = STASH;
  static constexpr bool kProcsInShared = STASH == 0;
  float nu_coarse[kMaxCoarse];  // block bounds of the total frequency of the current condition
  unsigned int count[kMaxProcesses];
  // energy changes per process and sign: the count of collisions that lost
  // energy, and the FP32 sums of dE - off, off the process's nominal change
  // (-threshold; 0 for attachment). The flush adds the nominal part back as
  // count x off in FP64, so FP32 only sums the small remainders (the recoil
  // of inelastic collisions): a block adds thousands of nearly equal
  // inelastic losses per process and interval, whose plain FP32 sum would
  // round by up to ~1e-4 relative
  unsigned int neg[kMaxProcesses];
  float gain[kMaxProcesses];
  float loss[kMaxProcesses];
  ProcF proc[kProcsInShared ? kMaxProcesses : 1];
  GasF gas[kMaxGases];
  float4 qa[WARPS][kLocalQ];  // (x, y, z, t_c)
  float4 qb[WARPS][kLocalQ];  // (vx, vy, vz, 0)
  int qn[WARPS];
  double red[WARPS];
  double redt[WARPS];
  unsigned long long redn[WARPS];
  unsigned long long redr[WARPS];
};
using AdvShared = AdvSharedT<kAdvanceWarps, AdvShape<0>::kChunk>;


// The values of one interval: launch arguments, overridden by the control block.
struct IntervalView {
  FieldF field;
  TablesF tab;
  float T, nu, inv_nu, phi0, phase_rate;
  float3 shift;
  uint64_t interval;
};

// MODE >= 0 fixes the field branch at compile time; -1 keeps the argument's
template <int MODE>
__device__ __forceinline__ IntervalView interval_view(const AdvanceArgs& a) {
  IntervalView iv;
  iv.field = a.field;
  if (MODE >= 0) iv.field.mode = MODE;
  iv.tab = a.t;
  iv.T = a.dt_sync;
  iv.nu = a.nu;
  iv.phi0 = a.phi0;
  iv.phase_rate = a.phase_rate;
  iv.shift = a.shift;
  iv.interval = a.interval;
  if (a.ctl) {
    const IntervalCtl c = *a.ctl;
    iv.T = c.dt_sync;
    iv.nu = c.nu;
    iv.phi0 = c.phi0;
    iv.phase_rate = c.phase_rate;
    iv.shift = make_float3(c.shift_x, c.shift_y, c.shift_z);
    iv.interval = c.interval;
    iv.tab.inv_step = c.inv_step;
  }
  iv.inv_nu = 1.0f / iv.nu;
  return iv;
}

// The electron a lane holds.
struct Lane {
  bool have;
  bool pending;  // a real collision waits for the warp's next collision turn
  int slot;      // ensemble slot, -1 for a secondary
  float3 p, v;
  float s, t, energy;
  float r;       // the pending collision's null-test draw (cold gas)
  int events;
  PcgStream rng;
};

// Per-lane sums of one condition, reduced when the block flushes.
struct LaneTally {
  float gain, time_adj, e_max;
  unsigned int null_n, real_n;
};

__device__ __forceinline__ void reset_lane(Lane& L) {
  L.have = false;
  L.pending = false;
  L.r = 0.0f;
  L.slot = 0;
  L.p = make_float3(0.f, 0.f, 0.f);
  L.v = make_float3(0.f, 0.f, 0.f);
  L.s = -1.0f;
  L.t = 0.0f;
  L.energy = 0.0f;
  L.events = 0;
}

__device__ __forceinline__ void reset_tally(LaneTally& tl) {
  tl.gain = 0.0f;
  tl.time_adj = 0.0f;
  tl.e_max = 0.0f;
  tl.null_n = 0u;
  tl.real_n = 0u;
}

// process constants to shared memory, tallies and queues cleared
template <class Sh>
__device__ __forceinline__ void load_block_consts(const AdvanceArgs& a, Sh& sh) {
  for (int q = threadIdx.x; q < a.P; q += blockDim.x) {
    sh.count[q] = 0u;
    sh.neg[q] = 0u;
    sh.gain[q] = 0.0f;
    sh.loss[q] = 0.0f;
    if constexpr (Sh::kProcsInShared) sh.proc[q] = a.procs[q];
  }
  if (threadIdx.x < a.c.G) sh.gas[threadIdx.x] = a.gases[threadIdx.x];
  if (threadIdx.x < Sh::kWarps) sh.qn[threadIdx.x] = 0;
  if (a.t.nu_coarse)
    for (int b = threadIdx.x; b < a.t.n_coarse; b += blockDim.x) sh.nu_coarse[b] = a.t.nu_coarse[b];
}

// an ensemble electron (left alone when its slot is attached)
__device__ __forceinline__ void lane_take_electron(const AdvanceArgs& a, const IntervalView& iv, Lane& L, int idx) {
  float4 A, B;
  load_record(a.state + 2 * idx, A, B);
  // the stream's seeding needs no state: it runs while the loads are in flight
  L.rng.init((uint32_t)idx, iv.interval, a.seed, a.salt);
  if (B.w == 0.0f) {
    L.slot = idx;
    L.p = make_float3(A.x - iv.shift.x, A.y - iv.shift.y, A.z - iv.shift.z);
    L.v = make_float3(B.x, B.y, B.z);
    L.s = A.w;  // remaining flight in units of 1/nu (exponential variate), <0: draw
    L.t = 0.0f;
    L.energy = energy_of(L.v, a.c.half_me_over_e);
    L.events = 0;
    L.pending = false;
    L.have = true;
  }
}

// a secondary, pushed from its creation time t_c = A.w. Its random stream is
// named by the warp that takes it (`warp_tag`) and that warp's running count of
// secondaries (`id`), with a salt apart from the ensemble electrons' streams.
__device__ __forceinline__ void lane_take_secondary(const AdvanceArgs& a, const IntervalView& iv, Lane& L,
                                                    LaneTally& tl, float4 A, float4 B, uint32_t warp_tag,
                                                    uint32_t id) {
  L.slot = -1;
  L.p = make_float3(A.x, A.y, A.z);  // created from shifted positions already
  L.v = make_float3(B.x, B.y, B.z);
  L.s = -1.0f;
  L.t = A.w;
  tl.time_adj += iv.T - L.t;  // electron-time this secondary adds to the interval
  L.rng.init(id, iv.interval, a.seed, a.salt + 1u, warp_tag);
  L.energy = energy_of(L.v, a.c.half_me_over_e);
  L.events = 0;
  L.pending = false;
  L.have = true;
}

// idle lanes take secondaries from their warp's queue (newest first);
// returns the entries left
template <class Sh>
__device__ __forceinline__ int lane_take_queued(const AdvanceArgs& a, const IntervalView& iv, Sh& sh, int wid,
                                                int lane, unsigned lt_mask, Lane& L, LaneTally& tl, uint32_t& sec_id,
                                                uint32_t warp_tag) {
  int qn = min(sh.qn[wid], a.local_q);
  const unsigned idle = __ballot_sync(0xffffffffu, !L.have);
  const int r = __popc(idle & lt_mask);
  const int take = min(__popc(idle), qn);
  if (((idle >> lane) & 1u) && r < take) {
    const int e = qn - 1 - r;
    lane_take_secondary(a, iv, L, tl, sh.qa[wid][e], sh.qb[wid][e], warp_tag, sec_id + (uint32_t)r);
  }
  // 2^32 secondaries taken by one warp in one interval would repeat streams
  if (sec_id + (uint32_t)take < sec_id && lane == 0) atomicExch(a.error_flag, 3);
  sec_id += (uint32_t)take;
  qn -= take;
  __syncwarp();
  if (lane == 0) sh.qn[wid] = qn;
  return qn;
}

// A finished electron: an ensemble electron goes back to its slot (attached
// ones flagged), a secondary to the list of secondaries at the
// synchronisation time.
__device__ __forceinline__ void lane_finish(const AdvanceArgs& a, Lane& L, LaneTally& tl, bool dead) {
  if (L.slot >= 0) {
    store_record(a.state + 2 * L.slot, make_float4(L.p.x, L.p.y, L.p.z, dead ? -1.0f : L.s),
                 make_float4(L.v.x, L.v.y, L.v.z, dead ? 1.0f : 0.0f));
  } else if (!dead) {
    const int k = append_slot(a.sec_count);
    if (k < a.sec_cap) {
      a.sec[2 * k] = make_float4(L.p.x, L.p.y, L.p.z, L.s);
      a.sec[2 * k + 1] = make_float4(L.v.x, L.v.y, L.v.z, 0.0f);
    } else {
      atomicExch(a.error_flag, 2);
    }
  }
  if (!dead) tl.e_max = fmaxf(tl.e_max, L.energy);
  L.have = false;
}

// The flight turn of a lane's electron: a free flight to the next collision
// or, when that lies beyond the synchronisation time, to the synchronisation
// time (BoltzmannMC.C:650-675; the flight code is the same for both so the
// lanes stay converged), then the null test of a cold gas. A real collision
// (or any thermal-target event) is left pending for the collision turn, which
// the warp takes once enough of its lanes have one: the long collision code
// then runs on most of the warp's lanes instead of a few. Each electron draws
// its random numbers in the same order either way.
template <int MODE, class Sh>
__device__ __forceinline__ void lane_flight(const AdvanceArgs& a, const Sh& sh, const IntervalView& iv, Lane& L,
                                            LaneTally& tl) {
  if (L.s < 0.0f) L.s = -__logf(L.rng.oo());
  const float tau = L.s * iv.inv_nu;
  const bool partial = L.t + tau > iv.T;
  const float dt = partial ? iv.T - L.t : tau;
  free_flight<MODE>(iv.field, __fmaf_rn(iv.phase_rate, L.t, iv.phi0), dt, L.p, L.v);
  {
    const float e1 = energy_of(L.v, a.c.half_me_over_e);
    tl.gain += e1 - L.energy;
    L.energy = e1;
  }
  if (partial) {
    L.s = fmaxf(__fmaf_rn(-iv.nu, dt, L.s), 0.0f);
    lane_finish(a, L, tl, false);
    return;
  }
  L.t += tau;
  if (is_thermal(a.c, L.energy) ||
      cold_real(iv.tab, iv.nu, L.energy, L.rng, L.r, (a.coarse && iv.tab.nu_coarse) ? sh.nu_coarse : nullptr)) {
    L.pending = true;
    return;
  }
  ++tl.null_n;
  L.s = -__logf(L.rng.oo());  // next free flight (BoltzmannMC.C:670)
  if (++L.events >= (1 << 20)) {
    atomicExch(a.error_flag, 3);  // collision budget of one interval exhausted
    lane_finish(a, L, tl, false);
  }
}

// the process constants of the block's condition
template <class Sh>
__device__ __forceinline__ const ProcF* procs_of(const AdvanceArgs& a, const Sh& sh) {
  if constexpr (Sh::kProcsInShared) return sh.proc;
  else return a.procs;
}

// A process's nominal energy change per collision (eV): minus its threshold
// (the gain of a superelastic process), none for attachment, whose loss is
// the electron's whole energy.
__device__ __forceinline__ float nominal_change(const ProcF& p) { return p.type == kAttachment ? 0.0f : -p.eloss; }

// The collision turn: process choice, kinematics, tallies, secondaries and
// attachment (BoltzmannMC.C:907-1280).
template <class Sh>
__device__ __forceinline__ void lane_real(const AdvanceArgs& a, Sh& sh, int wid, const IntervalView& iv,
                                          Lane& L, LaneTally& tl) {
  L.pending = false;
  CollResult cr;
  const ProcF* procs = procs_of(a, sh);
  collide_pending(a.c, iv.tab, procs, sh.gas, iv.nu, L.r, L.v, L.energy, L.rng, cr);
  bool finished = false, dead = false;
  if (cr.chosen < 0) {
    ++tl.null_n;
  } else {
    ++tl.real_n;
    atomicAdd(&sh.count[cr.chosen], 1u);
    const int ptype = procs[cr.chosen].type;
    const float rest = cr.dE - nominal_change(procs[cr.chosen]);
    if (cr.dE >= 0.0f) {
      if (rest != 0.0f) atomicAdd(&sh.gain[cr.chosen], rest);
    } else {
      atomicAdd(&sh.neg[cr.chosen], 1u);
      if (rest != 0.0f) atomicAdd(&sh.loss[cr.chosen], rest);
    }
    if (ptype == kIonization) {
      const float4 A = make_float4(L.p.x, L.p.y, L.p.z, L.t);
      const float4 B = make_float4(cr.ej_v.x, cr.ej_v.y, cr.ej_v.z, 0.0f);
      const int k = atomicAdd(&sh.qn[wid], 1);
      if (k < a.local_q) {
        sh.qa[wid][k] = A;
        sh.qb[wid][k] = B;
      } else {
        const int g = append_slot(a.spill_count);
        if (g < a.spill_cap) {
          a.spill[2 * g] = A;
          a.spill[2 * g + 1] = B;
        } else {
          atomicExch(a.error_flag, 2);  // spill buffer full: the host reports it
        }
      }
    } else if (ptype == kAttachment) {
      dead = true;
      finished = true;
      tl.time_adj -= iv.T - L.t;  // electron-time the attached electron no longer spends
      if (L.slot >= 0) {
        const int k = append_slot(a.att_count);
        a.att_list[k] = L.slot;
      }
    }
  }
  L.s = -__logf(L.rng.oo());  // next free flight (BoltzmannMC.C:670)
  if (++L.events >= (1 << 20) && !finished) {
    atomicExch(a.error_flag, 3);  // collision budget of one interval exhausted
    finished = true;
  }
  if (finished) lane_finish(a, L, tl, dead);
}

// One turn of a warp: the collision turn when a.real_batch lanes (or every
// lane with an electron) have a pending collision, else the flight turn.
template <int MODE, class Sh>
__device__ __forceinline__ void warp_turn(const AdvanceArgs& a, Sh& sh, int wid, const IntervalView& iv,
                                          Lane& L, LaneTally& tl, unsigned live) {
  const unsigned pend = __ballot_sync(0xffffffffu, L.pending);
  if (__popc(pend) >= a.real_batch || pend == live) {
    if (L.pending) lane_real(a, sh, wid, iv, L, tl);
  } else if (L.have && !L.pending) {
    lane_flight<MODE>(a, sh, iv, L, tl);
  }
}

// block reductions of the lane sums and the per-process tallies -> the
// condition's global tallies (every thread of the block calls this)
template <class Sh>
__device__ __forceinline__ void block_flush(const AdvanceArgs& a, Sh& sh, const LaneTally& tl, int lane,
                                            int wid) {
  const double g = warp_sum((double)tl.gain);
  const double ta = warp_sum((double)tl.time_adj);
  const unsigned long long nn = warp_sum_u64((unsigned long long)tl.null_n);
  const unsigned long long nr = warp_sum_u64((unsigned long long)tl.real_n);
  const float em = warp_max(tl.e_max);
  if (lane == 0) {
    sh.red[wid] = g;
    sh.redt[wid] = ta;
    sh.redn[wid] = nn;
    sh.redr[wid] = nr;
    if (em > 0.0f) atomic_max_energy(a.max_energy_bits, em);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double gs = 0.0, ts = 0.0;
    unsigned long long ns = 0, rs = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      gs += sh.red[w];
      ts += sh.redt[w];
      ns += sh.redn[w];
      rs += sh.redr[w];
    }
    if (gs != 0.0) atomicAdd(a.field_gain, gs);
    if (ts != 0.0) atomicAdd(a.time_adjust, ts);
    if (ns) atomicAdd(a.null_count, ns);
    if (rs) atomicAdd(a.real_count, rs);
  }
  const ProcF* procs = procs_of(a, sh);
  for (int q = threadIdx.x; q < a.P; q += blockDim.x) {
    if (sh.count[q]) {
      atomicAdd(&a.proc_count[q], (unsigned long long)sh.count[q]);
      const double off = (double)nominal_change(procs[q]);
      const unsigned int n_loss = sh.neg[q], n_gain = sh.count[q] - n_loss;
      if (n_gain) atomicAdd(&a.proc_gain[q], (double)n_gain * off + (double)sh.gain[q]);
      if (n_loss) atomicAdd(&a.proc_loss[q], (double)n_loss * off + (double)sh.loss[q]);
    }
  }
}

// Bulk prefetch of [p, p + bytes) into L2 (p and bytes multiples of 16).
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
constexpr bool kPrefetchChunk = true;  // a claimed chunk's states, at the claim
constexpr bool kPrefetchRows = true;   // a parked collision's cumulative row (stash shapes)

// The index of the ensemble electron a lane claims (-1: none): the `n_want`
// claiming lanes (this one `wants` it, rank r among them) take the next
// electrons of the warp's chunk, and of a new chunk from the work counter
// when it runs out; `next`, `end` and `exhausted` are the warp-uniform cursors.
template <int CHUNK>
__device__ __forceinline__ int lane_claim(const AdvanceArgs& a, int n_want, int r, bool wants, int lane, int n_el,
                                          int& next, int& end, bool& exhausted) {
  int idx = -1;
  const int take = min(n_want, end - next);
  if (wants && r < take) idx = next + r;
  next += take;
  if (n_want > take) {
    int base = 0;
    if (lane == 0) base = atomicAdd(a.work_counter, CHUNK);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n_el) {
      exhausted = true;
    } else {
      next = base;
      end = min(base + CHUNK, n_el);
      if (kPrefetchChunk && lane == 0) prefetch_l2(a.state + 2 * base, (uint32_t)(end - base) * 2u * sizeof(float4));
      const int r2 = r - take;
      const int take2 = min(n_want - take, end - next);
      if (wants && r2 >= 0 && r2 < take2) idx = next + r2;
      next += take2;
    }
  }
  return idx;
}

// Lanes without an electron (`need`) take the next ones of the warp's chunk.
template <int CHUNK>
__device__ __forceinline__ void lane_take_chunk(const AdvanceArgs& a, const IntervalView& iv, Lane& L,
                                                unsigned need, int lane, unsigned lt_mask, int n_el, int& next,
                                                int& end, bool& exhausted) {
  const int idx = lane_claim<CHUNK>(a, __popc(need), __popc(need & lt_mask), !L.have, lane, n_el, next, end,
                                    exhausted);
  if (idx >= 0) lane_take_electron(a, iv, L, idx);
}

// The warps' work on one condition: the ensemble in 128-electron warp chunks
// from the condition's work counter, then each warp's queued secondaries (or,
// drain, only the spilled secondaries). Returns when the condition's counter
// and the warp's queue are exhausted; the caller flushes the lane sums.
template <int MODE, class Sh>
__device__ __forceinline__ void warp_loop(const AdvanceArgs& a, Sh& sh, const IntervalView& iv,
                                          LaneTally& tl, uint32_t& sec_id, uint32_t warp_tag) {
  const bool drain = a.queue_only != 0;
  const int n_el = drain ? 0 : a.n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  Lane L;
  reset_lane(L);
  // warp-uniform cursors: ensemble chunk, spill buffer (drain only)
  int next = 0, end = 0, sp_next = 0;
  bool exhausted = drain;

  for (;;) {
    __syncwarp();
    if (drain) __threadfence();
    // ---- refill lanes without an electron: the warp's own queued secondaries
    // first (the queue stays short, so it rarely spills), then the ensemble
    // chunk, then (drain) the spilled secondaries
    int qn = min(sh.qn[wid], a.local_q);
    if (qn > 0) qn = lane_take_queued(a, iv, sh, wid, lane, lt_mask, L, tl, sec_id, warp_tag);
    const unsigned need = __ballot_sync(0xffffffffu, !L.have);
    if (need && !exhausted) lane_take_chunk<Sh::kChunk>(a, iv, L, need, lane, lt_mask, n_el, next, end, exhausted);
    if (exhausted) {
      if (drain) {
        const unsigned idle2 = __ballot_sync(0xffffffffu, !L.have);
        const int cnt = min(*(volatile int*)a.spill_count, a.spill_cap);
        const int r2 = __popc(idle2 & lt_mask);
        const int take2 = min(__popc(idle2), cnt - sp_next);
        if (((idle2 >> lane) & 1u) && r2 < take2) {
          const int k = sp_next + r2;
          lane_take_secondary(a, iv, L, tl, __ldcg(&a.spill[2 * k]), __ldcg(&a.spill[2 * k + 1]),
                              0xFFFFFFFFu, (uint32_t)k);
        }
        sp_next += max(take2, 0);
      }
    }
    const unsigned live = __ballot_sync(0xffffffffu, L.have);
    if (!live) {
      const bool spill_left = drain && sp_next < min(*(volatile int*)a.spill_count, a.spill_cap);
      if (exhausted && qn == 0 && !spill_left) break;
      continue;
    }
    warp_turn<MODE>(a, sh, wid, iv, L, tl, live);
  }
}

// ------------------------------------------------------------ collision stash
// A stash record holds one electron in flight (64 bytes); a warp's NS records
// lie word-major in shared memory (four planes of NS 16-byte words), so lanes
// touching consecutive records touch consecutive words.
template <int NS>
__device__ __forceinline__ void stash_put(float4* wst, int e, const Lane& L) {
  wst[e] = make_float4(L.p.x, L.p.y, L.p.z, L.s);
  wst[NS + e] = make_float4(L.v.x, L.v.y, L.v.z, L.t);
  wst[2 * NS + e] = make_float4(L.energy, L.r, __int_as_float(L.slot), __int_as_float(L.events));
  wst[3 * NS + e] = make_float4(__uint_as_float((uint32_t)L.rng.state), __uint_as_float((uint32_t)(L.rng.state >> 32)),
                                __uint_as_float((uint32_t)L.rng.inc), __uint_as_float((uint32_t)(L.rng.inc >> 32)));
}

template <int NS>
__device__ __forceinline__ void stash_get(const float4* wst, int e, Lane& L) {
  const float4 w0 = wst[e], w1 = wst[NS + e], w2 = wst[2 * NS + e], w3 = wst[3 * NS + e];
  L.p = make_float3(w0.x, w0.y, w0.z);
  L.s = w0.w;
  L.v = make_float3(w1.x, w1.y, w1.z);
  L.t = w1.w;
  L.energy = w2.x;
  L.r = w2.y;
  L.slot = __float_as_int(w2.z);
  L.events = __float_as_int(w2.w);
  L.rng.state = ((uint64_t)__float_as_uint(w3.y) << 32) | __float_as_uint(w3.x);
  L.rng.inc = ((uint64_t)__float_as_uint(w3.w) << 32) | __float_as_uint(w3.z);
  L.have = true;
  L.pending = false;
}

// exchange of the lane's electron with record e, one 16-byte word at a time
// (never two whole electrons in registers)
template <int NS>
__device__ __forceinline__ void stash_swap(float4* wst, int e, Lane& L) {
  float4 w = wst[e];
  wst[e] = make_float4(L.p.x, L.p.y, L.p.z, L.s);
  L.p = make_float3(w.x, w.y, w.z);
  L.s = w.w;
  w = wst[NS + e];
  wst[NS + e] = make_float4(L.v.x, L.v.y, L.v.z, L.t);
  L.v = make_float3(w.x, w.y, w.z);
  L.t = w.w;
  w = wst[2 * NS + e];
  wst[2 * NS + e] = make_float4(L.energy, L.r, __int_as_float(L.slot), __int_as_float(L.events));
  L.energy = w.x;
  L.r = w.y;
  L.slot = __float_as_int(w.z);
  L.events = __float_as_int(w.w);
  w = wst[3 * NS + e];
  wst[3 * NS + e] = make_float4(__uint_as_float((uint32_t)L.rng.state), __uint_as_float((uint32_t)(L.rng.state >> 32)),
                                __uint_as_float((uint32_t)L.rng.inc), __uint_as_float((uint32_t)(L.rng.inc >> 32)));
  L.rng.state = ((uint64_t)__float_as_uint(w.y) << 32) | __float_as_uint(w.x);
  L.rng.inc = ((uint64_t)__float_as_uint(w.w) << 32) | __float_as_uint(w.z);
  L.have = true;
  L.pending = false;
}

// The warp loop of the stash shapes. A lane whose electron draws a real
// collision (or any thermal-target event) parks the electron in its warp's
// stash and takes another at once, so flight turns run on every lane that has
// work; once 32 collisions wait (or nothing is left to fly) the warp's
// collision turn takes 32 of them, one per lane: each lane parks the electron
// it is flying in the record it takes, so the collision code runs on full
// warps without holding two electrons. Parked flying electrons are ready
// ones, which idle lanes take before queued secondaries and new ensemble
// electrons. Every electron draws its random numbers in the same order as in
// warp_loop.
//
// The stash holds NS >= 64 records: pending collisions [0, np), ready
// electrons [np, np + nr) right above them (np, nr warp-uniform), so every
// exchange stays in place. A flight turn starts with np < 32; its r-th
// pending lane swaps its electron with record np + r, a ready one while
// r < nr (np + nr unchanged), else a free one (np grows to at most 63, nr
// to 0). The collision turn reads the top min(np, 32) pending records; lanes
// flying an electron take the lowest of them and leave their electron in its
// place, on top of the ready ones; empty lanes, which exist only once nothing
// is ready, take the rest. So np + nr <= 63 throughout.
template <int MODE, class Sh>
__device__ __forceinline__ void warp_loop_stash(const AdvanceArgs& a, Sh& sh, float4* wst, const IntervalView& iv,
                                                LaneTally& tl, uint32_t& sec_id, uint32_t warp_tag) {
  constexpr int NS = Sh::kStash;
  static_assert(NS >= 64, "the stash holds up to 63 records");
  const int n_el = a.n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  Lane L;
  reset_lane(L);
  int next = 0, end = 0, np = 0, nr = 0;
  bool exhausted = false;

  for (;;) {
    __syncwarp();
    // ---- refill lanes without an electron: ready electrons from the top of
    // the stash, then the warp's queued secondaries, then the ensemble chunk
    unsigned need = __ballot_sync(0xffffffffu, !L.have);
    if (need && nr > 0) {
      const int r = __popc(need & lt_mask);
      const int take = min(__popc(need), nr);
      if (!L.have && r < take) stash_get<NS>(wst, np + nr - 1 - r, L);
      nr -= take;
      need = __ballot_sync(0xffffffffu, !L.have);
    }
    int qn = min(sh.qn[wid], a.local_q);
    if (need && qn > 0) {
      qn = lane_take_queued(a, iv, sh, wid, lane, lt_mask, L, tl, sec_id, warp_tag);
      need = __ballot_sync(0xffffffffu, !L.have);
    }
    if (need && !exhausted) lane_take_chunk<Sh::kChunk>(a, iv, L, need, lane, lt_mask, n_el, next, end, exhausted);
    const unsigned live = __ballot_sync(0xffffffffu, L.have);

    // ---- collision turn on the top min(np, 32) pending records
    if (np >= 32 || (np > 0 && !live)) {
      const int k = min(np, 32), h = __popc(live);
      const int rank = L.have ? __popc(live & lt_mask) : h + __popc(~live & lt_mask);
      if (rank < k) {
        const int e = np - k + rank;
        if (L.have) stash_swap<NS>(wst, e, L);
        else stash_get<NS>(wst, e, L);
        lane_real(a, sh, wid, iv, L, tl);  // L.have turns false when the electron is done
      }
      np -= k;
      nr += min(k, h);
      continue;
    }
    if (!live) {
      // np == 0 and nr == 0 here: idle lanes take every ready record first
      if (exhausted && qn == 0) break;
      continue;
    }

    // ---- flight turn; a lane that drew a collision parks its electron and
    // takes a ready one in exchange while there are some
    if (L.have) lane_flight<MODE>(a, sh, iv, L, tl);
    const unsigned pend = __ballot_sync(0xffffffffu, L.pending);
    if (pend) {
      if (L.pending) {
        if (kPrefetchRows && !is_thermal(a.c, L.energy)) {
          // the process choice reads this row at the collision turn
          int i1;
          float w1, w2;
          row_weights(L.energy * iv.tab.inv_step, iv.tab.M, i1, w1, w2);
          prefetch_l2(iv.tab.cum_pair + (size_t)i1 * iv.tab.stride, (uint32_t)iv.tab.stride * (uint32_t)sizeof(float2));
        }
        const int r = __popc(pend & lt_mask), e = np + r;
        if (r < nr) {
          stash_swap<NS>(wst, e, L);
        } else {
          stash_put<NS>(wst, e, L);
          L.pending = false;
          L.have = false;
        }
      }
      const int k = __popc(pend);
      np += k;
      nr = max(nr - k, 0);
    }
  }
}

// One condition per launch (or, drain, its spilled secondaries).
template <int MODE, class Sh>
__device__ __forceinline__ void advance_body(const AdvanceArgs& a, Sh& sh) {
  load_block_consts(a, sh);
  __syncthreads();
  const IntervalView iv = interval_view<MODE>(a);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // drain launches: one block, whose warp tag stays below the spill's 0xFFFFFFFF
  const uint32_t warp_tag = (uint32_t)(blockIdx.x * Sh::kWarps + wid);
  LaneTally tl;
  reset_tally(tl);
  uint32_t sec_id = 0;
  warp_loop<MODE>(a, sh, iv, tl, sec_id, warp_tag);
  block_flush(a, sh, tl, lane, wid);
}

// ------------------------------------------------------------ batched advance
// word copy of a slot's advance arguments into shared memory (all threads)
__device__ __forceinline__ void load_slot_args(const AdvanceArgs* src, AdvanceArgs* dst) {
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int k = threadIdx.x; k < (int)(sizeof(AdvanceArgs) / sizeof(int)); k += blockDim.x) d[k] = s[k];
}

// Many conditions of one field branch in one persistent grid. A block works
// on one condition (slot) at a time: its warps take 128-electron chunks from
// that slot's own work counter, as in the single-condition kernel, and the
// slot's constants and per-process tallies stay in the block's shared memory.
// Blocks start spread over the branch's slots in proportion to their
// electrons; a block whose slot runs dry flushes its tallies and moves to the
// next slot of the branch that still has electrons, so the block synchronises
// only when it changes slot and idle blocks help finish large slots.
template <int MODE, int SHAPE>
__global__ void __launch_bounds__(AdvShape<SHAPE>::kThreads, AdvShape<SHAPE>::kBlocksPerSM)
    k_advance_batch(BatchArgs b) {
  using Sh = AdvSharedT<AdvShape<SHAPE>::kThreads / 32, AdvShape<SHAPE>::kChunk, AdvShape<SHAPE>::kStash>;
  __shared__ Sh sh;
  extern __shared__ float4 adv_stash[];  // adv_stash_bytes<SHAPE>() of dynamic shared memory
  __shared__ AdvanceArgs s_a;
  __shared__ IntervalView s_iv;
  __shared__ int s_slot;
  const int s0 = b.hdr->mode_slot[MODE], s1 = b.hdr->mode_slot[MODE + 1];
  if (s0 >= s1) return;  // no slot with this field branch (uniform over the grid)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t warp_tag = (uint32_t)(blockIdx.x * Sh::kWarps + wid);
  const int n_slots = b.hdr->n_slots;
  if (threadIdx.x == 0) {
    const int c0 = b.hdr->mode_chunk[MODE], c1 = b.hdr->mode_chunk[MODE + 1];
    const int c = c0 + (int)(((long long)blockIdx.x * (c1 - c0)) / gridDim.x);
    s_slot = slot_of_chunk(b.adv_prefix, n_slots, min(c, c1 - 1));
  }
  __syncthreads();
  LaneTally tl;
  uint32_t sec_id = 0;
  for (;;) {
    const int slot = s_slot;
    if (slot < 0) break;
    load_slot_args(&b.slots[slot].adv, &s_a);
    __syncthreads();
    load_block_consts(s_a, sh);
    if (threadIdx.x == 0) s_iv = interval_view<-1>(s_a);
    __syncthreads();
    reset_tally(tl);
    if constexpr (Sh::kStash > 0)
      warp_loop_stash<MODE>(s_a, sh, adv_stash + wid * 4 * Sh::kStash, s_iv, tl, sec_id, warp_tag);
    else
      warp_loop<MODE>(s_a, sh, s_iv, tl, sec_id, warp_tag);
    __syncthreads();  // every warp is done with the slot
    block_flush(s_a, sh, tl, lane, wid);
    __syncthreads();  // the flush has read the shared tallies and arguments
    // the next slot of the branch with electrons left, in rotation order from
    // this one: warp 0 checks 32 slots' counters per round
    if (wid == 0) {
      const int cnt = s1 - s0;
      int nxt = -1;
      for (int base = 1; base <= cnt && nxt < 0; base += 32) {
        const int k = base + lane;
        int s = -1;
        bool left = false;
        if (k <= cnt) {
          s = s0 + (slot - s0 + k) % cnt;
          const AdvanceArgs& o = b.slots[s].adv;
          left = *(volatile int*)o.work_counter < o.n;
        }
        const unsigned m = __ballot_sync(0xffffffffu, left);
        if (m) nxt = __shfl_sync(0xffffffffu, s, __ffs(m) - 1);
      }
      if (lane == 0) s_slot = nxt;
    }
    __syncthreads();
  }
}

}  // namespace

}  // namespace lgpu

namespace lgpu {
namespace {

// The batched advance of every field branch in `parts`, in launch shape SHAPE.
template <int SHAPE>
int launch_batch_advance_shape(const BatchArgs& b, int sm_count, unsigned parts, cudaStream_t s) {
  constexpr int kT = AdvShape<SHAPE>::kThreads, kDyn = adv_stash_bytes<SHAPE>();
  const int grid = sm_count * AdvShape<SHAPE>::kBlocksPerSM;
  int n = 0;
  if (parts & (1u << kFieldDC)) k_advance_batch<kFieldDC, SHAPE><<<grid, kT, kDyn, s>>>(b), ++n;
  if (parts & (1u << kFieldAC)) k_advance_batch<kFieldAC, SHAPE><<<grid, kT, kDyn, s>>>(b), ++n;
  if (parts & (1u << kFieldB)) k_advance_batch<kFieldB, SHAPE><<<grid, kT, kDyn, s>>>(b), ++n;
  if (parts & (1u << kFieldECR)) k_advance_batch<kFieldECR, SHAPE><<<grid, kT, kDyn, s>>>(b), ++n;
  if (parts & (1u << kFieldACB)) k_advance_batch<kFieldACB, SHAPE><<<grid, kT, kDyn, s>>>(b), ++n;
  return n;
}

// the dynamic shared memory of a stash shape's kernels, above the default limit
template <int SHAPE>
cudaError_t prepare_batch_advance_shape() {
  constexpr int kDyn = adv_stash_bytes<SHAPE>();
  cudaError_t e = cudaSuccess;
  if (kDyn == 0) return e;
  for (auto k : {k_advance_batch<kFieldDC, SHAPE>, k_advance_batch<kFieldAC, SHAPE>, k_advance_batch<kFieldB, SHAPE>,
                 k_advance_batch<kFieldECR, SHAPE>, k_advance_batch<kFieldACB, SHAPE>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kDyn);
  return e;
}

template <int SHAPE>
void shape_of(int* threads, int* blocks_per_sm, int* chunk, int* stash) {
  *threads = AdvShape<SHAPE>::kThreads;
  *blocks_per_sm = AdvShape<SHAPE>::kBlocksPerSM;
  *chunk = AdvShape<SHAPE>::kChunk;
  *stash = AdvShape<SHAPE>::kStash;
}

}  // namespace
}  // namespace lgpu
