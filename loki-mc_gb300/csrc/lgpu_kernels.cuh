// lgpu_kernels.cuh - launch interface of the electron Monte Carlo kernels
// (implemented in lgpu_kernels.cu, called by the host runtime).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lgpu_chunks.h"
#include "lgpu_types.h"

namespace lgpu {

constexpr int kMaxProcesses = 512;
constexpr int kMaxGases = 16;
constexpr int kMoments = 22;  // sum e, r(3), v(3), r r^T (6 unique), r v^T (9)

// Device scalars of one condition, read back after every interval.
// Per-interval fields first (cleared before every interval), cumulative after.
struct DevScalars {
  int sec_count, att_count, spill_count, error_flag;
  unsigned int max_energy_bits;
  int work_counter;
  int pop_counts[3];    // population control: alive secondaries, removed slots, surviving secondaries
  int pad1;
  unsigned long long null_count;
  unsigned long long real_count;
  double field_gain;
  double growth;
  double time_adjust;   // electron-time beyond N x interval: + secondaries, - attachments (s)
  unsigned int sample_max_bits;
  int pad2;
  double moments[kMoments];
};

// Arguments of one advance launch: every electron of the ensemble is pushed
// from the start of the synchronisation interval to its end, colliding on the
// way; secondaries created on the way are queued and pushed from their
// creation time to the end of the interval by the same launch.
struct AdvanceArgs {
  float4* state;            // [2*N]: (x, y, z, s) and (vx, vy, vz, dead flag) per electron
  int n;                    // electrons of the ensemble
  float dt_sync;            // interval length (s)
  float phi0;               // phase at the interval start (rad), FP64-reduced on the host
  float phase_rate;         // w (AC, AC+B) or W (resonance)
  float nu;                 // trial collision frequency (1/s)
  uint64_t seed;
  uint64_t interval;        // synchronisation interval index (random-number counter)
  uint32_t salt;
  float3 shift;             // origin shift subtracted from every position on load
  FieldF field;
  Consts c;
  TablesF t;
  const ProcF* procs;
  const GasF* gases;
  int P;
  // secondaries pushed to the end of the interval: (x, y, z, s), (vx, vy, vz, 0)
  float4* sec;
  int* sec_count;
  int sec_cap;
  // secondaries a warp could not keep in its own queue: (x, y, z, t_c), (vx, vy, vz, 0)
  float4* spill;
  int* spill_count;
  int spill_cap;
  int* att_list;                   // attached ensemble slots
  int* att_count;
  unsigned long long* proc_count;  // [P]
  double* proc_gain;               // [P]
  double* proc_loss;               // [P]
  unsigned long long* null_count;
  unsigned long long* real_count;
  double* field_gain;
  double* time_adjust;             // simulated electron-time beyond N * dt: + secondaries, - attachments (s)
  unsigned int* max_energy_bits;   // float bits of the largest final energy
  int* error_flag;                 // 2: secondary buffer full, 3: collision budget exhausted
  int* work_counter;               // chunk counter of the persistent grid (zero before the launch)
  int sm_count;
  const IntervalCtl* ctl;          // when set: per-interval values are read from here
  int queue_only;                  // 1: only drain the spilled secondaries (one warp)
  int real_batch;                  // pending real collisions that start a warp's collision turn (1..32)
  int coarse;                      // 1: null test against the block bounds first (t.nu_coarse)
  int local_q;                     // secondaries a warp queues before it spills (1..kLocalQ)
};
constexpr int kDefaultRealBatch = 20;

void launch_advance(const AdvanceArgs& a, cudaStream_t s);

// Per-process kernel attributes (dynamic shared memory of the histogram
// kernels); called on the current device before any launch or capture.
cudaError_t prepare_kernels();

struct InitArgs {
  float4* state;
  int n;
  float sd;                 // sqrt(k T_e / m)
  uint64_t seed;
  float half_me_over_e;
  unsigned int* max_energy_bits;
};
void launch_init(const InitArgs& a, cudaStream_t s);

// Table build on the device in FP64 (BoltzmannMC.C:561-615).
struct TableBuildArgs {
  int M, P, stride;
  double step, N;
  const int* is_super;
  const double* superw;
  const double* emin;
  const double* emax;
  const double* rel_dens;
  const int* raw_off;
  const int* raw_len;
  const double* raw_e;
  const double* raw_v;
  float2* nu_pair;
  float2* cum_pair;
  float2* sig_pair;
  double* nu_tot;     // FP64 total frequency per row
  double* nu_max;     // FP64 running maximum
  double* sig64;      // optional FP64 sigma*n [M*P] (tests), may be null
  double* cum64;      // optional FP64 cumulative [M*P] (tests), may be null
  float* nu_coarse;   // block bounds for the coarse null test [n_coarse], may be null
  int coarse_shift, n_coarse;
};
void launch_build_tables(const TableBuildArgs& a, cudaStream_t s);

// Ensemble sample: moment sums (FP64) and the largest energy.
struct SampleArgs {
  const float4* state;
  int n;
  float half_me_over_e;
  double* moments;                 // [kMoments], accumulated (zeroed by the caller)
  unsigned int* max_energy_bits;
};
// grid: at most four blocks per SM (sm_count = the device's multiprocessors)
void launch_sample(const SampleArgs& a, int sm_count, cudaStream_t s);

// Distribution tallies of one sample (BoltzmannMC.C:1550-1571).
struct HistArgs {
  const float4* state;
  int n;
  float half_me_over_e;
  int n_e_cells;
  float inv_e_step;                // 1 / EEDF energy step
  double* eedf;                    // [n_e_cells]
  double* eedf_periodic_row;       // [n_e_cells] or null
  int cylindrical;
  int n_cos;                       // EADF: [n_e_cells x n_cos]
  double* eadf;
  int n_rad, n_ax;                 // EVDF: [n_rad x n_ax]
  float inv_rad_step, inv_ax_step, max_speed;
  double* evdf;
  int evdf_done;                   // the EVDF of this sample was counted with its moments (batches)
  int pad;
};
void launch_hist(const HistArgs& a, cudaStream_t s);

// Population control (BoltzmannMC.C:1282-1408) at the end of an interval,
// when every electron and every secondary is at the synchronisation time.
struct PopArgs {
  float4* state;
  int n_electrons;
  const float4* sec;               // advanced secondaries (x, y, z, s), (vx, vy, vz, dead flag)
  const int* sec_count;            // may exceed sec_cap after an overflow (reported by the host)
  int sec_cap;
  int* counts;                     // [3] zero on entry: alive secondaries, removed slots, surviving secondaries
  const int* att_list;
  const int* att_count;
  unsigned int* claim;             // bitmap over n_electrons + sec_cap, all zero on entry and on exit
  int* alive;                      // [sec_cap] scratch: indices of secondaries that did not attach
  int* removed;                    // [sec_cap] scratch
  int* pair_slot;                  // [sec_cap] scratch
  int* pair_sec;                   // [sec_cap] scratch
  double* growth;                  // energy growth accumulator (eV)
  float half_me_over_e;
  uint64_t seed;
  const IntervalCtl* ctl;
  int* error_flag;                 // set when a bounded retry loop gives up
};
// Five launches (compaction, filling of attached slots, clones or removal
// draws, listing, pairing), each spread over many blocks.
void launch_pop_control(const PopArgs& a, cudaStream_t s);
constexpr int kPopLaunches = 5;

// ------------------------------------------------------------------ batches
// Many swarm conditions (slots) advanced by one launch sequence per interval.
// Each slot carries the same argument blocks a single-condition launch takes;
// the kernels split every slot's ensemble into fixed-size chunks and find the
// slot of a chunk by bisection over exclusive prefix sums of the chunk counts.
// kSlotEvdf: this interval's sample also counts the EVDF (its grid is fixed
// from the steady state on, so it needs no re-binning check)
enum SlotFlags : int { kSlotIonAtt = 1, kSlotSample = 2, kSlotEvdf = 8 };

struct BatchSlot {
  AdvanceArgs adv;        // adv.ctl points at ctl_dst
  PopArgs pop;
  SampleArgs smp;
  HistArgs hist;          // distribution staging only: the deferred tallies of a previous sample
  HistArgs vhist;         // EVDF counted with this interval's sample (kSlotEvdf)
  IntervalCtl ctl;        // this interval's values, copied to *ctl_dst by the prep kernel
  IntervalCtl* ctl_dst;
  DevScalars* sc;         // the condition's scalars; the per-interval part is cleared by prep
  int flags;              // SlotFlags
  int pad;
};

constexpr int kFieldModes = 5;

// Slots are ordered by field mode; the advance runs one launch per mode over
// that mode's slots [mode_slot[m], mode_slot[m + 1]).
struct BatchHeader {
  int n_slots;
  int adv_chunks, smp_chunks, hist_chunks;  // totals (last prefix entries)
  int mode_chunk[kFieldModes + 1];          // first advance chunk of each mode's slots
  int mode_slot[kFieldModes + 1];           // first slot of each mode
  int hist2_chunks;                         // velocity-distribution chunks (cylindrical slots)
  // the moment and distribution passes list each slot's full chunks first
  // (prefix over slots) and then one partial chunk per slot, largest first,
  // so that the blocks' static shares of the list come out even
  int smp_full, hist_full, hist2_full;
};

constexpr int kBatchMaxSlots = 1024;
constexpr int kBatchAdvanceChunk = 4096;   // granularity of the advance's initial spread of blocks over slots
constexpr int kBatchSampleChunk = 65535;   // electrons per block of the moment sums (and EVDF: < 2^16)
constexpr int kBatchHistChunk = 65535;     // electrons per block of the histograms (16-bit counts)

// Staging layout (host pinned mirror and device copy are identical):
//   BatchHeader | adv_prefix | smp_prefix | hist_prefix | hist2_prefix (kBatchMaxSlots+1 ints
//   each) | smp_part | hist_part | hist2_part (kBatchMaxSlots ints each, padded) | BatchSlot[...]
// The interval's staging fills the advance and moment parts, the distribution
// passes' staging (same layout) the hist parts and each slot's `hist`.
struct BatchArgs {
  BatchHeader* hdr;
  const BatchSlot* slots;
  const int* adv_prefix;
  const int* smp_prefix;    // full chunks before each slot
  const int* hist_prefix;   // energy and energy-angle distributions
  const int* hist2_prefix;  // velocity distribution (cylindrical slots)
  const int* smp_part;      // slots with a partial chunk, largest partial first
  const int* hist_part;
  const int* hist2_part;
  DevScalars* gather;       // [kBatchMaxSlots]: each slot's scalars after the interval
};
size_t batch_prefix_offset();   // bytes from the staging start to adv_prefix
size_t batch_slots_offset();    // bytes from the staging start to slots[0]
// One batched interval is three launch groups on one stream:
//   pre:     slot control blocks and per-interval scalars
//   advance: one persistent launch per field mode
//   post:    drain of spilled secondaries, population control, moments, gather
// ahead of them, from a second staging area of the same layout, the
// distribution passes of the previous interval's samples (`hist` of each
// slot), launched before the host prepares the interval so that its work
// runs beside them.
// `parts` leaves out the launches no slot of the interval needs: bit m (m <
// kFieldModes) for field mode m, then the flags below. Each returns the
// kernels it launched.
enum BatchParts : unsigned {
  kPartHistA = 1u << 8,   // a slot records its energy distributions
  kPartHistB = 1u << 9,   // a slot records its velocity distribution in a separate pass
  kPartSample = 1u << 10, // a slot samples its moments
  kPartIonAtt = 1u << 11, // a slot has ionization or attachment (drain, population control)
};
int launch_batch_pre(const BatchArgs& b, int sm_count, int max_slots, unsigned parts, cudaStream_t s);
int launch_batch_hist(const BatchArgs& b, int sm_count, unsigned parts, cudaStream_t s);
// The batched advance in one of kAdvShapes launch shapes (threads per block,
// blocks per SM, electrons a warp takes at a time, records of a warp's
// collision stash); advance_shape() names them. Shapes from 4 on are stash
// shapes (lgpu_advance_stash.cu).
constexpr int kAdvShapes = 6;
constexpr int kFirstStashShape = 4;
int launch_batch_advance(const BatchArgs& b, int sm_count, unsigned parts, int shape, cudaStream_t s);
int launch_batch_advance_stash(const BatchArgs& b, int sm_count, unsigned parts, int shape, cudaStream_t s);
void advance_shape(int shape, int* threads, int* blocks_per_sm, int* chunk, int* stash);
// dynamic shared memory of the stash shapes' kernels (part of prepare_kernels)
cudaError_t prepare_advance_stash();
int launch_batch_post(const BatchArgs& b, int sm_count, int max_slots, unsigned parts, cudaStream_t s);

// End-of-job EEDF post-processing in FP64 (lgpu_post.cu): the EEDF-convolved
// rate coefficient of every MC process (Collision.C:355-397) for each of
// n_eedf EEDFs (one block each), and the two-term swarm parameters
// (BoltzmannMC.C:2186-2266) of the first unless rates_only.
struct EedfPostArgs {
  int nc, P, n_eedf, rates_only;
  double max_energy, gas_density, omega, omega_c;
  const double* eedf_in;   // normalised EEDFs [n_eedf][nc], or null: normalise eeh
  const double* eeh;       // histogram sums [n_eedf][nc]
  const int* kind;         // per process: 0 elastic, 1 inelastic, 2 superelastic copy
  const int* ion;          // 1 ionization, 2 attachment
  const double* dens;      // target (product) relative density
  const double* thr;       // threshold (eV)
  const double* mass_ratio;
  const double* stat;      // g_target / g_product
  const int* int_off;
  const int* int_len;
  const int* mom_off;
  const int* mom_len;
  const double* raw_ie;
  const double* raw_iv;
  const double* raw_me;
  const double* raw_mv;
  double* scratch;         // [n_eedf][5 x (nc + 1)]
  double* rates;           // [n_eedf][P]
  double* params;          // [16], lgpu_eedf_params order
};
void launch_eedf_post(const EedfPostArgs& a, cudaStream_t s);

// Replay kernels for the parity tests: the production device functions
// driven by given inputs and recorded uniforms.
struct ReplayFlightArgs {
  int n;
  const double* phi0;     // phase at flight start (rad, already reduced)
  const double* dt;
  const double* pos;      // [n*3]
  const double* vel;      // [n*3]
  double* pos_out;
  double* vel_out;
  double* energy_out;
  double* gain_out;
  FieldF field;
  float half_me_over_e;
};
void launch_replay_flight(const ReplayFlightArgs& a, cudaStream_t s);

struct ReplayCollArgs {
  int n;
  const double* nu;
  const double* vel;      // [n*3]
  const double* energy;
  const double* u;        // [n*u_stride]
  int u_stride;
  double* out;            // [n*11]: chosen, v(3), energy, dE, dE/E, ej v(3), ej energy
  int* used;
  Consts c;
  TablesF t;
  const ProcF* procs;
  const GasF* gases;
  int coarse;             // 1: the null test of the advance kernels (block bounds first)
};
void launch_replay_collide(const ReplayCollArgs& a, cudaStream_t s);

}  // namespace lgpu
