// lgpu_batch.h - many swarm conditions per launch sequence.
//
// A Batch drives any number of Engines (one swarm condition each) through
// their own solve steps - the control flow of BoltzmannMC::evaluateEEDF
// (BoltzmannMC.C:299-426) stays per condition, on the host - while the device
// work of one synchronisation interval of every running condition is two CUDA
// graph launches: first the previous samples' distribution tallies (launched
// before the host works through the conditions, so that its work runs beside
// them), then slot control blocks and scalars (prep), one persistent advance
// launch per field branch over all slots' electrons, the drain of spilled
// secondaries, population control over all slots' items, the moment sums and
// a gather of every slot's scalars into mapped host memory. Per interval the
// host stages one BatchSlot per running condition (the argument blocks the
// single-condition launches take, plus the interval's control block) into
// pinned memory and copies it over once. A condition whose energy grid is
// re-built sits an interval out while the re-build runs on its own stream.
//
// Slots: at most max_slots conditions run at a time; conditions beyond that
// wait in order of addition and start as running ones finish, so a long run
// of uneven conditions keeps the device busy (continuous batching).
#pragma once

#include <algorithm>
#include <chrono>
#include <array>
#include <deque>
#include <mutex>
#include <map>
#include <string>
#include <vector>

#include "lgpu_engine.h"

namespace lgpu {

class Batch {
 public:
  std::string err_;
  int device_ = 0, max_slots_ = 0, sm_count_ = 1;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  // field branches after the first run their advance on side streams, forked
  // from and joined to the batch stream inside the interval graph
  cudaStream_t side_[kFieldModes - 1] = {};
  cudaEvent_t fork_ = nullptr, join_[kFieldModes - 1] = {};
  char* h_stage_ = nullptr;
  char* d_stage_ = nullptr;
  char* h_hstage_ = nullptr;  // the distribution passes' staging (same layout)
  char* d_hstage_ = nullptr;
  DevScalars* h_gather_ = nullptr;  // mapped pinned memory: the gather kernel writes it directly
  DevScalars* d_gather_ = nullptr;  // its device address
  // one instantiated graph per set of launch groups in use (BatchParts; the
  // distribution passes' graphs carry kGraphHist)
  static constexpr unsigned kGraphHist = 1u << 16;
  std::map<unsigned, std::pair<cudaGraphExec_t, int>> graphs_;
  // scratch of the pass layouts (lgpu_chunks.h): electrons and inclusion per
  // slot, remainders
  std::vector<int> n_;
  std::vector<unsigned char> take_, all_;
  std::vector<std::pair<int, int>> rem_;
  // totals since creation
  long long intervals_ = 0, launches_ = 0;
  double adv_ms_ = 0, electron_steps_ = 0, h2d_bytes_ = 0, d2h_bytes_ = 0;
  double real_ = 0, null_ = 0;  // collisions of the batched intervals
  double host_ms_ = 0, secondaries_ = 0, spilled_ = 0, attached_ = 0, regrids_ = 0;

  // On-line autotuner of the advance's scheduling, which changes no result
  // (what an electron draws and decides does not depend on it), so tuning
  // intervals are ordinary intervals. Two stages, each candidate taking
  // kTuneRounds intervals (in turn, every other round in reverse order) and
  // the least advance time per trial event (median) winning:
  //  0. the launch shape (kAdvShapes: threads per block x blocks per SM, i.e.
  //     the register budget, and the electrons a warp takes at a time);
  //  1. for members whose config leaves the threshold at 0, the
  //     collision-turn threshold (AdvanceArgs::real_batch) and the table
  //     staging of the null test: block bounds of the total frequency staged
  //     in shared memory first, or the table rows straight from L2
  //     (AdvanceArgs::coarse). A stash shape's collision turn always takes
  //     32 collisions, so for it only the staging is tuned.
  // The choice is kept per mixture, keyed by (largest process count, table
  // points, field branches in use, thermal targets), for the life of the
  // process: a later batch or server interval with the same key starts tuned.
  static constexpr int kTuneThresholds[5] = {12, 16, 20, 24, 28};
  static constexpr int kTuneCandidates = 10;  // thresholds x coarse test off / on
  static constexpr int kTuneDefault = 7;      // threshold 20 with the block bounds
  static constexpr int kTuneRounds = 3;
  int tune_stage_ = 0;  // 0 launch shape, 1 threshold x staging, 2 tuned
  int tune_next_ = 0;   // intervals measured in the current stage
  int shape_ = 0;       // launch shape (from stage 0 on)
  int tuned_ = -1;      // threshold x staging candidate, -1 while tuning
  std::array<long long, 4> tune_key_{};
  std::vector<double> tune_cost_[kTuneCandidates];
  static int tune_threshold(int c) { return kTuneThresholds[c % 5]; }
  static int tune_coarse(int c) { return c / 5; }
  static_assert(kAdvShapes <= kTuneCandidates, "stage costs share tune_cost_");
  // stage 1: the candidates of the chosen shape, and the k-th one's index
  int stage1_count() const { return shape_ >= kFirstStashShape ? 2 : kTuneCandidates; }
  int stage1_cand(int k) const { return shape_ >= kFirstStashShape ? 5 * k + 2 : k; }
  struct TunePoint {
    int shape, cand;
  };
  static std::map<std::array<long long, 4>, TunePoint>& tune_cache() {
    static std::map<std::array<long long, 4>, TunePoint> m;
    return m;
  }
  static std::mutex& tune_mutex() {
    static std::mutex mu;
    return mu;
  }
  // a pinned schedule (shape >= 0) or on-line tuning again (shape -1)
  int set_schedule(int shape, int real_batch, int coarse) {
    if (shape < 0) {
      tune_stage_ = 0;
      tune_next_ = 0;
      tuned_ = -1;
      for (auto& c : tune_cost_) c.clear();
      return LGPU_OK;
    }
    int t = 0;
    while (t < 5 && kTuneThresholds[t] != real_batch) ++t;
    if (shape >= kAdvShapes || (coarse != 0 && coarse != 1) || (t == 5 && shape < kFirstStashShape))
      return fail(LGPU_ERR_BAD_ARG, "schedule: shape " + std::to_string(shape) + " (0.." +
                                        std::to_string(kAdvShapes - 1) + "), threshold " + std::to_string(real_batch) +
                                        " (12, 16, 20, 24, 28), coarse " + std::to_string(coarse) + " (0, 1)");
    shape_ = shape;
    tuned_ = (t == 5 ? 2 : t) + 5 * coarse;
    tune_stage_ = 2;
    tune_next_ = 0;
    return LGPU_OK;
  }
  // the median cost of each candidate: the cheapest
  int tune_pick(int n) {
    double best = 0;
    int pick = 0;
    for (int k = 0; k < n; ++k) {
      std::vector<double> v = tune_cost_[k];
      std::sort(v.begin(), v.end());
      const double med = v[v.size() / 2];
      if (k == 0 || med < best) {
        best = med;
        pick = k;
      }
    }
    for (auto& c : tune_cost_) c.clear();
    return pick;
  }

  struct Member {
    Engine* e = nullptr;
    bool started = false, done = false;
    bool released = false;  // done and no longer looked at by its owner
    int status = LGPU_OK;
    lgpu_result result{};
  };
  // Members by id, in the order added: member id k is members_[k - base_].
  // A long-running owner (the server) releases finished members, and
  // compact() drops released ones from the front, so the bookkeeping stays
  // bounded by the members added during the longest running one's solve.
  std::deque<Member> members_;
  int base_ = 0;             // id of members_.front()
  std::vector<int> active_;  // ids of started, unfinished members
  int next_start_ = 0;       // id of the first member not started yet

  Member& member(int id) { return members_[(size_t)(id - base_)]; }
  int end_id() const { return base_ + (int)members_.size(); }
  void release_member(int id) {
    Member& m = member(id);
    m.e = nullptr;
    m.released = true;
  }
  void compact() {
    while (!members_.empty() && members_.front().released && base_ < next_start_) {
      members_.pop_front();
      ++base_;
    }
  }
  void clear_members() {
    members_.clear();
    active_.clear();
    base_ = 0;
    next_start_ = 0;
  }

  ~Batch() { release(); }

  int fail(int code, const std::string& msg) {
    err_ = msg;
    return code;
  }
  int cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LGPU_OK;
    return fail(e == cudaErrorMemoryAllocation ? LGPU_ERR_OOM : LGPU_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
  }

  static size_t stage_bytes() { return batch_slots_offset() + (size_t)kBatchMaxSlots * sizeof(BatchSlot); }

  int init(int device, int max_slots) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(LGPU_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(LGPU_ERR_BAD_ARG, "device out of range");
    if (max_slots < 1 || max_slots > kBatchMaxSlots)
      return fail(LGPU_ERR_BAD_ARG, "max_slots must be 1.." + std::to_string(kBatchMaxSlots));
    device_ = device;
    max_slots_ = max_slots;
    int rc;
    if ((rc = cuda(cudaSetDevice(device), "cudaSetDevice"))) return rc;
    if ((rc = cuda(prepare_kernels(), "kernel attributes"))) return rc;
    if ((rc = cuda(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device), "attribute"))) return rc;
    if ((rc = cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream"))) return rc;
    if ((rc = cuda(cudaEventCreate(&ev0_), "event")) || (rc = cuda(cudaEventCreate(&ev1_), "event"))) return rc;
    if ((rc = cuda(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming), "event"))) return rc;
    for (int k = 0; k < kFieldModes - 1; ++k)
      if ((rc = cuda(cudaStreamCreateWithFlags(&side_[k], cudaStreamNonBlocking), "stream")) ||
          (rc = cuda(cudaEventCreateWithFlags(&join_[k], cudaEventDisableTiming), "event")))
        return rc;
    const size_t sb = stage_bytes();
    if ((rc = cuda(cudaMallocHost((void**)&h_stage_, sb), "cudaMallocHost"))) return rc;
    if ((rc = cuda(cudaMalloc((void**)&d_stage_, sb), "cudaMalloc"))) return rc;
    std::memset(h_stage_, 0, sb);
    if ((rc = cuda(cudaMemsetAsync(d_stage_, 0, sb, stream_), "memset"))) return rc;
    if ((rc = cuda(cudaMallocHost((void**)&h_hstage_, sb), "cudaMallocHost"))) return rc;
    if ((rc = cuda(cudaMalloc((void**)&d_hstage_, sb), "cudaMalloc"))) return rc;
    std::memset(h_hstage_, 0, sb);
    if ((rc = cuda(cudaMemsetAsync(d_hstage_, 0, sb, stream_), "memset"))) return rc;
    if ((rc = cuda(cudaHostAlloc((void**)&h_gather_, (size_t)max_slots * sizeof(DevScalars), cudaHostAllocMapped),
                   "cudaHostAlloc")))
      return rc;
    if ((rc = cuda(cudaHostGetDevicePointer((void**)&d_gather_, h_gather_, 0), "cudaHostGetDevicePointer"))) return rc;
    return cuda(cudaStreamSynchronize(stream_), "init");
  }

  void release() {
    if (stream_) cudaStreamSynchronize(stream_);
    for (Member& m : members_)
      if (m.e && !m.done) m.e->leave_batch();
    clear_members();
    for (auto& g : graphs_) cudaGraphExecDestroy(g.second.first);
    graphs_.clear();
    if (d_stage_) cudaFree(d_stage_);
    if (h_stage_) cudaFreeHost(h_stage_);
    if (d_hstage_) cudaFree(d_hstage_);
    if (h_hstage_) cudaFreeHost(h_hstage_);
    d_hstage_ = h_hstage_ = nullptr;
    if (h_gather_) cudaFreeHost(h_gather_);
    d_stage_ = h_stage_ = nullptr;
    d_gather_ = h_gather_ = nullptr;
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    ev0_ = ev1_ = nullptr;
    if (fork_) cudaEventDestroy(fork_);
    fork_ = nullptr;
    for (int k = 0; k < kFieldModes - 1; ++k) {
      if (join_[k]) cudaEventDestroy(join_[k]);
      if (side_[k]) cudaStreamDestroy(side_[k]);
      join_[k] = nullptr;
      side_[k] = nullptr;
    }
    if (stream_) cudaStreamDestroy(stream_);
    stream_ = nullptr;
  }

  BatchArgs args(char* stage) const {
    BatchArgs b{};
    b.hdr = reinterpret_cast<BatchHeader*>(stage);
    b.adv_prefix = reinterpret_cast<const int*>(stage + batch_prefix_offset());
    b.smp_prefix = b.adv_prefix + (kBatchMaxSlots + 1);
    b.hist_prefix = b.smp_prefix + (kBatchMaxSlots + 1);
    b.hist2_prefix = b.hist_prefix + (kBatchMaxSlots + 1);
    b.smp_part = b.hist2_prefix + (kBatchMaxSlots + 1);
    b.hist_part = b.smp_part + kBatchMaxSlots;
    b.hist2_part = b.hist_part + kBatchMaxSlots;
    b.slots = reinterpret_cast<const BatchSlot*>(stage + batch_slots_offset());
    b.gather = d_gather_;
    return b;
  }

  // the kernels of one interval (or of the distribution passes, kGraphHist),
  // captured once per set of launch groups: their sizes come from the staged
  // header, so one graph serves every interval and every membership
  // graph keys: the launch groups (BatchParts) and, above bit 20, the shape
  static constexpr int kGraphShapeShift = 20;
  int graph(unsigned parts, cudaGraphExec_t* out, int* kernels) {
    auto it = graphs_.find(parts);
    if (it == graphs_.end()) {
      cudaGraph_t g;
      int rc;
      if ((rc = cuda(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture"))) return rc;
      int n = 0;
      if (parts & kGraphHist) {
        n = launch_batch_hist(args(d_hstage_), sm_count_, parts, stream_);
      } else {
        const BatchArgs b = args(d_stage_);
        n = launch_batch_pre(b, sm_count_, max_slots_, parts, stream_);
        cudaEventRecordWithFlags(ev0_, stream_, cudaEventRecordExternal);
        // one persistent launch per field branch; with several branches they
        // run side by side, so the blocks of one fill the SMs another's tail
        // leaves idle (each branch's slots are its own: nothing is shared)
        const int shape = (int)(parts >> kGraphShapeShift);
        const unsigned modes = parts & ((1u << kFieldModes) - 1u);
        const unsigned rest = parts & ~((1u << kFieldModes) - 1u);
        int first = 0;
        while (first < kFieldModes && !(modes & (1u << first))) ++first;
        int k = 0;
        if (modes & ~(1u << first)) cudaEventRecord(fork_, stream_);
        for (int m = first + 1; m < kFieldModes; ++m) {
          if (!(modes & (1u << m))) continue;
          cudaStreamWaitEvent(side_[k], fork_, 0);
          n += launch_batch_advance(b, sm_count_, rest | (1u << m), shape, side_[k]);
          cudaEventRecord(join_[k], side_[k]);
          ++k;
        }
        if (first < kFieldModes) n += launch_batch_advance(b, sm_count_, rest | (1u << first), shape, stream_);
        for (int j = 0; j < k; ++j) cudaStreamWaitEvent(stream_, join_[j], 0);
        cudaEventRecordWithFlags(ev1_, stream_, cudaEventRecordExternal);
        n += launch_batch_post(b, sm_count_, max_slots_, parts, stream_);
      }
      if ((rc = cuda(cudaStreamEndCapture(stream_, &g), "capture"))) return rc;
      cudaGraphExec_t ge = nullptr;
      rc = cuda(cudaGraphInstantiate(&ge, g, 0), "instantiate");
      cudaGraphDestroy(g);
      if (rc) return rc;
      it = graphs_.emplace(parts, std::make_pair(ge, n)).first;
    }
    *out = it->second.first;
    *kernels = it->second.second;
    return LGPU_OK;
  }

  // ------------------------------------------------------------ membership
  int add(Engine* e) {
    if (!e) return fail(LGPU_ERR_BAD_ARG, "null context");
    if (e->batch_) return fail(LGPU_ERR_STATE, "the context is already in a batch");
    if (e->cfg_.device != device_) return fail(LGPU_ERR_BAD_ARG, "the context is on another device");
    if (!e->have_procs_ || !e->have_cond_) return fail(LGPU_ERR_STATE, "set_processes and set_conditions come first");
    for (const Member& m : members_)
      if (m.e == e && !m.done) return fail(LGPU_ERR_BAD_ARG, "the context was added twice");
    Member m;
    m.e = e;
    members_.push_back(m);
    e->enter_batch(stream_);  // held by the batch from here on
    return LGPU_OK;
  }

  void finish(Member& m, int rc) {
    if (rc == LGPU_OK) rc = m.e->solve_end(&m.result);
    if (rc != LGPU_OK) m.e->sync("finish");  // the context's own work ends before it leaves
    m.status = rc;
    m.done = true;
    m.e->leave_batch();
  }

  // starts waiting members while slots are free
  void admit() {
    while ((int)active_.size() < max_slots_ && next_start_ < end_id()) {
      Member& m = member(next_start_);
      m.started = true;
      const int rc = m.e->solve_begin();
      if (rc != LGPU_OK) finish(m, rc);
      else active_.push_back(next_start_);
      ++next_start_;
    }
  }

  bool idle() const { return active_.empty() && next_start_ >= end_id(); }

  // ends a running member between intervals with the given status
  void stop_member(int idx, int status) {
    Member& m = member(idx);
    if (!m.started || m.done) return;
    m.e->sync("stop");
    m.status = status;
    m.done = true;
    m.e->leave_batch();
    active_.erase(std::remove(active_.begin(), active_.end(), idx), active_.end());
  }

  // One synchronisation interval of every running member. Members whose stop
  // criteria hold (or that fail) finish here; *finished lists them. A member
  // whose energy grid is being re-built (on its own stream, concurrently with
  // this interval) sits the interval out and goes on at the next step.
  int step(std::vector<int>* finished = nullptr) {
    const auto h0 = std::chrono::steady_clock::now();
    // the previous samples' distribution passes first: the host work below
    // (stop criteria, trial frequencies, staging) runs while they do
    if (int rc = launch_pending_hists()) return rc;
    std::vector<int> go, wait;
    go.reserve(active_.size());
    for (int idx : active_) {
      Member& m = member(idx);
      bool done = false, ready = true;
      int rc = m.e->solve_next(&done);
      if (rc == LGPU_OK && !done) rc = m.e->interval_pre(&ready);
      if (rc != LGPU_OK || done) {
        finish(m, rc);
        if (finished) finished->push_back(idx);
      } else if (!ready) {
        wait.push_back(idx);
        ++regrids_;
      } else {
        go.push_back(idx);
      }
    }
    active_ = go;
    active_.insert(active_.end(), wait.begin(), wait.end());
    if (go.empty()) {
      // only re-grids in flight: let them finish before the next step
      for (int idx : wait)
        if (int rc = member(idx).e->settle_tables()) return rc;
      return LGPU_OK;
    }
    // slots ordered by field branch: one advance launch per branch
    std::stable_sort(go.begin(), go.end(),
                     [&](int a, int b) { return member(a).e->field_mode() < member(b).e->field_mode(); });
    const int n = (int)go.size();
    auto* hdr = reinterpret_cast<BatchHeader*>(h_stage_);
    int* ap = reinterpret_cast<int*>(h_stage_ + batch_prefix_offset());
    int* sp = ap + (kBatchMaxSlots + 1);
    int* spart = sp + 3 * (kBatchMaxSlots + 1);  // after the two distribution prefixes (other staging)
    n_.resize(n);
    take_.resize(n);
    auto* sl = reinterpret_cast<BatchSlot*>(h_stage_ + batch_slots_offset());
    int na = 0;
    unsigned parts = 0;
    double electrons = 0;
    if (tune_stage_ == 0 && tune_next_ == 0) {
      // the mixture's key; a known one starts tuned
      tune_key_ = {0, 0, 0, 0};
      for (int s = 0; s < n; ++s) {
        Engine* e = member(go[s]).e;
        tune_key_[0] = std::max<long long>(tune_key_[0], e->P_);
        tune_key_[1] = std::max<long long>(tune_key_[1], e->M_);
        tune_key_[2] |= 1ll << e->field_mode();
        tune_key_[3] |= e->cfg_.gas_temperature_effect != 0;
      }
      std::lock_guard<std::mutex> lock(tune_mutex());
      auto it = tune_cache().find(tune_key_);
      if (it != tune_cache().end()) {
        shape_ = it->second.shape;
        tuned_ = it->second.cand;
        tune_stage_ = 2;
      }
    }
    // candidates in turn, every other round in reverse order, so that a drift
    // of the ensemble during tuning (heating from the start) favours none
    auto turn = [&](int n) {
      const int k = tune_next_ % n;
      return (tune_next_ / n) & 1 ? n - 1 - k : k;
    };
    const int shape = tune_stage_ == 0 ? turn(kAdvShapes) : shape_;
    const int k1 = tune_stage_ == 1 ? turn(stage1_count()) : 0;
    const int cand = tune_stage_ == 0 ? kTuneDefault : (tune_stage_ == 1 ? stage1_cand(k1) : tuned_);
    for (int s = 0; s < n; ++s) {
      Engine* e = member(go[s]).e;
      e->fill_slot(&sl[s]);
      if (e->cfg_.advance_real_batch == 0) {
        sl[s].adv.real_batch = tune_threshold(cand);
        sl[s].adv.coarse = tune_coarse(cand);
      }
      const int N = e->n_electrons();
      electrons += N;
      parts |= 1u << e->field_mode();
      if (sl[s].flags & kSlotIonAtt) parts |= kPartIonAtt;
      ap[s] = na;
      na += (N + kBatchAdvanceChunk - 1) / kBatchAdvanceChunk;
      n_[s] = N;
      take_[s] = (sl[s].flags & kSlotSample) ? 1 : 0;
    }
    ap[n] = na;
    const auto smp = layout_pass(n, n_.data(), take_.data(), kBatchSampleChunk, sp, spart, rem_);
    std::memset(hdr, 0, sizeof(BatchHeader));
    hdr->n_slots = n;
    hdr->adv_chunks = na;
    hdr->smp_full = smp.first;
    hdr->smp_chunks = smp.first + smp.second;
    if (hdr->smp_chunks) parts |= kPartSample;
    for (int m = 0, s = 0; m <= kFieldModes; ++m) {
      while (s < n && member(go[s]).e->field_mode() < m) ++s;
      hdr->mode_chunk[m] = ap[s];
      hdr->mode_slot[m] = s;
    }
    cudaGraphExec_t ge;
    int rc, kernels = 0;
    if ((rc = graph(parts | ((unsigned)shape << kGraphShapeShift), &ge, &kernels))) return rc;
    const size_t up = batch_slots_offset() + (size_t)n * sizeof(BatchSlot);
    const size_t down = (size_t)n * sizeof(DevScalars);
    if ((rc = cuda(cudaMemcpyAsync(d_stage_, h_stage_, up, cudaMemcpyHostToDevice, stream_), "stage"))) return rc;
    if ((rc = cuda(cudaGraphLaunch(ge, stream_), "graph launch"))) return rc;
    const auto h1 = std::chrono::steady_clock::now();
    if ((rc = cuda(cudaStreamSynchronize(stream_), "batched interval"))) return rc;
    const auto h2 = std::chrono::steady_clock::now();
    if ((rc = cuda(cudaGetLastError(), "batched interval"))) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    adv_ms_ += ms;
    if (tune_stage_ < 2 && electrons > 0) {
      // cost per trial event (real + null collisions of the interval): the
      // events per electron-interval change as the ensemble relaxes
      double events = 0;
      for (int s = 0; s < n; ++s) {
        const Member& m = member(go[s]);
        events += (double)(h_gather_[s].real_count - m.e->h_sc_->real_count) +
                  (double)(h_gather_[s].null_count - m.e->h_sc_->null_count);
      }
      const int nc = tune_stage_ == 0 ? kAdvShapes : stage1_count();
      tune_cost_[tune_stage_ == 0 ? shape : k1].push_back(ms / std::max(events, electrons));
      if (++tune_next_ >= nc * kTuneRounds) {
        const int pick = tune_pick(nc);
        tune_next_ = 0;
        if (tune_stage_ == 0) {
          shape_ = pick;
          tune_stage_ = 1;
        } else {
          tuned_ = stage1_cand(pick);
          tune_stage_ = 2;
          std::lock_guard<std::mutex> lock(tune_mutex());
          tune_cache()[tune_key_] = TunePoint{shape_, tuned_};
        }
      }
    }
    electron_steps_ += electrons;
    ++intervals_;
    launches_ += kernels;
    h2d_bytes_ += (double)up;
    d2h_bytes_ += (double)down;
    std::vector<int> still;
    still.reserve(go.size());
    for (int s = 0; s < n; ++s) {
      Member& m = member(go[s]);
      real_ += (double)(h_gather_[s].real_count - m.e->h_sc_->real_count);
      null_ += (double)(h_gather_[s].null_count - m.e->h_sc_->null_count);
      secondaries_ += h_gather_[s].sec_count;
      spilled_ += h_gather_[s].spill_count;
      attached_ += h_gather_[s].att_count;
      std::memcpy(m.e->h_sc_, &h_gather_[s], sizeof(DevScalars));
      rc = m.e->interval_post();
      if (rc == LGPU_OK) rc = m.e->solve_post();
      if (rc != LGPU_OK) {
        finish(m, rc);
        if (finished) finished->push_back(go[s]);
      } else {
        still.push_back(go[s]);
      }
    }
    // re-grids end within the step that launched them (they ran beside it)
    for (int idx : wait)
      if ((rc = member(idx).e->settle_tables())) return rc;
    still.insert(still.end(), wait.begin(), wait.end());
    active_ = still;
    const auto h3 = std::chrono::steady_clock::now();
    host_ms_ += 1e3 * (std::chrono::duration<double>(h1 - h0).count() + std::chrono::duration<double>(h3 - h2).count());
    return LGPU_OK;
  }

  // The deferred distribution tallies of the running members' last samples
  // (EEDF, EADF and, before the velocity grid is fixed, EVDF), staged in the
  // second staging area and launched as their own graph on the batch stream,
  // ahead of the interval that would otherwise advance the ensemble first.
  int launch_pending_hists() {
    auto* hdr = reinterpret_cast<BatchHeader*>(h_hstage_);
    int* hp = reinterpret_cast<int*>(h_hstage_ + batch_prefix_offset()) + 2 * (kBatchMaxSlots + 1);
    int* vp = hp + (kBatchMaxSlots + 1);
    int* hpart = vp + (kBatchMaxSlots + 1) + kBatchMaxSlots;
    int* vpart = hpart + kBatchMaxSlots;
    auto* sl = reinterpret_cast<BatchSlot*>(h_hstage_ + batch_slots_offset());
    int n = 0;
    n_.clear();
    take_.clear();
    for (int idx : active_) {
      HistArgs h;
      if (!member(idx).e->take_pending_hist(&h)) continue;
      sl[n++].hist = h;
      n_.push_back(h.n);
      take_.push_back(h.cylindrical && !h.evdf_done ? 1 : 0);  // pass B: the EVDF not counted yet
    }
    if (n == 0) return LGPU_OK;
    all_.assign(n, 1);
    const auto pa = layout_pass(n, n_.data(), all_.data(), kBatchHistChunk, hp, hpart, rem_);
    const auto pb = layout_pass(n, n_.data(), take_.data(), kBatchHistChunk, vp, vpart, rem_);
    std::memset(hdr, 0, sizeof(BatchHeader));
    hdr->n_slots = n;
    hdr->hist_full = pa.first;
    hdr->hist2_full = pb.first;
    hdr->hist_chunks = pa.first + pa.second;
    hdr->hist2_chunks = pb.first + pb.second;
    const unsigned parts = kGraphHist | (hdr->hist_chunks ? kPartHistA : 0u) | (hdr->hist2_chunks ? kPartHistB : 0u);
    cudaGraphExec_t ge;
    int rc, kernels = 0;
    if ((rc = graph(parts, &ge, &kernels))) return rc;
    const size_t up = batch_slots_offset() + (size_t)n * sizeof(BatchSlot);
    if ((rc = cuda(cudaMemcpyAsync(d_hstage_, h_hstage_, up, cudaMemcpyHostToDevice, stream_), "stage"))) return rc;
    if ((rc = cuda(cudaGraphLaunch(ge, stream_), "graph launch"))) return rc;
    launches_ += kernels;
    h2d_bytes_ += (double)up;
    return LGPU_OK;
  }

  // every added member to the end
  int run() {
    for (;;) {
      admit();
      if (active_.empty()) break;
      const int rc = step();
      if (rc != LGPU_OK) return rc;
    }
    return LGPU_OK;
  }
};

}  // namespace lgpu

struct lgpu_batch {
  lgpu::Batch* b;
};
