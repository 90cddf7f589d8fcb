// lgpu_batch.cpp - the batch entry points of include/loki_gpu.h over lgpu::Batch.
#include "lgpu_batch.h"

#include <new>

extern "C" {

int lgpu_batch_create(int device, int max_slots, lgpu_batch** out) {
  if (!out) return LGPU_ERR_BAD_ARG;
  *out = nullptr;
  lgpu::Batch* b = new (std::nothrow) lgpu::Batch();
  if (!b) return LGPU_ERR_OOM;
  lgpu_batch* h = new (std::nothrow) lgpu_batch{b};
  if (!h) {
    delete b;
    return LGPU_ERR_OOM;
  }
  *out = h;
  return b->init(device, max_slots);
}

int lgpu_batch_destroy(lgpu_batch* batch) {
  if (!batch) return LGPU_OK;
  delete batch->b;
  delete batch;
  return LGPU_OK;
}

int lgpu_batch_last_error(const lgpu_batch* batch, char* buf, size_t size) {
  if (!batch || !batch->b) return 0;
  const std::string& s = batch->b->err_;
  if (buf && size) std::snprintf(buf, size, "%s", s.c_str());
  return (int)s.size();
}

int lgpu_batch_add(lgpu_batch* batch, lgpu_ctx* ctx) {
  if (!batch || !batch->b || !ctx || !ctx->e) return LGPU_ERR_BAD_ARG;
  return batch->b->add(ctx->e);
}

void* lgpu_batch_stream(lgpu_batch* batch) { return (batch && batch->b) ? (void*)batch->b->stream_ : nullptr; }

int lgpu_batch_start(lgpu_batch* batch) {
  if (!batch || !batch->b) return LGPU_ERR_BAD_ARG;
  batch->b->admit();
  return LGPU_OK;
}

int lgpu_batch_set_schedule(lgpu_batch* batch, int shape, int real_batch, int coarse) {
  if (!batch || !batch->b) return LGPU_ERR_BAD_ARG;
  return batch->b->set_schedule(shape, real_batch, coarse);
}

int lgpu_batch_step(lgpu_batch* batch, int n, int* running, lgpu_batch_report* report) {
  if (!batch || !batch->b || n < 0) return LGPU_ERR_BAD_ARG;
  lgpu::Batch& b = *batch->b;
  const long long i0 = b.intervals_, l0 = b.launches_;
  const double a0 = b.adv_ms_, s0 = b.electron_steps_, u0 = b.h2d_bytes_, d0 = b.d2h_bytes_, r0 = b.real_,
               n0 = b.null_, hm0 = b.host_ms_, se0 = b.secondaries_, sp0 = b.spilled_, at0 = b.attached_, rg0 = b.regrids_;
  const auto t0 = std::chrono::steady_clock::now();
  int rc = LGPU_OK;
  for (int i = 0; i < n && rc == LGPU_OK; ++i) {
    b.admit();
    if (b.active_.empty()) break;
    rc = b.step();
  }
  if (running) *running = (int)b.active_.size();
  if (report) {
    report->intervals = b.intervals_ - i0;
    report->kernel_launches = b.launches_ - l0;
    report->elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    report->real_collisions = b.real_ - r0;
    report->null_collisions = b.null_ - n0;
    report->advance_ms = b.adv_ms_ - a0;
    report->electron_steps = b.electron_steps_ - s0;
    report->h2d_bytes = b.h2d_bytes_ - u0;
    report->d2h_bytes = b.d2h_bytes_ - d0;
    report->host_ms = b.host_ms_ - hm0;
    report->secondaries = b.secondaries_ - se0;
    report->spilled = b.spilled_ - sp0;
    report->attached = b.attached_ - at0;
    report->regrids = b.regrids_ - rg0;
    int th = 0, bl = 0, ch = 0, st = 0;
    lgpu::advance_shape(b.shape_, &th, &bl, &ch, &st);
    // a stash shape's collision turn always takes 32 collisions
    report->real_batch = b.tuned_ >= 0 ? (st ? 32 : lgpu::Batch::tune_threshold(b.tuned_)) : 0;
    report->coarse_null_test = b.tuned_ >= 0 ? lgpu::Batch::tune_coarse(b.tuned_) : -1;
    report->advance_threads = b.tune_stage_ >= 1 ? th : 0;
    report->advance_blocks_per_sm = b.tune_stage_ >= 1 ? bl : 0;
    report->advance_chunk = b.tune_stage_ >= 1 ? ch : 0;
    report->advance_stash = b.tune_stage_ >= 1 ? st : -1;
  }
  return rc;
}

int lgpu_batch_run(lgpu_batch* batch, lgpu_result* results, int* status, int n, lgpu_batch_report* report) {
  if (!batch || !batch->b) return LGPU_ERR_BAD_ARG;
  lgpu::Batch& b = *batch->b;
  if (n != (int)b.members_.size()) return b.fail(LGPU_ERR_BAD_ARG, "n must be the number of added contexts");
  const long long i0 = b.intervals_, l0 = b.launches_;
  const double a0 = b.adv_ms_, s0 = b.electron_steps_, u0 = b.h2d_bytes_, d0 = b.d2h_bytes_, hm0 = b.host_ms_,
               se0 = b.secondaries_, sp0 = b.spilled_, at0 = b.attached_, rg0 = b.regrids_;
  const auto t0 = std::chrono::steady_clock::now();
  int rc = b.run();
  const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  // a failed launch sequence ends every member that is still running
  for (auto& m : b.members_)
    if (!m.done) {
      if (m.started) m.e->sync("batch");
      m.status = rc != LGPU_OK ? rc : LGPU_ERR_STATE;
      m.done = true;
      m.e->leave_batch();
    }
  double real = 0, null = 0;
  for (int i = 0; i < n; ++i) {
    const auto& m = b.members_[i];
    if (results) results[i] = m.result;
    if (status) status[i] = m.status;
    real += m.result.real_collisions;
    null += m.result.null_collisions;
  }
  if (report) {
    report->intervals = b.intervals_ - i0;
    report->kernel_launches = b.launches_ - l0;
    report->elapsed = elapsed;
    report->real_collisions = real;
    report->null_collisions = null;
    report->advance_ms = b.adv_ms_ - a0;
    report->electron_steps = b.electron_steps_ - s0;
    report->h2d_bytes = b.h2d_bytes_ - u0;
    report->d2h_bytes = b.d2h_bytes_ - d0;
    report->host_ms = b.host_ms_ - hm0;
    report->secondaries = b.secondaries_ - se0;
    report->spilled = b.spilled_ - sp0;
    report->attached = b.attached_ - at0;
    report->regrids = b.regrids_ - rg0;
    int th = 0, bl = 0, ch = 0, st = 0;
    lgpu::advance_shape(b.shape_, &th, &bl, &ch, &st);
    // a stash shape's collision turn always takes 32 collisions
    report->real_batch = b.tuned_ >= 0 ? (st ? 32 : lgpu::Batch::tune_threshold(b.tuned_)) : 0;
    report->coarse_null_test = b.tuned_ >= 0 ? lgpu::Batch::tune_coarse(b.tuned_) : -1;
    report->advance_threads = b.tune_stage_ >= 1 ? th : 0;
    report->advance_blocks_per_sm = b.tune_stage_ >= 1 ? bl : 0;
    report->advance_chunk = b.tune_stage_ >= 1 ? ch : 0;
    report->advance_stash = b.tune_stage_ >= 1 ? st : -1;
  }
  b.clear_members();
  return rc;
}

}  // extern "C"
