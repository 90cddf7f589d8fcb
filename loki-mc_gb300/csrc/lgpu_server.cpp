// lgpu_server.cpp - continuous batching of swarm jobs (the lgpu_server_*
// entry points of include/loki_gpu.h).
//
// One device-owner thread runs a Batch without pause. Jobs wait in arrival
// order; the job at the head of the queue is admitted when a slot is free and
// its device footprint fits the memory budget (strict order, so a large job
// is never starved by small ones behind it). Admission creates the job's
// context (its own ensemble, tables and tallies) and starts its solve; every
// loop turn then advances all admitted jobs by one synchronisation interval in
// one launch sequence. A job whose own stop criteria hold leaves the batch:
// its results and per-process rates are copied to the host and its context is
// destroyed, which frees its device memory for the next admission. Requests
// that arrive while others are on the device join at the next interval.
//
// Host threads: any number of submitters/pollers (one mutex), one worker that
// owns every CUDA call.
#include <algorithm>
#include <array>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>

#include "lgpu_batch.h"

namespace lgpu {

struct JobRec {
  long long id = 0;
  lgpu_config cfg{};
  int n_procs = 0;
  std::vector<lgpu_process> procs;  // until admission (the context copies them)
  std::vector<std::vector<double>> raw_e, raw_v;
  std::vector<lgpu_gas> gases;
  double emax = 0;
  lgpu_conditions cond{};
  long long raw_points = 0;
  // status (guarded by the server mutex)
  int state = LGPU_JOB_QUEUED;
  int status = LGPU_OK;
  double t_submit = 0, t_start = 0, t_end = 0, footprint = 0;
  bool cancel = false;
  bool holds = false;  // its footprint counts against the budget
  std::string error;
  lgpu_result result{};
  std::vector<unsigned long long> counts;
  std::vector<double> rate;
  // two-term inputs (until admission) and the EEDF post-processing's results
  std::vector<lgpu_twoterm_process> twoterm;
  std::vector<std::array<std::vector<double>, 4>> twoterm_tabs;
  bool has_eedf = false;
  lgpu_eedf_params eedf{};
  std::vector<double> eedf_rate;
  // worker-only
  Engine* engine = nullptr;
  int member = -1;
};

class Server {
 public:
  std::string err_;
  int device_ = 0, max_slots_ = 1;
  double budget_ = 0, held_ = 0, peak_ = 0;
  Batch batch_;
  std::thread worker_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<long long> queue_;
  std::map<long long, std::shared_ptr<JobRec>> jobs_;  // a waiter keeps its record alive
  std::vector<JobRec*> running_;  // worker-only
  // finished jobs in the order they finished: their records (results, rates)
  // are kept until lgpu_server_forget or until more than kRetainFinished
  // finished jobs are held, when the oldest go first
  static constexpr size_t kRetainFinished = 1 << 16;
  std::deque<long long> finished_;
  long long running_count_ = 0;
  bool stop_ = false;
  long long next_id_ = 1;
  long long submitted_ = 0, completed_ = 0, failed_ = 0, intervals_ = 0;
  double real_ = 0, null_ = 0, busy_ = 0;
  std::chrono::steady_clock::time_point t0_ = std::chrono::steady_clock::now();

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count(); }

  int start(int device, int max_slots, double budget) {
    int rc = batch_.init(device, max_slots);
    if (rc != LGPU_OK) {
      err_ = batch_.err_;
      return rc;
    }
    device_ = device;
    max_slots_ = max_slots;
    if (budget <= 0) {
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        err_ = "cudaMemGetInfo failed";
        return LGPU_ERR_CUDA;
      }
      budget = 0.8 * (double)free_b;
    }
    budget_ = budget;
    t0_ = std::chrono::steady_clock::now();
    worker_ = std::thread([this] { loop(); });
    return LGPU_OK;
  }

  int submit(const lgpu_job& j, long long* id) {
    if (j.n_procs < 1 || j.n_procs > kMaxProcesses || j.n_gases < 1 || j.n_gases > kMaxGases || !j.procs || !j.gases)
      return LGPU_ERR_BAD_ARG;
    if (j.config.n_electrons < 1) return LGPU_ERR_BAD_ARG;
    auto r = std::make_shared<JobRec>();
    r->cfg = j.config;
    r->n_procs = j.n_procs;
    r->cfg.device = device_;
    r->procs.assign(j.procs, j.procs + j.n_procs);
    r->raw_e.resize(j.n_procs);
    r->raw_v.resize(j.n_procs);
    for (int p = 0; p < j.n_procs; ++p) {
      const lgpu_process& q = j.procs[p];
      if (!q.is_super && (q.raw_len < 2 || !q.raw_e || !q.raw_v)) return LGPU_ERR_BAD_ARG;
      if (!q.is_super) {
        r->raw_e[p].assign(q.raw_e, q.raw_e + q.raw_len);
        r->raw_v[p].assign(q.raw_v, q.raw_v + q.raw_len);
        r->raw_points += q.raw_len;
      }
      r->procs[p].raw_e = r->raw_e[p].data();
      r->procs[p].raw_v = r->raw_v[p].data();
    }
    r->gases.assign(j.gases, j.gases + j.n_gases);
    r->emax = j.emax_elastic;
    r->cond = j.conditions;
    if (j.twoterm) {
      r->twoterm.assign(j.twoterm, j.twoterm + j.n_procs);
      r->twoterm_tabs.resize(j.n_procs);
      for (int p = 0; p < j.n_procs; ++p) {
        lgpu_twoterm_process& t = r->twoterm[p];
        if (t.n_int < 2 || !t.int_e || !t.int_v || (t.n_mom && (!t.mom_e || !t.mom_v))) return LGPU_ERR_BAD_ARG;
        auto& tb = r->twoterm_tabs[p];
        tb[0].assign(t.int_e, t.int_e + t.n_int);
        tb[1].assign(t.int_v, t.int_v + t.n_int);
        if (t.n_mom) {
          tb[2].assign(t.mom_e, t.mom_e + t.n_mom);
          tb[3].assign(t.mom_v, t.mom_v + t.n_mom);
        }
        t.int_e = tb[0].data();
        t.int_v = tb[1].data();
        t.mom_e = t.n_mom ? tb[2].data() : nullptr;
        t.mom_v = t.n_mom ? tb[3].data() : nullptr;
      }
    }
    r->footprint = Engine::footprint_bytes(r->cfg, j.n_procs, r->raw_points);
    std::lock_guard<std::mutex> lock(mu_);
    if (stop_) return LGPU_ERR_STATE;
    r->id = next_id_++;
    r->t_submit = now();
    *id = r->id;
    queue_.push_back(r->id);
    jobs_[r->id] = std::move(r);
    ++submitted_;
    cv_work_.notify_one();
    return LGPU_OK;
  }

  void fill_status(const JobRec& r, lgpu_job_status* st) const {
    std::memset(st, 0, sizeof(*st));
    st->state = r.state;
    st->status = r.status;
    st->submit_time = r.t_submit;
    st->start_time = r.t_start;
    st->end_time = r.t_end;
    st->footprint_bytes = r.footprint;
    st->result = r.result;
    std::snprintf(st->error, sizeof(st->error), "%s", r.error.c_str());
  }

  static bool final_state(int s) { return s == LGPU_JOB_DONE || s == LGPU_JOB_FAILED || s == LGPU_JOB_CANCELLED; }

  int poll(long long id, lgpu_job_status* st) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return LGPU_ERR_BAD_ARG;
    fill_status(*it->second, st);
    return LGPU_OK;
  }

  int wait(long long id, double timeout_s, lgpu_job_status* st) {
    std::unique_lock<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return LGPU_ERR_BAD_ARG;
    const std::shared_ptr<JobRec> r = it->second;
    auto pred = [&] { return final_state(r->state); };
    if (timeout_s > 0) {
      if (!cv_done_.wait_for(lock, std::chrono::duration<double>(timeout_s), pred)) {
        if (st) fill_status(*r, st);
        return LGPU_ERR_TIMEOUT;
      }
    } else {
      cv_done_.wait(lock, pred);
    }
    if (st) fill_status(*r, st);
    return LGPU_OK;
  }

  int eedf_results(long long id, lgpu_eedf_params* out, double* rate, int n) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return LGPU_ERR_BAD_ARG;
    const JobRec& r = *it->second;
    if (r.state != LGPU_JOB_DONE || !r.has_eedf) return LGPU_ERR_STATE;
    if (rate && n != r.n_procs) return LGPU_ERR_BAD_ARG;
    if (out) *out = r.eedf;
    if (rate) std::copy(r.eedf_rate.begin(), r.eedf_rate.end(), rate);
    return LGPU_OK;
  }

  int rates(long long id, unsigned long long* counts, double* rate, int n) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return LGPU_ERR_BAD_ARG;
    const JobRec& r = *it->second;
    if (r.state != LGPU_JOB_DONE) return LGPU_ERR_STATE;
    if (n != r.n_procs) return LGPU_ERR_BAD_ARG;
    if (n != (int)r.rate.size()) return LGPU_ERR_BAD_ARG;
    for (int p = 0; p < n; ++p) {
      if (counts) counts[p] = r.counts[p];
      if (rate) rate[p] = r.rate[p];
    }
    return LGPU_OK;
  }

  int cancel(long long id) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return LGPU_ERR_BAD_ARG;
    JobRec& r = *it->second;
    if (r.state == LGPU_JOB_QUEUED) {
      queue_.erase(std::remove(queue_.begin(), queue_.end(), id), queue_.end());
      r.state = LGPU_JOB_CANCELLED;
      r.t_end = now();
      cv_done_.notify_all();
    } else if (r.state == LGPU_JOB_RUNNING) {
      r.cancel = true;
    }
    return LGPU_OK;
  }

  void report(lgpu_server_report* rep) {
    std::lock_guard<std::mutex> lock(mu_);
    std::memset(rep, 0, sizeof(*rep));
    rep->submitted = submitted_;
    rep->completed = completed_;
    rep->failed = failed_;
    rep->queued = (long long)queue_.size();
    rep->running = running_count_;
    rep->intervals = intervals_;
    rep->real_collisions = real_;
    rep->null_collisions = null_;
    rep->busy_seconds = busy_;
    rep->peak_footprint_bytes = peak_;
  }

  void stop() {
    {
      std::lock_guard<std::mutex> lock(mu_);
      stop_ = true;
      cv_work_.notify_all();
    }
    if (worker_.joinable()) worker_.join();
  }

  // ---------------------------------------------------------------- worker
  // (called with the mutex held) ends a job, frees its context
  // drops the record of a finished job (lgpu_server_forget)
  int forget(long long id) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return LGPU_ERR_BAD_ARG;
    if (!final_state(it->second->state)) return LGPU_ERR_STATE;
    jobs_.erase(it);
    finished_.erase(std::remove(finished_.begin(), finished_.end(), id), finished_.end());
    return LGPU_OK;
  }

  void retire(JobRec* r, int state, int status) {
    if (r->state == LGPU_JOB_RUNNING) --running_count_;
    finished_.push_back(r->id);
    while (finished_.size() > kRetainFinished) {
      jobs_.erase(finished_.front());
      finished_.pop_front();
    }
    r->state = state;
    r->status = status;
    r->t_end = now();
    if (r->holds) held_ -= r->footprint;
    r->holds = false;
    if (state == LGPU_JOB_DONE) {
      ++completed_;
      real_ += r->result.real_collisions;
      null_ += r->result.null_collisions;
    } else if (state == LGPU_JOB_FAILED) {
      ++failed_;
    }
    cv_done_.notify_all();
  }

  void destroy_engine(JobRec* r) {
    if (r->member >= 0) {
      batch_.release_member(r->member);
      batch_.compact();
      r->member = -1;
    }
    delete r->engine;
    r->engine = nullptr;
  }

  // creates the job's context and starts its solve (worker, without the mutex)
  int create(JobRec* r) {
    Engine* e = new (std::nothrow) Engine(r->cfg);
    if (!e) return LGPU_ERR_OOM;
    r->engine = e;
    int rc = e->init();
    if (rc == LGPU_OK) rc = e->set_processes(r->procs.data(), (int)r->procs.size(), r->gases.data(), (int)r->gases.size(), r->emax);
    if (rc == LGPU_OK) rc = e->set_conditions(r->cond);
    if (rc == LGPU_OK && !r->twoterm.empty()) rc = e->set_twoterm(r->twoterm.data(), (int)r->twoterm.size());
    if (rc == LGPU_OK) rc = batch_.add(e);
    if (rc != LGPU_OK) return rc;
    r->member = batch_.end_id() - 1;
    // the context holds its own copies of the inputs from here on
    std::vector<lgpu_process>().swap(r->procs);
    std::vector<std::vector<double>>().swap(r->raw_e);
    std::vector<std::vector<double>>().swap(r->raw_v);
    std::vector<lgpu_twoterm_process>().swap(r->twoterm);
    std::vector<std::array<std::vector<double>, 4>>().swap(r->twoterm_tabs);
    batch_.admit();
    const Batch::Member& m = batch_.member(r->member);
    if (m.done) return m.status == LGPU_OK ? LGPU_ERR_STATE : m.status;
    return LGPU_OK;
  }

  void loop() {
    cudaSetDevice(device_);
    auto busy_from = std::chrono::steady_clock::now();
    for (;;) {
      // ---- admissions, in arrival order
      std::vector<JobRec*> admit;
      {
        std::unique_lock<std::mutex> lock(mu_);
        cv_work_.wait(lock, [&] { return stop_ || !running_.empty() || !queue_.empty(); });
        if (stop_) break;
        while (!queue_.empty() && (int)(running_.size() + admit.size()) < max_slots_) {
          JobRec* r = jobs_[queue_.front()].get();
          if (held_ + r->footprint > budget_) {
            if (running_.empty() && admit.empty()) {  // can never fit
              queue_.pop_front();
              r->error = "device footprint above the server's memory budget";
              retire(r, LGPU_JOB_FAILED, LGPU_ERR_OOM);
              continue;
            }
            break;
          }
          queue_.pop_front();
          held_ += r->footprint;
          r->holds = true;
          peak_ = std::max(peak_, held_);
          r->state = LGPU_JOB_RUNNING;
          ++running_count_;
          r->t_start = now();
          admit.push_back(r);
        }
      }
      if (running_.empty() && !admit.empty()) busy_from = std::chrono::steady_clock::now();
      for (JobRec* r : admit) {
        const int rc = create(r);
        if (rc != LGPU_OK) {
          const std::string msg = r->engine ? r->engine->err_ : std::string("out of host memory");
          destroy_engine(r);
          std::lock_guard<std::mutex> lock(mu_);
          r->error = msg.empty() ? batch_.err_ : msg;
          retire(r, LGPU_JOB_FAILED, rc);
        } else {
          running_.push_back(r);
        }
      }
      // ---- cancellations between intervals
      {
        std::vector<JobRec*> cancelled;
        {
          std::lock_guard<std::mutex> lock(mu_);
          for (JobRec* r : running_)
            if (r->cancel) cancelled.push_back(r);
        }
        for (JobRec* r : cancelled) {
          batch_.stop_member(r->member, LGPU_ERR_STATE);
          destroy_engine(r);
          running_.erase(std::remove(running_.begin(), running_.end(), r), running_.end());
          std::lock_guard<std::mutex> lock(mu_);
          retire(r, LGPU_JOB_CANCELLED, LGPU_OK);
        }
      }
      if (running_.empty()) continue;
      // ---- one interval of every running job
      std::vector<int> finished;
      const int rc = batch_.step(&finished);
      if (rc != LGPU_OK) {
        // the launch sequence itself failed: every running job fails with it
        for (JobRec* r : running_) {
          batch_.stop_member(r->member, rc);
          destroy_engine(r);
          std::lock_guard<std::mutex> lock(mu_);
          retire(r, LGPU_JOB_FAILED, rc);
        }
        running_.clear();
        std::lock_guard<std::mutex> lock(mu_);
        err_ = batch_.err_;
        continue;
      }
      {
        std::lock_guard<std::mutex> lock(mu_);
        intervals_ = batch_.intervals_;
      }
      for (int idx : finished) {
        auto it = std::find_if(running_.begin(), running_.end(), [&](JobRec* r) { return r->member == idx; });
        if (it == running_.end()) continue;
        JobRec* r = *it;
        running_.erase(it);
        const Batch::Member& m = batch_.member(idx);
        int status = m.status;
        std::vector<unsigned long long> counts;
        std::vector<double> rate, eedf_rate;
        lgpu_eedf_params eedf{};
        bool has_eedf = false;
        if (status == LGPU_OK) {
          const int P = r->n_procs;
          counts.resize(P);
          rate.resize(P);
          status = r->engine->process_results(counts.data(), rate.data(), nullptr, nullptr, P);
          // the end-of-job post-processing of the EEDF, on the device
          if (status == LGPU_OK && r->engine->has_twoterm()) {
            eedf_rate.resize(P);
            status = r->engine->eedf_postprocess(nullptr, 0, 0.0, &eedf, eedf_rate.data(), P);
            has_eedf = status == LGPU_OK;
          }
        }
        const lgpu_result res = m.result;
        const std::string msg = status == LGPU_OK ? std::string() : r->engine->err_;
        destroy_engine(r);
        std::lock_guard<std::mutex> lock(mu_);
        r->error = msg;
        r->result = res;
        r->counts = std::move(counts);
        r->rate = std::move(rate);
        r->has_eedf = has_eedf;
        r->eedf = eedf;
        r->eedf_rate = std::move(eedf_rate);
        retire(r, status == LGPU_OK ? LGPU_JOB_DONE : LGPU_JOB_FAILED, status);
      }
      if (running_.empty()) {
        std::lock_guard<std::mutex> lock(mu_);
        busy_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - busy_from).count();
      }
    }
    // stopping: whatever is left is cancelled
    for (JobRec* r : running_) {
      batch_.stop_member(r->member, LGPU_ERR_STATE);
      destroy_engine(r);
      std::lock_guard<std::mutex> lock(mu_);
      retire(r, LGPU_JOB_CANCELLED, LGPU_OK);
    }
    running_.clear();
    std::lock_guard<std::mutex> lock(mu_);
    while (!queue_.empty()) {
      JobRec* r = jobs_[queue_.front()].get();
      queue_.pop_front();
      r->state = LGPU_JOB_CANCELLED;
      r->t_end = now();
    }
    cv_done_.notify_all();
  }
};

}  // namespace lgpu

struct lgpu_server {
  lgpu::Server* s;
};

extern "C" {

int lgpu_server_start(int device, int max_slots, double memory_budget_bytes, lgpu_server** out) {
  if (!out) return LGPU_ERR_BAD_ARG;
  *out = nullptr;
  lgpu::Server* s = new (std::nothrow) lgpu::Server();
  if (!s) return LGPU_ERR_OOM;
  lgpu_server* h = new (std::nothrow) lgpu_server{s};
  if (!h) {
    delete s;
    return LGPU_ERR_OOM;
  }
  *out = h;
  return s->start(device, max_slots, memory_budget_bytes);
}

int lgpu_server_submit(lgpu_server* server, const lgpu_job* job, long long* job_id) {
  if (!server || !server->s || !job || !job_id) return LGPU_ERR_BAD_ARG;
  return server->s->submit(*job, job_id);
}

int lgpu_server_poll(lgpu_server* server, long long job_id, lgpu_job_status* status) {
  if (!server || !server->s || !status) return LGPU_ERR_BAD_ARG;
  return server->s->poll(job_id, status);
}

int lgpu_server_wait(lgpu_server* server, long long job_id, double timeout_s, lgpu_job_status* status) {
  if (!server || !server->s) return LGPU_ERR_BAD_ARG;
  return server->s->wait(job_id, timeout_s, status);
}

int lgpu_server_job_rates(lgpu_server* server, long long job_id, unsigned long long* counts, double* rate, int n) {
  if (!server || !server->s) return LGPU_ERR_BAD_ARG;
  return server->s->rates(job_id, counts, rate, n);
}

int lgpu_server_job_eedf(lgpu_server* server, long long job_id, lgpu_eedf_params* params, double* rate, int n) {
  if (!server || !server->s) return LGPU_ERR_BAD_ARG;
  return server->s->eedf_results(job_id, params, rate, n);
}

int lgpu_server_cancel(lgpu_server* server, long long job_id) {
  if (!server || !server->s) return LGPU_ERR_BAD_ARG;
  return server->s->cancel(job_id);
}

int lgpu_server_forget(lgpu_server* server, long long job_id) {
  if (!server || !server->s) return LGPU_ERR_BAD_ARG;
  return server->s->forget(job_id);
}

int lgpu_server_report_get(lgpu_server* server, lgpu_server_report* report) {
  if (!server || !server->s || !report) return LGPU_ERR_BAD_ARG;
  server->s->report(report);
  return LGPU_OK;
}

int lgpu_server_last_error(const lgpu_server* server, char* buf, size_t size) {
  if (!server || !server->s) return 0;
  const std::string& e = server->s->err_;
  if (buf && size) std::snprintf(buf, size, "%s", e.c_str());
  return (int)e.size();
}

int lgpu_server_stop(lgpu_server* server) {
  if (!server) return LGPU_OK;
  if (server->s) {
    server->s->stop();
    delete server->s;
  }
  delete server;
  return LGPU_OK;
}

}  // extern "C"
