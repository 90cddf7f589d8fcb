// lgpu_engine.h - host runtime of the electron Monte Carlo backend.
//
// class Engine owns the device state of one swarm condition and drives the
// kernels through the reference's control flow: per synchronisation interval
// the trial-frequency check, one advance launch (ensemble and secondaries) and
// population control; per sample the ensemble moments, steady-state detection,
// error control and distribution tallies; at the end the time averages. The
// control flow and the FP64 bookkeeping restate Code/LoKI-MC/Sources/BoltzmannMC.C
// (line numbers cited per routine). The solve loop is split into steps
// (solve_begin / solve_next / interval_pre / interval_post / solve_end) so that
// the batched runtime (lgpu_batch.cpp) drives many engines through the same
// host logic while one set of launches advances all of them.
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cstddef>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/loki_gpu.h"
#include "lgpu_kernels.cuh"

namespace lgpu {

constexpr double kQeD = 1.6021766208e-19;  // Constant.h:7
constexpr double kMeD = 9.10938356e-31;    // Constant.h:8
constexpr double kKbD = 1.38064852e-23;    // Constant.h:6
constexpr double kNonDef = -123456789.0;   // Constant.h:23
constexpr double kPi = 3.14159265358979323846;

struct Kahan {
  double s = 0, c = 0;
  void add(double x) {
    double y = x - c;
    double t = s + y;
    c = (t - s) - y;
    s = t;
  }
};


// Batch-means error of the mean (MathFunctions.C:211-231).
inline double statistical_error(const double* a, long long n, double nbins) {
  if (n == 0) return 0;
  if (n < nbins) return NAN;
  long long np = (long long)(n / nbins);
  Kahan mean;
  for (long long i = 0; i < n; ++i) mean.add(a[i]);
  const double m = mean.s / n;
  double sum = 0;
  for (int b = 0; b < (int)nbins; ++b) {
    Kahan bm;
    for (long long i = 0; i < np; ++i) bm.add(a[b * np + i]);
    sum += std::pow(bm.s / np - m, 2);
  }
  return std::sqrt(sum) / nbins;
}

class Engine {
 public:
  explicit Engine(const lgpu_config& c) : cfg_(c) {}
  ~Engine() { release(); }

  std::string err_;
  lgpu_config cfg_;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;

  // ---------------------------------------------------------------- errors
  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err_ = buf;
    return code;
  }
  int cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LGPU_OK;
    if (e == cudaErrorMemoryAllocation) return fail(LGPU_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(LGPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
#define LGPU_TRY(expr)           \
  do {                           \
    int _rc = (expr);            \
    if (_rc != LGPU_OK) return _rc; \
  } while (0)
#define LGPU_CU(expr) LGPU_TRY(cuda((expr), #expr))

  template <class T>
  int dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cuda(cudaMalloc((void**)p, n * sizeof(T)), "cudaMalloc");
  }

  // Buffers carved from one allocation, each on a 256-byte boundary: a
  // context makes a handful of allocations instead of dozens (creating the
  // 64 contexts of a sweep took 0.36 ms each in allocation calls alone).
  struct Carve {
    size_t bytes = 0;
    template <class T>
    size_t take(size_t n) {
      const size_t o = (bytes + 255) & ~(size_t)255;
      bytes = o + std::max<size_t>(n, 1) * sizeof(T);
      return o;
    }
  };
  template <class T>
  static T* at(char* base, size_t off) {
    return reinterpret_cast<T*>(base + off);
  }

  // The secondary, spill and population-control buffers for `cap` records
  // in one allocation.
  struct SecondarySet {
    char* base = nullptr;
    int *alive = nullptr, *removed = nullptr, *pair_slot = nullptr, *pair_sec = nullptr;
    float4 *spill = nullptr, *sec = nullptr;
    unsigned int* claim = nullptr;
    size_t claim_words = 0;
  };
  cudaError_t alloc_secondaries(int cap, SecondarySet* o) const {
    Carve cv;
    const size_t words = ((size_t)N_ + cap + 31) / 32;
    const size_t a = cv.take<int>(cap), sp = cv.take<float4>(2 * (size_t)cap), se = cv.take<float4>(2 * (size_t)cap);
    const size_t cl = cv.take<unsigned int>(words), rm = cv.take<int>(cap), ps = cv.take<int>(cap);
    const size_t pc = cv.take<int>(cap);
    const cudaError_t e = cudaMalloc((void**)&o->base, cv.bytes);
    if (e != cudaSuccess) {
      o->base = nullptr;
      return e;
    }
    o->alive = at<int>(o->base, a);
    o->spill = at<float4>(o->base, sp);
    o->sec = at<float4>(o->base, se);
    o->claim = at<unsigned int>(o->base, cl);
    o->removed = at<int>(o->base, rm);
    o->pair_slot = at<int>(o->base, ps);
    o->pair_sec = at<int>(o->base, pc);
    o->claim_words = words;
    return cudaSuccess;
  }
  void use_secondaries(const SecondarySet& q) {
    d_secbuf_ = q.base;
    d_alive_ = q.alive;
    d_spill_ = q.spill;
    d_sec_ = q.sec;
    d_claim_ = q.claim;
    d_removed_ = q.removed;
    d_pair_slot_ = q.pair_slot;
    d_pair_sec_ = q.pair_sec;
    claim_words_ = q.claim_words;
  }

  int init() {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(LGPU_ERR_NO_DEVICE, "no CUDA device");
    if (cfg_.device < 0 || cfg_.device >= ndev) return fail(LGPU_ERR_BAD_ARG, "device %d out of range", cfg_.device);
    if (cfg_.n_electrons < 1 || cfg_.n_electrons > 2.0e9) return fail(LGPU_ERR_BAD_ARG, "nElectrons out of range");
    if (cfg_.n_interp < 2 || cfg_.n_interp > (1 << 24)) return fail(LGPU_ERR_BAD_ARG, "nInterpPoints out of range");
    if (cfg_.n_energy_cells < 1 || cfg_.n_energy_cells > 4096) return fail(LGPU_ERR_BAD_ARG, "nEnergyCells must be 1..4096");
    if (cfg_.sync_oversampling < 1) return fail(LGPU_ERR_BAD_ARG, "synchronizationOverSampling must be >= 1");
    if (cfg_.advance_real_batch < 0 || cfg_.advance_real_batch > 32)
      return fail(LGPU_ERR_BAD_ARG, "advance_real_batch must be 0..32");
    if (cfg_.advance_queue < 0 || cfg_.advance_queue > 32) return fail(LGPU_ERR_BAD_ARG, "advance_queue must be 0..32");
    LGPU_CU(cudaSetDevice(cfg_.device));
    LGPU_CU(prepare_kernels());
    LGPU_CU(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, cfg_.device));
    LGPU_CU(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    LGPU_CU(cudaEventCreate(&ev0_));
    LGPU_CU(cudaEventCreate(&ev1_));
    LGPU_CU(cudaEventCreateWithFlags(&tables_ev_, cudaEventDisableTiming));
    N_ = (int)cfg_.n_electrons;
    M_ = cfg_.n_interp;
    sec_cap_ = initial_sec_cap(cfg_);
    coarse_shift_ = 0;
    while (((M_ + (1 << coarse_shift_) - 1) >> coarse_shift_) > kMaxCoarse) ++coarse_shift_;
    n_coarse_ = (M_ + (1 << coarse_shift_) - 1) >> coarse_shift_;
    const int nEC = cfg_.n_energy_cells;
    // the fixed device buffers: ensemble, scalars, tables, tallies, constants
    Carve cv;
    const size_t o_state = cv.take<float4>(2 * (size_t)N_), o_att = cv.take<int>(N_);
    const size_t o_sc = cv.take<DevScalars>(1), o_ctl = cv.take<IntervalCtl>(1);
    const size_t o_nup = cv.take<float2>(M_), o_nut = cv.take<double>(M_), o_num = cv.take<double>(M_);
    const size_t o_nuc = cv.take<float>(kMaxCoarse);
    const size_t o_eedf = cv.take<double>(nEC);
    const size_t o_eper = cv.take<double>((size_t)std::max(cfg_.n_phases, 1) * nEC);
    const size_t o_eadf = cv.take<double>((size_t)nEC * std::max(cfg_.n_cos_cells, 1));
    const size_t o_evdf = cv.take<double>((size_t)std::max(cfg_.n_radial_cells, 1) * std::max(cfg_.n_axial_cells, 1));
    const size_t o_procf = cv.take<ProcF>(kMaxProcesses), o_gasf = cv.take<GasF>(kMaxGases);
    LGPU_TRY(dalloc(&d_core_, cv.bytes));
    d_state_ = at<float4>(d_core_, o_state);
    // the kernels move a record with one 32-byte access
    if (reinterpret_cast<uintptr_t>(d_state_) % 32 != 0) return fail(LGPU_ERR_CUDA, "ensemble not 32-byte aligned");
    d_att_ = at<int>(d_core_, o_att);
    d_sc_ = at<DevScalars>(d_core_, o_sc);
    d_ctl_ = at<IntervalCtl>(d_core_, o_ctl);
    d_nu_pair_ = at<float2>(d_core_, o_nup);
    d_nu_tot_ = at<double>(d_core_, o_nut);
    d_nu_max_ = at<double>(d_core_, o_num);
    d_nu_coarse_ = at<float>(d_core_, o_nuc);
    d_eedf_ = at<double>(d_core_, o_eedf);
    d_eedf_per_ = at<double>(d_core_, o_eper);
    d_eadf_ = at<double>(d_core_, o_eadf);
    d_evdf_ = at<double>(d_core_, o_evdf);
    d_procf_ = at<ProcF>(d_core_, o_procf);
    d_gasf_ = at<GasF>(d_core_, o_gasf);
    SecondarySet q;
    LGPU_CU(alloc_secondaries(sec_cap_, &q));
    use_secondaries(q);
    // pinned host: the scalar read-back, the control block, the running maximum
    Carve ch;
    const size_t o_hsc = ch.take<DevScalars>(1), o_hctl = ch.take<IntervalCtl>(1), o_hnum = ch.take<double>(M_);
    LGPU_CU(cudaMallocHost((void**)&h_pinned_, ch.bytes));
    h_sc_ = at<DevScalars>(h_pinned_, o_hsc);
    h_ctl_ = at<IntervalCtl>(h_pinned_, o_hctl);
    h_nu_max_ = at<double>(h_pinned_, o_hnum);
    std::memset(h_ctl_, 0, sizeof(IntervalCtl));
    std::memset(h_nu_max_, 0, (size_t)M_ * sizeof(double));
    LGPU_CU(cudaMemsetAsync(d_claim_, 0, claim_words_ * sizeof(unsigned int), stream_));
    LGPU_CU(cudaMemsetAsync(d_sc_, 0, sizeof(DevScalars), stream_));
    return sync("init");
  }

  void release() {
    if (batch_ && stream_) cudaStreamSynchronize(stream_);
    leave_batch();  // the batch's stream is not this context's to destroy
    if (stream_) cudaStreamSynchronize(stream_);
    drop_graphs();
    void* ptrs[] = {d_core_, d_secbuf_, d_procbuf_, d_rp_in_, d_rp_out_, d_tt_i_, d_tt_d_, d_tt_raw_, d_post_};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    d_core_ = d_secbuf_ = d_procbuf_ = nullptr;
    if (h_pinned_) cudaFreeHost(h_pinned_);
    h_pinned_ = nullptr;
    h_sc_ = nullptr;
    h_ctl_ = nullptr;
    h_nu_max_ = nullptr;
    if (tables_ev_) cudaEventDestroy(tables_ev_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (stream_) cudaStreamDestroy(stream_);
    stream_ = nullptr;
  }

  // every host<->device copy goes through here so the bytes are counted
  cudaError_t copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    if (kind == cudaMemcpyHostToDevice) h2d_bytes_ += (double)bytes;
    else if (kind == cudaMemcpyDeviceToHost) d2h_bytes_ += (double)bytes;
    return cudaMemcpyAsync(dst, src, bytes, kind, stream_);
  }

  int sync(const char* what) {
    LGPU_CU(cudaStreamSynchronize(stream_));
    return cuda(cudaGetLastError(), what);
  }

  // ------------------------------------------------------------ processes
  int set_processes(const lgpu_process* pr, int nP, const lgpu_gas* gs, int nG, double emax_el) {
    if (nP < 1 || nP > kMaxProcesses) return fail(LGPU_ERR_BAD_ARG, "process count %d outside 1..%d", nP, kMaxProcesses);
    if (nG < 1 || nG > kMaxGases) return fail(LGPU_ERR_BAD_ARG, "gas count %d outside 1..%d", nG, kMaxGases);
    std::vector<int> is_super(nP), raw_off(nP), raw_len(nP);
    std::vector<double> superw(nP), emin(nP), emax(nP), rel(nP), raw_e, raw_v;
    procs_.assign(pr, pr + nP);
    for (int p = 0; p < nP; ++p) {
      if (pr[p].is_super && (p == 0 || pr[p - 1].is_super))
        return fail(LGPU_ERR_BAD_ARG, "superelastic process %d must follow its inelastic partner", p);
      if (!pr[p].is_super && (pr[p].raw_len < 2 || !pr[p].raw_e || !pr[p].raw_v))
        return fail(LGPU_ERR_BAD_ARG, "process %d needs a raw cross section with >= 2 points", p);
      if (pr[p].type < 0 || pr[p].type > 2 || pr[p].sampler < 0 || pr[p].sampler > 5)
        return fail(LGPU_ERR_BAD_ARG, "process %d: bad type or sampler", p);
      is_super[p] = pr[p].is_super;
      superw[p] = pr[p].superw;
      emin[p] = pr[p].emin;
      emax[p] = pr[p].emax;
      rel[p] = pr[p].rel_dens;
      raw_off[p] = (int)raw_e.size();
      raw_len[p] = pr[p].is_super ? 0 : pr[p].raw_len;
      for (int k = 0; k < raw_len[p]; ++k) {
        raw_e.push_back(pr[p].raw_e[k]);
        raw_v.push_back(pr[p].raw_v[k]);
      }
    }
    for (int g = 0; g < nG; ++g) {
      if (gs[g].first < 0 || gs[g].last >= nP || gs[g].first > gs[g].last)
        return fail(LGPU_ERR_BAD_ARG, "gas %d: bad process range", g);
    }
    gases_.assign(gs, gs + nG);
    P_ = nP;
    emax_elastic_ = emax_el;
    // device copies: the process arrays in one allocation, uploaded with one copy
    stride_ = (nP + 1) & ~1;
    Carve cv;
    const size_t o_sup = cv.take<int>(nP), o_sw = cv.take<double>(nP), o_emin = cv.take<double>(nP);
    const size_t o_emax = cv.take<double>(nP), o_rel = cv.take<double>(nP), o_roff = cv.take<int>(nP);
    const size_t o_rlen = cv.take<int>(nP), o_re = cv.take<double>(raw_e.size()), o_rv = cv.take<double>(raw_v.size());
    const size_t uploaded = cv.bytes;
    const size_t o_cum = cv.take<float2>((size_t)M_ * stride_), o_sig = cv.take<float2>((size_t)M_ * stride_);
    const size_t o_gain = cv.take<double>(nP), o_loss = cv.take<double>(nP);
    const size_t o_cnt = cv.take<unsigned long long>(nP);
    std::vector<char> stage(uploaded, 0);
    auto put = [&](size_t off, const auto& h) {
      using T = typename std::remove_reference<decltype(h)>::type::value_type;
      if (!h.empty()) std::memcpy(stage.data() + off, h.data(), h.size() * sizeof(T));
    };
    put(o_sup, is_super);
    put(o_sw, superw);
    put(o_emin, emin);
    put(o_emax, emax);
    put(o_rel, rel);
    put(o_roff, raw_off);
    put(o_rlen, raw_len);
    put(o_re, raw_e);
    put(o_rv, raw_v);
    if (d_procbuf_) {
      LGPU_TRY(sync("set_processes"));  // nothing in flight still reads the old arrays
      cudaFree(d_procbuf_);
      d_procbuf_ = nullptr;
    }
    LGPU_TRY(dalloc(&d_procbuf_, cv.bytes));
    d_is_super_ = at<int>(d_procbuf_, o_sup);
    d_superw_ = at<double>(d_procbuf_, o_sw);
    d_emin_ = at<double>(d_procbuf_, o_emin);
    d_emax_ = at<double>(d_procbuf_, o_emax);
    d_rel_dens_ = at<double>(d_procbuf_, o_rel);
    d_raw_off_ = at<int>(d_procbuf_, o_roff);
    d_raw_len_ = at<int>(d_procbuf_, o_rlen);
    d_raw_e_ = at<double>(d_procbuf_, o_re);
    d_raw_v_ = at<double>(d_procbuf_, o_rv);
    d_cum_pair_ = at<float2>(d_procbuf_, o_cum);
    d_sig_pair_ = at<float2>(d_procbuf_, o_sig);
    d_proc_gain_ = at<double>(d_procbuf_, o_gain);
    d_proc_loss_ = at<double>(d_procbuf_, o_loss);
    d_proc_count_ = at<unsigned long long>(d_procbuf_, o_cnt);
    LGPU_CU(copy(d_procbuf_, stage.data(), uploaded, cudaMemcpyHostToDevice));
    have_ion_att_ = false;
    for (int p = 0; p < nP; ++p) have_ion_att_ |= (pr[p].type != kConservative);
    have_procs_ = true;
    max_interp_ = -1.0;
    return sync("set_processes");
  }

  // FP32 process/gas constants for the kernels (depend on Tg through the thermal spread)
  int upload_proc_consts() {
    std::vector<ProcF> pf(P_);
    for (int p = 0; p < P_; ++p) {
      const lgpu_process& q = procs_[p];
      const double M = q.mass, rm = kMeD * M / (kMeD + M);  // BoltzmannMC.C:168
      pf[p].type = q.type;
      pf[p].sampler = q.sampler;
      pf[p].sp0 = (float)q.sampler_p0;
      pf[p].sp1 = (float)q.sampler_p1;
      pf[p].eloss = (float)q.eloss;
      pf[p].mass = (float)M;
      pf[p].red_mass = (float)rm;
      pf[p].mass_factor = (float)(2.0 * rm / (kMeD + M));
      pf[p].wparam = (float)q.wparam;
      pf[p].pad = 0;
    }
    std::vector<GasF> gf(gases_.size());
    for (size_t g = 0; g < gases_.size(); ++g) {
      const lgpu_process& q = procs_[gases_[g].first];
      gf[g].first = gases_[g].first;
      gf[g].last = gases_[g].last;
      gf[g].fraction = (float)gases_[g].fraction;
      gf[g].thermal_sd = (float)std::sqrt(kKbD * Tg_ / q.mass);  // BoltzmannMC.C:170
      gf[g].red_mass = (float)(kMeD * q.mass / (kMeD + q.mass));
    }
    LGPU_CU(copy(d_procf_, pf.data(), pf.size() * sizeof(ProcF), cudaMemcpyHostToDevice));
    LGPU_CU(copy(d_gasf_, gf.data(), gf.size() * sizeof(GasF), cudaMemcpyHostToDevice));
    return LGPU_OK;
  }

  // ------------------------------------------------------------ conditions
  // BoltzmannMC.C:428-489 (field vector, AC sqrt(2), cyclotron frequency)
  int set_conditions(const lgpu_conditions& c) {
    if (!(c.gas_density > 0) || !(c.gas_temperature > 0)) return fail(LGPU_ERR_BAD_ARG, "gas density and temperature must be > 0");
    Ngas_ = c.gas_density;
    Tg_ = c.gas_temperature;
    gas_energy_ = 1.5 * kKbD * Tg_ / kQeD;
    red_field_ = c.reduced_field_td;
    angle_ = c.field_angle_deg;
    const double Ev = c.reduced_field_td * 1e-21 * Ngas_;  // WorkingConditions.h:81
    if (angle_ == 180) {
      E_[0] = 0;
      E_[1] = 0;
      E_[2] = -Ev;
    } else {
      E_[0] = Ev * std::sin(angle_ / 180.0 * kPi);
      E_[1] = 0;
      E_[2] = Ev * std::cos(angle_ / 180.0 * kPi);
    }
    freq_ = c.excitation_freq_hz;
    omega_ = freq_ * 2.0 * kPi;
    if (freq_ != 0)
      for (double& e : E_) e *= std::sqrt(2.0);
    red_mag_ = c.reduced_mag_field_hx;
    const double B = red_mag_ * 1e-27 * Ngas_;  // WorkingConditions.h:86
    omega_c_ = kQeD * B / kMeD;
    cylindrical_ = (angle_ == 180);  // WorkingConditions.h:164-172
    have_cond_ = true;
    return set_field_mode();
  }

  int set_field_raw(const double e[3], double fhz, double redmag, double wc) {
    E_[0] = e[0];
    E_[1] = e[1];
    E_[2] = e[2];
    freq_ = fhz;
    omega_ = fhz * 2.0 * kPi;
    red_mag_ = redmag;
    omega_c_ = wc;
    return set_field_mode();
  }

  int set_field_mode() {
    FieldF f{};
    const double a = -kQeD / kMeD;
    f.ax = (float)(a * E_[0]);
    f.ay = (float)(a * E_[1]);
    f.az = (float)(a * E_[2]);
    f.Ex = (float)E_[0];
    f.Ez = (float)E_[2];
    f.w = (float)omega_;
    f.W = (float)omega_c_;
    f.e_me = (float)(kQeD / kMeD);
    // branch selection of BoltzmannMC.C:811-897
    if (red_mag_ == 0) f.mode = (freq_ == 0) ? kFieldDC : kFieldAC;
    else if (freq_ == 0) f.mode = kFieldB;
    else if (std::abs(omega_ - omega_c_) / omega_ < 1E-6) f.mode = kFieldECR;
    else f.mode = kFieldACB;
    field_ = f;
    return LGPU_OK;
  }

  Consts consts() const {
    Consts c{};
    c.qe = (float)kQeD;
    c.me = (float)kMeD;
    c.inv_qe = (float)(1.0 / kQeD);
    c.half_me_over_e = (float)(0.5 * kMeD / kQeD);
    c.two_qe_over_me = (float)(2.0 * kQeD / kMeD);
    c.sharing = cfg_.sharing;
    c.sharing_factor = (float)(cfg_.sharing == 0 ? 0.5 : (cfg_.sharing == 1 ? 0.0 : 0.5));  // BoltzmannMC.h:263-276
    c.gas_temp = cfg_.gas_temperature_effect;
    c.smart_energy = (float)(20.0 * gas_energy_);
    c.G = (int)gases_.size();
    return c;
  }

  TablesF tables() const {
    TablesF t{};
    t.nu_pair = d_nu_pair_;
    t.cum_pair = d_cum_pair_;
    t.sig_pair = d_sig_pair_;
    t.M = M_;
    t.P = P_;
    t.stride = stride_;
    t.inv_step = (float)(1.0 / step_);
    t.inv_N = (float)(1.0 / Ngas_);
    t.nu_coarse = d_nu_coarse_;
    t.coarse_shift = coarse_shift_;
    t.n_coarse = n_coarse_;
    return t;
  }

  // ------------------------------------------------------------ tables
  // interpolateCrossSections (BoltzmannMC.C:561-615), on the device
  // With `async` (a context in a batch) the tables are built on the context's
  // own stream and the running maximum comes back into pinned memory behind
  // tables_ev_; the context sits out batched intervals until that event has
  // completed (settle_tables), so no batched launch reads half-built tables.
  int build_tables(double max_energy, double* sig64 = nullptr, double* cum64 = nullptr, bool async = false) {
    LGPU_TRY(settle_tables());
    if (max_energy == max_interp_) return LGPU_OK;
    max_interp_ = max_energy;
    step_ = max_energy / (double)(M_ - 1);
    TableBuildArgs a{};
    a.M = M_;
    a.P = P_;
    a.stride = stride_;
    a.step = step_;
    a.N = Ngas_;
    a.is_super = d_is_super_;
    a.superw = d_superw_;
    a.emin = d_emin_;
    a.emax = d_emax_;
    a.rel_dens = d_rel_dens_;
    a.raw_off = d_raw_off_;
    a.raw_len = d_raw_len_;
    a.raw_e = d_raw_e_;
    a.raw_v = d_raw_v_;
    a.nu_pair = d_nu_pair_;
    a.cum_pair = d_cum_pair_;
    a.sig_pair = d_sig_pair_;
    a.nu_tot = d_nu_tot_;
    a.nu_max = d_nu_max_;
    a.sig64 = sig64;
    a.cum64 = cum64;
    a.nu_coarse = d_nu_coarse_;
    a.coarse_shift = coarse_shift_;
    a.n_coarse = n_coarse_;
    cudaStream_t st = async && batch_ ? own_stream_ : stream_;
    launch_build_tables(a, st);
    launches_ += 3;
    d2h_bytes_ += (double)M_ * sizeof(double);
    LGPU_CU(cudaMemcpyAsync(h_nu_max_, d_nu_max_, M_ * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (async) {
      LGPU_CU(cudaEventRecord(tables_ev_, st));
      tables_inflight_ = true;
      return cuda(cudaGetLastError(), "build_tables");
    }
    LGPU_CU(cudaStreamSynchronize(st));
    return cuda(cudaGetLastError(), "build_tables");
  }

  // waits for tables built asynchronously (a no-op once they are done)
  int settle_tables() {
    if (!tables_inflight_) return LGPU_OK;
    tables_inflight_ = false;
    LGPU_CU(cudaEventSynchronize(tables_ev_));
    return cuda(cudaGetLastError(), "build_tables");
  }

  // maximizationAccelerationEnergy (BoltzmannMC.C:765-802)
  double max_accel_energy(double e0, double dt) const {
    const double e = kQeD, me = kMeD, e_me = e / me;
    const double Ex0 = std::abs(E_[0]), Ez0 = std::abs(E_[2]);
    const double Ex02 = Ex0 * Ex0, Ez02 = Ez0 * Ez0, E02 = Ex02 + Ez02, E0 = std::sqrt(E02);
    const double v0 = std::sqrt(e0 * e * 2.0 / me);
    const double w = omega_, W = omega_c_;
    double gain = (E0 * v0 + 0.5 * e_me * E02 * dt) * dt;
    if (W == 0) {
      if (w != 0) gain = std::fmin(gain, 2.0 / w * (e_me * E02 / w + v0 * (Ex0 + Ez0)));
    } else if (w == 0) {
      gain = std::fmin(gain, 0.5 * e_me * Ez02 * dt * dt + (2.0 * e_me * Ex02 / W + 3.0 * v0 * Ex0) / W + v0 * dt * Ez0);
    } else if (std::abs(w - W) / w < 1E-6) {
      const double W2 = W * W;
      gain = std::fmin(gain, 2.0 * e_me * Ez02 / W2 + e_me * Ex02 / (8.0 * W2) * (4.0 + W * dt * (2.0 + W * dt)) +
                                 (v0 * dt + v0 / W) * Ex0 + 2.0 * v0 * Ez0 / W);
    } else {
      const double w2 = w * w, W2 = W * W, d = w2 - W2;
      gain = std::fmin(gain, 2.0 * e_me * Ez02 / w2 + 0.5 * e_me * Ex02 / (d * d) * (5.0 * w2 + 8.0 * w * W + 5.0 * W * W) +
                                 3.0 * v0 * Ex0 / std::abs(w - W) + 2.0 * v0 * Ez0 / w);
    }
    return e0 + gain;
  }

  // checkMaxCollisionFrequency (BoltzmannMC.C:716-763)
  // With `ready` the check returns *ready = false after launching a table
  // re-grid asynchronously; calling it again once the tables are built
  // resumes it with the same decisions (max_interp_ now matches maxE).
  int check_max_frequency(double max_energy_before, bool* ready = nullptr) {
    LGPU_TRY(settle_tables());
    if (ready) *ready = true;
    const double thermal = (cfg_.gas_temperature_effect == 1 || cfg_.gas_temperature_effect == 2) ? 10.0 * gas_energy_ : 0.0;
    for (int it = 0; it < 100000; ++it) {
      const double maxE = max_accel_energy(max_energy_before, 10.0 / nu_trial_) + thermal;
      if (maxE > max_interp_ || 2.5 * maxE < max_interp_) {
        const double target = 2.0 * maxE < emax_elastic_ ? 2.0 * maxE : emax_elastic_;
        if (ready && target != max_interp_) {
          LGPU_TRY(build_tables(target, nullptr, nullptr, true));
          *ready = false;
          return LGPU_OK;
        }
        LGPU_TRY(build_tables(target));
      }
      const int idx = (int)std::fmin(std::ceil(maxE / step_), M_ - 1);
      if (nu_trial_ < h_nu_max_[idx]) {
        nu_trial_ *= 1.1;
        continue;
      }
      return LGPU_OK;
    }
    return fail(LGPU_ERR_OVERFLOW, "trial frequency search did not converge");
  }

  // ------------------------------------------------------------ ensemble
  int init_ensemble() {
    if (!have_procs_ || !have_cond_) return fail(LGPU_ERR_STATE, "set_processes and set_conditions come first");
    drop_graphs();  // kernel arguments (field, constants, sizes) may have changed
    hist_pending_ = false;
    LGPU_TRY(upload_proc_consts());
    time_ = 0;
    ss_time_ = kNonDef;
    interval_ = 0;
    origin_[0] = origin_[1] = origin_[2] = 0;
    shift_[0] = shift_[1] = shift_[2] = 0;
    LGPU_CU(cudaMemsetAsync(d_sc_, 0, sizeof(DevScalars), stream_));
    InitArgs ia{};
    ia.state = d_state_;
    ia.n = N_;
    ia.sd = (float)std::sqrt(kKbD * cfg_.init_temp_ratio * Tg_ / kMeD);  // BoltzmannMC.C:496
    ia.seed = cfg_.seed;
    ia.half_me_over_e = (float)(0.5 * kMeD / kQeD);
    ia.max_energy_bits = &d_sc_->max_energy_bits;
    launch_init(ia, stream_);
    ++launches_;
    LGPU_TRY(read_scalars());
    double maxE;
    {
      float f;
      std::memcpy(&f, &h_sc_->max_energy_bits, 4);
      maxE = f;
    }
    max_interp_ = -1.0;
    LGPU_TRY(build_tables(2.0 * maxE));  // BoltzmannMC.C:512
    nu_trial_ = h_nu_max_[M_ - 1];       // BoltzmannMC.C:515
    cur_max_energy_ = maxE;
    max_elec_energy_ = maxE;
    // tallies
    LGPU_CU(cudaMemsetAsync(d_proc_count_, 0, P_ * sizeof(unsigned long long), stream_));
    LGPU_CU(cudaMemsetAsync(d_proc_gain_, 0, P_ * sizeof(double), stream_));
    LGPU_CU(cudaMemsetAsync(d_proc_loss_, 0, P_ * sizeof(double), stream_));
    total_coll_ = null_coll_ = coll_at_ss_ = null_at_ss_ = 0;
    field_gain_ = growth_ = 0;
    base_proc_count_.assign(P_, 0);
    base_proc_gain_.assign(P_, 0.0);
    base_proc_loss_.assign(P_, 0.0);
    base_null_ = 0;
    base_field_gain_ = base_growth_ = base_time_adjust_ = 0;
    // series
    ts_.clear();
    me_.clear();
    mp_.clear();
    mv_.clear();
    fd_.clear();
    pc_.clear();
    bv_.clear();
    bd_.clear();
    n_samp_ = 1;
    n_sync_ = 1;
    n_int_ = 0;
    first_int_ = 0;
    total_int_time_ = 0;
    const int nPh = std::max(cfg_.n_phases, 1);
    phase_n_.assign(nPh, 0.0);
    phase_me_.assign(nPh, 0.0);
    phase_fv_.assign(3 * nPh, 0.0);
    phase_bv_.assign(3 * nPh, 0.0);
    phase_fd_.assign(9 * nPh, 0.0);
    phase_bd_.assign(9 * nPh, 0.0);
    max_eedf_ = 0;
    eedf_step_ = 0;
    initialized_ = true;
    status_ = LGPU_OK;
    // the first sample (BoltzmannMC.C:306-310)
    LGPU_TRY(sample_moments());
    return LGPU_OK;
  }

  int read_scalars() {
    LGPU_CU(copy(h_sc_, d_sc_, sizeof(DevScalars), cudaMemcpyDeviceToHost));
    return sync("read_scalars");
  }

  AdvanceArgs advance_args() const {
    AdvanceArgs a{};
    a.state = d_state_;
    a.n = N_;
    a.seed = cfg_.seed;
    a.field = field_;
    a.c = consts();
    a.t = tables();
    a.procs = d_procf_;
    a.gases = d_gasf_;
    a.P = P_;
    a.sec = d_sec_;
    a.sec_count = &d_sc_->sec_count;
    a.sec_cap = sec_cap_;
    a.spill = d_spill_;
    a.spill_count = &d_sc_->spill_count;
    a.spill_cap = sec_cap_;
    a.att_list = d_att_;
    a.att_count = &d_sc_->att_count;
    a.proc_count = d_proc_count_;
    a.proc_gain = d_proc_gain_;
    a.proc_loss = d_proc_loss_;
    a.null_count = &d_sc_->null_count;
    a.real_count = &d_sc_->real_count;
    a.field_gain = &d_sc_->field_gain;
    a.time_adjust = &d_sc_->time_adjust;
    a.max_energy_bits = &d_sc_->max_energy_bits;
    a.error_flag = &d_sc_->error_flag;
    a.work_counter = &d_sc_->work_counter;
    a.sm_count = sm_count_;
    a.ctl = d_ctl_;
    a.real_batch = cfg_.advance_real_batch > 0 ? std::min(cfg_.advance_real_batch, 32) : kDefaultRealBatch;
    a.coarse = 1;
    a.local_q = cfg_.advance_queue > 0 ? cfg_.advance_queue : 32;
    return a;
  }

  PopArgs pop_args() const {
    PopArgs p{};
    p.state = d_state_;
    p.n_electrons = N_;
    p.sec = d_sec_;
    p.sec_count = &d_sc_->sec_count;
    p.sec_cap = sec_cap_;
    p.counts = d_sc_->pop_counts;
    p.att_list = d_att_;
    p.att_count = &d_sc_->att_count;
    p.claim = d_claim_;
    p.alive = d_alive_;
    p.removed = d_removed_;
    p.pair_slot = d_pair_slot_;
    p.pair_sec = d_pair_sec_;
    p.growth = &d_sc_->growth;
    p.half_me_over_e = (float)(0.5 * kMeD / kQeD);
    p.seed = cfg_.seed;
    p.ctl = d_ctl_;
    p.error_flag = &d_sc_->error_flag;
    return p;
  }

  // The device work of one interval: the advance of every electron and of the
  // secondaries they create, the drain of any secondary left in the queue,
  // population control (when the mixture ionizes or attaches), the ensemble
  // sample and the scalar read-back. Captured once as a CUDA graph.
  void enqueue_interval(bool sample) {
    copy(d_ctl_, h_ctl_, sizeof(IntervalCtl), cudaMemcpyHostToDevice);
    cudaMemsetAsync(d_sc_, 0, offsetof(DevScalars, null_count), stream_);
    AdvanceArgs a = advance_args();
    cudaEventRecordWithFlags(ev0_, stream_, cudaEventRecordExternal);
    launch_advance(a, stream_);
    cudaEventRecordWithFlags(ev1_, stream_, cudaEventRecordExternal);
    ++launches_;
    if (have_ion_att_) {
      AdvanceArgs d = a;
      d.queue_only = 1;
      d.salt = 2;
      launch_advance(d, stream_);
      launch_pop_control(pop_args(), stream_);
      launches_ += 1 + kPopLaunches;
    }
    if (sample) enqueue_sample();
    copy(h_sc_, d_sc_, sizeof(DevScalars), cudaMemcpyDeviceToHost);
  }

  void enqueue_sample() {
    cudaMemsetAsync(d_sc_->moments, 0, sizeof(double) * kMoments, stream_);
    cudaMemsetAsync(&d_sc_->sample_max_bits, 0, sizeof(unsigned int), stream_);
    SampleArgs s{};
    s.state = d_state_;
    s.n = N_;
    s.half_me_over_e = (float)(0.5 * kMeD / kQeD);
    s.moments = d_sc_->moments;
    s.max_energy_bits = &d_sc_->sample_max_bits;
    launch_sample(s, sm_count_, stream_);
    ++launches_;
  }

  int graph_for(bool sample, cudaGraphExec_t* out) {
    cudaGraphExec_t& ge = graph_[sample ? 1 : 0];
    if (!ge) {
      cudaGraph_t g;
      const long long l0 = launches_;
      LGPU_CU(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
      enqueue_interval(sample);
      LGPU_CU(cudaStreamEndCapture(stream_, &g));
      LGPU_CU(cudaGraphInstantiate(&ge, g, 0));
      cudaGraphDestroy(g);
      graph_launches_[sample ? 1 : 0] = launches_ - l0;
      launches_ = l0;
      h2d_bytes_ -= sizeof(IntervalCtl);
      d2h_bytes_ -= sizeof(DevScalars);
    }
    *out = ge;
    return LGPU_OK;
  }

  void drop_graphs() {
    for (auto& g : graph_)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }

  // The first half of a synchronisation interval (BoltzmannMC.C:617-688):
  // the trial-frequency check and the interval's control block in h_ctl_.
  // In a batch (`ready` given) a table re-grid is launched asynchronously and
  // *ready = false: the context sits this batched interval out and calls
  // again at the next one.
  int interval_pre(bool* ready = nullptr) {
    LGPU_TRY(check_max_frequency(cur_max_energy_, ready));
    if (ready && !*ready) return LGPU_OK;
    pending_dt_ = cfg_.sync_x / nu_trial_;
    double phi0 = 0.0, rate = 0.0;
    if (field_.mode == kFieldAC || field_.mode == kFieldACB) {
      phi0 = std::fmod(omega_ * time_, 2.0 * kPi);
      rate = omega_;
    } else if (field_.mode == kFieldECR) {
      phi0 = std::fmod(omega_c_ * time_, 2.0 * kPi);
      rate = omega_c_;
    }
    IntervalCtl& c = *h_ctl_;
    c.dt_sync = (float)pending_dt_;
    c.phi0 = (float)phi0;
    c.phase_rate = (float)rate;
    c.nu = (float)nu_trial_;
    c.inv_step = (float)(1.0 / step_);
    c.shift_x = (float)shift_[0];
    c.shift_y = (float)shift_[1];
    c.shift_z = (float)shift_[2];
    c.interval = interval_;
    // in a batch the sample of this interval counts its EVDF in the moment
    // pass when it will record distributions (grid fixed since the steady state)
    evdf_fused_ = batch_ && sampling_ && ss_time_ != kNonDef && cylindrical_;
    return LGPU_OK;
  }

  // The second half, once the interval's device work is done and its scalars
  // are in h_sc_.
  int interval_post() {
    // the origin shift is now part of the stored offsets
    for (int k = 0; k < 3; ++k) {
      origin_[k] += (double)(float)shift_[k];
      shift_[k] = 0;
    }
    LGPU_TRY(check_device_errors());
    if (h_sc_->sec_count > sec_cap_)
      return fail(LGPU_ERR_OVERFLOW, "secondary buffer overflow (%d > %d)", h_sc_->sec_count, sec_cap_);
    // the reference's secondary list grows without bound; here the buffers
    // grow ahead of need: an interval that filled a quarter of them makes
    // them at least twice as large (and four times its own count) before
    // the next one, so a slowly heating, ionizing swarm never overflows
    if (h_sc_->sec_count > sec_cap_ / 4)
      LGPU_TRY(grow_secondaries(std::max(2 * (long long)sec_cap_, 4 * (long long)h_sc_->sec_count)));
    {
      float f;
      std::memcpy(&f, &h_sc_->max_energy_bits, 4);
      cur_max_energy_ = f;
    }
    time_ += pending_dt_;
    ++interval_;
    ++n_sync_;
    return LGPU_OK;
  }

  // Secondary records the buffers first hold: the ensemble's size, times one
  // per four trial collisions an electron makes in an interval (up to 8x);
  // they grow from there when a run needs more.
  static int initial_sec_cap(const lgpu_config& c) {
    const double base = std::max(c.n_electrons, 4096.0);
    const double per = std::min(8.0, std::max(1.0, std::ceil(c.sync_x / 4.0)));
    return (int)std::max(base, std::min(base * per, (double)(INT32_MAX / 2)));
  }

  // The secondary, spill and population-control buffers at `cap` records
  // (between intervals: nothing in flight uses them, and population control
  // leaves every claim bit clear). The new buffers are allocated before the
  // old ones go, so a failed allocation keeps the old capacity (an interval
  // that then overflows fails cleanly). Launch arguments built from the old
  // pointers (the interval graphs, a batch slot) are rebuilt.
  int grow_secondaries(long long cap) {
    const long long max_cap = std::min<long long>(INT32_MAX / 2, (long long)INT32_MAX - N_ - 32);
    if (sec_cap_ >= max_cap) return LGPU_OK;
    const int new_cap = (int)std::min<long long>(cap, max_cap);
    SecondarySet q;
    if (alloc_secondaries(new_cap, &q) != cudaSuccess) {
      cudaGetLastError();  // the failed allocation is not the next call's error
      return LGPU_OK;
    }
    LGPU_TRY(sync("grow"));
    cudaFree(d_secbuf_);
    use_secondaries(q);
    sec_cap_ = new_cap;
    LGPU_CU(cudaMemsetAsync(d_claim_, 0, claim_words_ * sizeof(unsigned int), stream_));
    drop_graphs();
    slot_built_ = -1;
    ++sec_grown_;
    return LGPU_OK;
  }

  // one synchronisation interval on this context's own stream; when `sample`,
  // the ensemble moments at its end are in h_sc_ afterwards
  int step_interval(bool sample) {
    if (batch_) return fail(LGPU_ERR_STATE, "the context is solved by a batch");
    LGPU_TRY(interval_pre());
    cudaGraphExec_t ge;
    LGPU_TRY(graph_for(sample, &ge));
    LGPU_CU(cudaGraphLaunch(ge, stream_));
    launches_ += graph_launches_[sample ? 1 : 0];
    h2d_bytes_ += sizeof(IntervalCtl);
    d2h_bytes_ += sizeof(DevScalars);
    LGPU_TRY(sync("interval"));
    {
      float ms = 0;
      LGPU_CU(cudaEventElapsedTime(&ms, ev0_, ev1_));
      adv_ms_ += ms;
      ++adv_launches_;
      adv_electron_steps_ += N_;
    }
    return interval_post();
  }

  int check_device_errors() {
    const int e = h_sc_->error_flag;
    if (e == 0) return LGPU_OK;
    if (e == 2) return fail(LGPU_ERR_OVERFLOW, "secondary or spill buffer full within one interval");
    if (e == 3) return fail(LGPU_ERR_OVERFLOW, "collision budget of one interval exhausted");
    if (e == 6) return fail(LGPU_ERR_STATE, "batched interval: chunk outside the ensemble");
    return fail(LGPU_ERR_OVERFLOW, "population control retry limit reached (code %d)", e);
  }

  // counters as the reference keeps them, from the device totals minus the
  // values at the steady-state reset (BoltzmannMC.C:1848-1856)
  // (the last scalar read-back is current: every launch sequence ends with one)
  int read_counters() {
    total_real_dev_ = h_sc_->real_count;
    total_null_dev_ = h_sc_->null_count;
    return LGPU_OK;
  }

  // ensemble moments at t = 0 (BoltzmannMC.C:306-310), outside the interval graph
  int sample_moments() {
    enqueue_sample();
    LGPU_TRY(read_scalars());
    return process_sample();
  }

  // calculateMeanDataForSwarmParams (BoltzmannMC.C:1410-1482) on the moment
  // sums of the last sample (h_sc_)
  int process_sample() {
    const double* S = h_sc_->moments;
    const double n = (double)N_;
    float fmax;
    std::memcpy(&fmax, &h_sc_->sample_max_bits, 4);
    cur_max_energy_ = fmax;
    max_elec_energy_ = std::fmax(max_elec_energy_, (double)fmax);
    if (max_elec_energy_ > emax_elastic_) {
      status_ = LGPU_ERR_ENERGY_ABOVE_TABLE;
      return fail(LGPU_ERR_ENERGY_ABOVE_TABLE,
                  "The energy of the electrons reached %f eV, while at least one of the elastic cross sections are "
                  "defined only until %f eV. Please reduce the electric field or change the cross sections.",
                  max_elec_energy_, emax_elastic_);
    }
    double mo[3], mv[3];
    for (int k = 0; k < 3; ++k) {
      mo[k] = S[1 + k] / n;
      mv[k] = S[4 + k] / n;
    }
    const double rr[9] = {S[7], S[8], S[9], S[8], S[10], S[11], S[9], S[11], S[12]};
    double pc[9], fd[9];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        pc[3 * a + b] = rr[3 * a + b] / n - mo[a] * mo[b];
        fd[3 * a + b] = S[13 + 3 * a + b] / n - mo[a] * mv[b];
      }
    const size_t cur = ts_.size();
    ts_.push_back(time_);
    me_.push_back(S[0] / n);
    for (int k = 0; k < 3; ++k) {
      mp_.push_back(origin_[k] + mo[k]);
      mv_.push_back(mv[k]);
    }
    for (int k = 0; k < 9; ++k) {
      pc_.push_back(pc[k]);
      fd_.push_back(fd[k]);
    }
    if (cur != 0) {
      const double dt = ts_[cur] - ts_[cur - 1];
      for (int k = 0; k < 3; ++k) bv_.push_back((mp_[3 * cur + k] - mp_[3 * (cur - 1) + k]) / dt);
      for (int k = 0; k < 9; ++k) bd_.push_back(0.5 * (pc_[9 * cur + k] - pc_[9 * (cur - 1) + k]) / dt);
    } else {
      for (int k = 0; k < 3; ++k) bv_.push_back(mv[k]);
      for (int k = 0; k < 9; ++k) bd_.push_back(fd[k]);
    }
    // AC phase bins after the steady state (BoltzmannMC.C:1468-1481)
    if (omega_ != 0 && ss_time_ != kNonDef) {
      const int nPh = cfg_.n_phases;
      const double ph = std::fmod(omega_ * time_, 2.0 * kPi);
      const int pi = (int)std::fmin(std::floor(ph / (2.0 * kPi / nPh)), nPh - 1);
      phase_n_[pi] += 1.0;
      phase_me_[pi] += me_[cur];
      for (int k = 0; k < 3; ++k) {
        phase_fv_[3 * pi + k] += mv_[3 * cur + k];
        phase_bv_[3 * pi + k] += bv_[3 * cur + k];
      }
      for (int k = 0; k < 9; ++k) {
        phase_fd_[9 * pi + k] += fd_[9 * cur + k];
        phase_bd_[9 * pi + k] += bd_[9 * cur + k];
      }
    }
    // recentre the FP32 position offsets on the ensemble mean: the next
    // advance subtracts this shift on load and the FP64 origin absorbs it
    for (int k = 0; k < 3; ++k) shift_[k] = (double)(float)mo[k];
    return LGPU_OK;
  }

  // EEDF grid update and remap of the accumulated tallies (BoltzmannMC.C:1495-1548)
  int rebin_distributions() {
    const int nEC = cfg_.n_energy_cells, nCos = cfg_.n_cos_cells, nPh = cfg_.n_phases;
    std::vector<double> eeh(nEC), eah((size_t)nEC * nCos), per((size_t)nPh * nEC);
    LGPU_CU(copy(eeh.data(), d_eedf_, eeh.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (cylindrical_)
      LGPU_CU(copy(eah.data(), d_eadf_, eah.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (omega_ != 0)
      LGPU_CU(copy(per.data(), d_eedf_per_, per.size() * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_TRY(sync("rebin read"));
    const double old_step = eedf_step_, old_max = max_eedf_;
    max_eedf_ = 1.2 * max_elec_energy_;
    eedf_step_ = max_eedf_ / nEC;
    std::vector<double> neeh(nEC, 0.0), neah((size_t)nEC * nCos, 0.0);
    // the periodic sums are not cleared before the remap and each old column
    // is added once per phase, as the reference does (BoltzmannMC.C:1523-1541)
    std::vector<double> nper = per;
    for (int o = 0; o < nEC; ++o) {
      const double lo = o * old_step, hi = (o + 1 == nEC) ? old_max : (o + 1) * old_step;
      const int nl = (int)(lo / eedf_step_), nr = (int)(hi / eedf_step_);
      const double lf = (nl == nr) ? 1.0 : (nr * eedf_step_ - lo) / old_step;
      neeh[nl] += lf * eeh[o];
      if (nl != nr) neeh[nr] += (1.0 - lf) * eeh[o];
      if (cylindrical_)
        for (int c = 0; c < nCos; ++c) {
          neah[(size_t)nl * nCos + c] += lf * eah[(size_t)o * nCos + c];
          if (nl != nr) neah[(size_t)nr * nCos + c] += (1.0 - lf) * eah[(size_t)o * nCos + c];
        }
      if (omega_ != 0)
        for (int rep = 0; rep < nPh; ++rep)
          for (int q = 0; q < nPh; ++q) {
            nper[(size_t)q * nEC + nl] += lf * per[(size_t)q * nEC + o];
            if (nl != nr) nper[(size_t)q * nEC + nr] += (1.0 - lf) * per[(size_t)q * nEC + o];
          }
    }
    LGPU_CU(copy(d_eedf_, neeh.data(), neeh.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (cylindrical_)
      LGPU_CU(copy(d_eadf_, neah.data(), neah.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (omega_ != 0)
      LGPU_CU(copy(d_eedf_per_, nper.data(), nper.size() * sizeof(double), cudaMemcpyHostToDevice));
    return sync("rebin write");
  }

  // getTimeDependDistributions (BoltzmannMC.C:1492-1572)
  int sample_distributions() {
    if (max_elec_energy_ > max_eedf_) LGPU_TRY(rebin_distributions());
    HistArgs h{};
    h.state = d_state_;
    h.n = N_;
    h.half_me_over_e = (float)(0.5 * kMeD / kQeD);
    h.n_e_cells = cfg_.n_energy_cells;
    h.inv_e_step = (float)(1.0 / eedf_step_);
    h.eedf = d_eedf_;
    h.eedf_periodic_row = nullptr;
    if (omega_ != 0) {
      const int nPh = cfg_.n_phases;
      const double ph = std::fmod(omega_ * time_, 2.0 * kPi);
      const int pi = (int)std::fmin(std::floor(ph / (2.0 * kPi / nPh)), nPh - 1);
      h.eedf_periodic_row = d_eedf_per_ + (size_t)pi * cfg_.n_energy_cells;
    }
    h.cylindrical = cylindrical_ ? 1 : 0;
    h.n_cos = cfg_.n_cos_cells;
    h.eadf = d_eadf_;
    h.n_rad = cfg_.n_radial_cells;
    h.n_ax = cfg_.n_axial_cells;
    h.inv_rad_step = (float)(1.0 / rad_step_);
    h.inv_ax_step = (float)(1.0 / ax_step_);
    h.max_speed = (float)max_speed_;
    h.evdf = d_evdf_;
    h.evdf_done = evdf_fused_ ? 1 : 0;
    evdf_fused_ = false;
    if (batch_) {
      pending_hist_ = h;
      hist_pending_ = true;
      return LGPU_OK;
    }
    launch_hist(h, stream_);
    launches_ += h.cylindrical ? 2 : 1;
    return LGPU_OK;
  }

  // checkSteadyState (BoltzmannMC.C:1787-1893)
  int check_steady_state() {
    const double t1 = 0.5 * time_, t2 = 0.75 * time_;
    double a1 = 0, a2 = 0, rs = 0;
    int n1 = 0, n2 = 0;
    for (size_t i = 0; i < ts_.size(); ++i) {
      const double st = ts_[i];
      if (st >= t1 && st <= t2) {
        a1 += me_[i];
        ++n1;
      } else if (st > t2) {
        a2 += me_[i];
        rs += me_[i] * me_[i];
        ++n2;
      }
    }
    a1 /= n1;
    a2 /= n2;
    rs = std::sqrt((rs / n2 - a2 * a2) / n2);
    LGPU_TRY(read_counters());
    if (!((a1 >= a2 && rs < 0.01) || (double)total_real_dev_ >= cfg_.max_coll_before_ss * N_)) return LGPU_OK;
    first_int_ = (long long)ts_.size() - 1;
    n_int_ = 1;
    ss_time_ = time_;
    coll_at_ss_ = total_real_dev_;
    null_at_ss_ = total_null_dev_;
    // reset of the integrated tallies: remember the device totals at this point
    {
      std::vector<unsigned long long> cnt(P_);
      LGPU_CU(copy(cnt.data(), d_proc_count_, P_ * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
      LGPU_CU(copy(base_proc_gain_.data(), d_proc_gain_, P_ * sizeof(double), cudaMemcpyDeviceToHost));
      LGPU_CU(copy(base_proc_loss_.data(), d_proc_loss_, P_ * sizeof(double), cudaMemcpyDeviceToHost));
      LGPU_TRY(sync("ss reset"));
      base_proc_count_ = cnt;
      base_field_gain_ = h_sc_->field_gain;
      base_growth_ = h_sc_->growth;
      base_time_adjust_ = h_sc_->time_adjust;
    }
    total_int_time_ = 0;
    // distribution grids (BoltzmannMC.C:1862-1889)
    max_eedf_ = 1.2 * max_elec_energy_;
    eedf_step_ = max_eedf_ / cfg_.n_energy_cells;
    max_speed_ = std::sqrt(2.0 * max_eedf_ * kQeD / kMeD);
    rad_step_ = max_speed_ / cfg_.n_radial_cells;
    ax_step_ = 2.0 * max_speed_ / cfg_.n_axial_cells;
    LGPU_CU(cudaMemsetAsync(d_eedf_, 0, cfg_.n_energy_cells * sizeof(double), stream_));
    LGPU_CU(cudaMemsetAsync(d_eadf_, 0, (size_t)cfg_.n_energy_cells * cfg_.n_cos_cells * sizeof(double), stream_));
    LGPU_CU(cudaMemsetAsync(d_evdf_, 0, (size_t)cfg_.n_radial_cells * cfg_.n_axial_cells * sizeof(double), stream_));
    LGPU_CU(cudaMemsetAsync(d_eedf_per_, 0, (size_t)std::max(cfg_.n_phases, 1) * cfg_.n_energy_cells * sizeof(double), stream_));
    return sample_distributions();
  }

  void col_stats(const std::vector<double>& d, int ncol, long long first, long long n, double* mean, double* err) const {
    std::vector<double> col((size_t)std::max<long long>(n, 1));
    for (int c = 0; c < ncol; ++c) {
      Kahan m;
      for (long long i = 0; i < n; ++i) {
        col[i] = d[(size_t)(first + i) * ncol + c];
        m.add(col[i]);
      }
      mean[c] = n ? m.s / n : NAN;
      err[c] = statistical_error(col.data(), n, 50);
    }
  }

  // Electron-time simulated since the steady state (s). The reference divides
  // by nElectrons x totalIntegratedTime (BoltzmannMC.C:1632, 1643-1648); here
  // secondaries are pushed from their creation time and attached electrons
  // stop at attachment, so the exact electron-time of the simulation is
  // N x time plus the time secondaries added minus the time attachments removed.
  double electron_time() const {
    return (double)N_ * total_int_time_ + (h_sc_->time_adjust - base_time_adjust_);
  }

  // power sums since the steady state (device totals minus the reset values)
  void power_sums(double* field, double* growth, std::vector<double>* gain, std::vector<double>* loss) {
    std::vector<double> g(P_), l(P_);
    copy(g.data(), d_proc_gain_, P_ * sizeof(double), cudaMemcpyDeviceToHost);
    copy(l.data(), d_proc_loss_, P_ * sizeof(double), cudaMemcpyDeviceToHost);
    cudaStreamSynchronize(stream_);
    for (int p = 0; p < P_; ++p) {
      g[p] -= base_proc_gain_[p];
      l[p] -= base_proc_loss_[p];
    }
    *field = h_sc_->field_gain - base_field_gain_;
    *growth = h_sc_->growth - base_growth_;
    if (gain) *gain = g;
    if (loss) *loss = l;
  }

  // checkPowerBalance (BoltzmannMC.C:1769-1785)
  double power_balance() {
    double field, growth;
    std::vector<double> g, l;
    power_sums(&field, &growth, &g, &l);
    double tg = field, tl = 0;
    if (growth > 0) tg += growth; else tl += growth;
    for (int p = 0; p < P_; ++p) {
      tg += g[p];
      tl += l[p];
    }
    return std::abs(tg + tl) / tg;
  }

  // checkStatisticalErrors (BoltzmannMC.C:1743-1767)
  bool statistical_errors_ok() {
    double m, e1, fv[3], fve[3], fdm[9], fde[9], bvm[3], bve[3], bdm[9], bde[9];
    col_stats(me_, 1, first_int_, n_int_, &m, &e1);
    col_stats(mv_, 3, first_int_, n_int_, fv, fve);
    col_stats(fd_, 9, first_int_, n_int_, fdm, fde);
    col_stats(bv_, 3, first_int_, n_int_, bvm, bve);
    col_stats(bd_, 9, first_int_, n_int_, bdm, bde);
    pb_rel_err_ = power_balance();
    auto sq = [](const double* v) { return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]; };
    const double rf = (std::abs(fv[0]) * fve[0] + std::abs(fv[1]) * fve[1] + std::abs(fv[2]) * fve[2]) / sq(fv);
    const double rb = (std::abs(bvm[0]) * bve[0] + std::abs(bvm[1]) * bve[1] + std::abs(bvm[2]) * bve[2]) / sq(bvm);
    return e1 / m <= cfg_.req_err_mean_energy && rf <= cfg_.req_err_flux_v && fde[0] / fdm[0] <= cfg_.req_err_flux_d &&
           fde[4] / fdm[4] <= cfg_.req_err_flux_d && fde[8] / fdm[8] <= cfg_.req_err_flux_d && rb <= cfg_.req_err_bulk_v &&
           bde[0] / bdm[0] <= cfg_.req_err_bulk_d && bde[4] / bdm[4] <= cfg_.req_err_bulk_d &&
           bde[8] / bdm[8] <= cfg_.req_err_bulk_d && pb_rel_err_ <= cfg_.req_err_power;
  }

  // ---------------------------------------------------------- solve steps
  // evaluateEEDF (BoltzmannMC.C:299-426) as steps: solve_begin, then per
  // interval solve_next (the loop condition and the caps), interval_pre, the
  // device work, interval_post and solve_post (sampling, steady state, error
  // control), and solve_end. solve() runs them on this context's stream; the
  // batched runtime runs the same steps for many contexts around one launch
  // sequence per interval.
  int solve_begin() {
    solve_t0_ = std::chrono::steady_clock::now();
    ++solve_serial_;
    LGPU_TRY(init_ensemble());
    solve_good_ = false;
    solve_capped_ = 0;
    solve_steps_ = 0;
    return LGPU_OK;
  }

  // *done when a stop criterion holds (BoltzmannMC.C:311-316) or a cap is hit;
  // otherwise sampling_ says whether the next interval ends with a sample
  int solve_next(bool* done) {
    *done = false;
    if (!((!solve_good_ && cfg_.errors_checked) || n_int_ < cfg_.req_integration_points ||
          total_int_time_ / ss_time_ < cfg_.req_ss_times || total_int_time_ < cfg_.req_abs_time)) {
      *done = true;
      return LGPU_OK;
    }
    if (ss_time_ != kNonDef && n_int_ > 100) {
      LGPU_TRY(read_counters());
      if ((double)(total_real_dev_ - coll_at_ss_) >= cfg_.max_coll_after_ss * N_) {
        *done = true;
        return LGPU_OK;
      }
    }
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - solve_t0_).count();
    if ((cfg_.max_seconds > 0 && el > cfg_.max_seconds) || (cfg_.max_sync_steps > 0 && solve_steps_ >= cfg_.max_sync_steps)) {
      solve_capped_ = 1;
      *done = true;
      return LGPU_OK;
    }
    sampling_ = (n_sync_ + 1) % cfg_.sync_oversampling == 0;
    return LGPU_OK;
  }

  // after an interval: the sample, steady-state and error checks of
  // BoltzmannMC.C:317-420
  int solve_post() {
    ++solve_steps_;
    if (!sampling_) return LGPU_OK;
    ++n_samp_;
    LGPU_TRY(process_sample());
    int dec = (int)std::fmax(std::log((double)n_samp_) / std::log(2.0) - 11, 6);
    const long long between_ss = (long long)std::pow(2, dec);
    if (ss_time_ != kNonDef) {
      ++n_int_;
      total_int_time_ = time_ - ss_time_;
      LGPU_TRY(sample_distributions());
    } else if (n_samp_ >= 100 && n_samp_ % between_ss == 0) {
      LGPU_TRY(read_counters());
      if ((double)total_real_dev_ > cfg_.min_coll_before_ss * N_) LGPU_TRY(check_steady_state());
    }
    dec = (int)std::fmax(std::log((double)n_int_) / std::log(2.0) - 9, 7);
    const long long between_err = (long long)std::pow(2, dec);
    if (ss_time_ != kNonDef && n_int_ > 200 && n_int_ % between_err == 0 && cfg_.errors_checked)
      solve_good_ = statistical_errors_ok();
    return LGPU_OK;
  }

  int solve_end(lgpu_result* r) {
    LGPU_TRY(flush_pending_hist());
    LGPU_TRY(sync("solve"));
    total_int_time_ = time_ - ss_time_;
    LGPU_TRY(read_counters());
    finals(r);
    r->capped = solve_capped_;
    r->sync_steps = solve_steps_;
    r->elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - solve_t0_).count();
    solved_ = true;
    return LGPU_OK;
  }

  int solve(lgpu_result* r) {
    if (batch_) return fail(LGPU_ERR_STATE, "the context is solved by a batch");
    LGPU_TRY(solve_begin());
    for (;;) {
      bool done = false;
      LGPU_TRY(solve_next(&done));
      if (done) break;
      LGPU_TRY(step_interval(sampling_));
      LGPU_TRY(solve_post());
    }
    return solve_end(r);
  }

  // ---------------------------------------------------------- batch mode
  // While a batch solves this context, its work goes on the batch's stream
  // and the distribution tallies of a sample run inside the batch's next
  // launch sequence (before that interval's advance, as they would here).
  void enter_batch(cudaStream_t s) {
    own_stream_ = stream_;
    stream_ = s;
    batch_ = true;
    hist_pending_ = false;
  }
  void leave_batch() {
    if (!batch_) return;
    stream_ = own_stream_;
    batch_ = false;
  }
  // launches a deferred tally (a context leaving the batch)
  int flush_pending_hist() {
    if (!hist_pending_) return LGPU_OK;
    hist_pending_ = false;
    launch_hist(pending_hist_, stream_);
    launches_ += pending_hist_.cylindrical ? 2 : 1;
    return LGPU_OK;
  }
  SampleArgs sample_args() const {
    SampleArgs s{};
    s.state = d_state_;
    s.n = N_;
    s.half_me_over_e = (float)(0.5 * kMeD / kQeD);
    s.moments = d_sc_->moments;
    s.max_energy_bits = &d_sc_->sample_max_bits;
    return s;
  }
  // this context's slot of the next batched interval (after interval_pre);
  // the argument blocks are fixed once the ensemble starts, so they are
  // built once per solve and only the control block and flags change
  void fill_slot(BatchSlot* sl) {
    if (slot_built_ != solve_serial_) {
      std::memset(&slot_, 0, sizeof(slot_));
      slot_.adv = advance_args();
      slot_.pop = pop_args();
      slot_.smp = sample_args();
      slot_.ctl_dst = d_ctl_;
      slot_.sc = d_sc_;
      slot_built_ = solve_serial_;
    }
    std::memcpy(sl, &slot_, sizeof(*sl));
    sl->ctl = *h_ctl_;
    sl->flags = (have_ion_att_ ? kSlotIonAtt : 0) | (sampling_ ? kSlotSample : 0);
    if (evdf_fused_) {
      sl->flags |= kSlotEvdf;
      HistArgs& v = sl->vhist;
      v.n_rad = cfg_.n_radial_cells;
      v.n_ax = cfg_.n_axial_cells;
      v.inv_rad_step = (float)(1.0 / rad_step_);
      v.inv_ax_step = (float)(1.0 / ax_step_);
      v.max_speed = (float)max_speed_;
      v.evdf = d_evdf_;
      v.cylindrical = 1;
    }
  }
  // the deferred tallies of the last sample, handed to the batch's
  // distribution passes (false when there are none)
  bool take_pending_hist(HistArgs* h) {
    if (!hist_pending_) return false;
    *h = pending_hist_;
    hist_pending_ = false;
    return true;
  }
  int field_mode() const { return field_.mode; }

  // Device memory a context with this configuration and process count holds
  // (bytes): ensemble and secondary buffers, population-control scratch,
  // tables, tallies and histograms, as init() and set_processes() allocate.
  static double footprint_bytes(const lgpu_config& c, int P, long long raw_points) {
    const double N = c.n_electrons, cap = initial_sec_cap(c), M = c.n_interp;
    const double stride = (double)((P + 1) & ~1);
    double b = N * 2 * sizeof(float4);                      // state
    b += cap * (sizeof(int) * 4 + 4 * sizeof(float4));      // alive, removed, pair_slot/sec; spill, sec
    b += N * sizeof(int) + (N + cap) / 8.0;                 // attached list, claim bitmap
    b += M * (sizeof(float2) + 2 * sizeof(double));         // nu pairs, nu_tot, nu_max
    b += 2.0 * M * stride * sizeof(float2);                 // cumulative and sigma row pairs
    b += P * (3 * sizeof(double) + 64) + (double)raw_points * 2 * sizeof(double);
    const double nEC = c.n_energy_cells;
    b += sizeof(double) * nEC * (1.0 + std::max(c.n_phases, 1) + std::max(c.n_cos_cells, 1));
    b += sizeof(double) * (double)std::max(c.n_radial_cells, 1) * std::max(c.n_axial_cells, 1);
    b += kMaxProcesses * sizeof(ProcF) + kMaxGases * sizeof(GasF) + 4096;
    return b;
  }
  int n_electrons() const { return N_; }

  void finals(lgpu_result* r) {
    std::memset(r, 0, sizeof(*r));
    if (n_int_ > 0) {
      col_stats(me_, 1, first_int_, n_int_, &r->mean_energy, &r->mean_energy_err);
      col_stats(mv_, 3, first_int_, n_int_, r->flux_v, r->flux_v_err);
      col_stats(fd_, 9, first_int_, n_int_, r->flux_d, r->flux_d_err);
      col_stats(bv_, 3, first_int_, n_int_, r->bulk_v, r->bulk_v_err);
      col_stats(bd_, 9, first_int_, n_int_, r->bulk_d, r->bulk_d_err);
    }
    double field, growth;
    power_sums(&field, &growth, nullptr, nullptr);
    const double denom = electron_time() * Ngas_;
    r->power_field = field / denom;
    r->power_growth = growth / denom;
    r->power_balance_rel_err = power_balance();
    r->ss_time = ss_time_;
    r->final_time = time_;
    r->trial_freq = nu_trial_;
    r->max_eedf_energy = max_eedf_;
    r->real_collisions = (double)total_real_dev_;
    r->null_collisions = (double)total_null_dev_;
    r->coll_at_ss = (double)coll_at_ss_;
    r->null_at_ss = (double)null_at_ss_;
    r->integration_points = n_int_;
    r->sampling_points = (long long)ts_.size();
    r->first_integration_index = first_int_;
  }

  int process_results(unsigned long long* counts, double* rate, double* gain, double* loss, int n) {
    if (n != P_) return fail(LGPU_ERR_BAD_ARG, "expected %d processes", P_);
    std::vector<unsigned long long> cnt(P_);
    std::vector<double> g(P_), l(P_);
    LGPU_CU(copy(cnt.data(), d_proc_count_, P_ * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    LGPU_CU(copy(g.data(), d_proc_gain_, P_ * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_CU(copy(l.data(), d_proc_loss_, P_ * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_TRY(sync("process_results"));
    const double etime = electron_time();
    for (int p = 0; p < P_; ++p) {
      const double c = (double)(cnt[p] - base_proc_count_[p]);
      if (counts) counts[p] = cnt[p] - base_proc_count_[p];
      // BoltzmannMC.C:1630-1637, over the simulated electron-time
      if (rate) rate[p] = procs_[p].rel_dens != 0 ? c / (etime * procs_[p].rel_dens * Ngas_) : 0.0;
      const double denom = etime * Ngas_;
      if (gain) gain[p] = (g[p] - base_proc_gain_[p]) / denom;
      if (loss) loss[p] = (l[p] - base_proc_loss_[p]) / denom;
    }
    return LGPU_OK;
  }

  // getTimeAverageDistributions + getAveragedPeriodicParams (BoltzmannMC.C:1574-1605, 1728-1741)
  int distributions(double* cells, double* eedf, double* efadf, double* esadf, double* eadf, double* evdf,
                    double* rcells, double* acells, double* eedf_per) {
    const int nEC = cfg_.n_energy_cells, nCos = cfg_.n_cos_cells, nR = cfg_.n_radial_cells, nA = cfg_.n_axial_cells;
    const int nPh = cfg_.n_phases;
    std::vector<double> eeh(nEC), eah((size_t)nEC * nCos), evh((size_t)nR * nA), per((size_t)std::max(nPh, 1) * nEC);
    LGPU_CU(copy(eeh.data(), d_eedf_, eeh.size() * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_CU(copy(eah.data(), d_eadf_, eah.size() * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_CU(copy(evh.data(), d_evdf_, evh.size() * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_CU(copy(per.data(), d_eedf_per_, per.size() * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_TRY(sync("distributions"));
    double norm = 0;
    for (double h : eeh) norm += h;
    std::vector<double> ecell(nEC);
    for (int c = 0; c < nEC; ++c) ecell[c] = eedf_step_ / 2.0 + c * eedf_step_;
    if (cells) std::copy(ecell.begin(), ecell.end(), cells);
    if (eedf)
      for (int c = 0; c < nEC; ++c) eedf[c] = eeh[c] / (std::sqrt(ecell[c]) * norm * eedf_step_);
    const double cstep = 2.0 / nCos;
    std::vector<double> ead((size_t)nEC * nCos, 0.0);
    if (cylindrical_) {
      for (int c = 0; c < nEC; ++c)
        for (int k = 0; k < nCos; ++k)
          ead[(size_t)c * nCos + k] = 2.0 * eah[(size_t)c * nCos + k] / (std::sqrt(ecell[c]) * norm * eedf_step_ * cstep);
    }
    if (eadf) std::copy(ead.begin(), ead.end(), eadf);
    for (int c = 0; c < nEC; ++c) {
      double f1 = 0, f2 = 0;
      for (int k = 0; k < nCos; ++k) {
        const double mu = -1.0 + cstep / 2.0 + k * cstep;
        f1 += ead[(size_t)c * nCos + k] * mu;
        f2 += ead[(size_t)c * nCos + k] * 0.5 * (3.0 * mu * mu - 1);
      }
      if (efadf) efadf[c] = 1.5 * f1 * cstep;
      if (esadf) esadf[c] = 2.5 * f2 * cstep;
    }
    if (rcells)
      for (int k = 0; k < nR; ++k) rcells[k] = rad_step_ / 2.0 + k * rad_step_;
    if (acells)
      for (int k = 0; k < nA; ++k) acells[k] = -max_speed_ + ax_step_ / 2.0 + k * ax_step_;
    if (evdf) {
      double den = 0;
      for (int k = 0; k < nR; ++k) {
        double row = 0;
        for (int j = 0; j < nA; ++j) row += evh[(size_t)k * nA + j];
        den += row * ax_step_ * 2.0 * kPi * (rad_step_ / 2.0 + k * rad_step_) * rad_step_;
      }
      for (size_t q = 0; q < evh.size(); ++q) evdf[q] = cylindrical_ && den > 0 ? evh[q] / den : 0.0;
    }
    if (eedf_per && omega_ != 0) {
      for (int q = 0; q < nPh; ++q) {
        double n = 0;
        for (int c = 0; c < nEC; ++c) n += per[(size_t)q * nEC + c];
        for (int c = 0; c < nEC; ++c)
          eedf_per[(size_t)q * nEC + c] = per[(size_t)q * nEC + c] / (std::sqrt(ecell[c]) * n * eedf_step_);
      }
    }
    return LGPU_OK;
  }

  // getAveragedPeriodicParams (BoltzmannMC.C:1728-1734)
  int periodic(double* n, double* me, double* fv, double* bv, double* fd, double* bd) const {
    const int nPh = (int)phase_n_.size();
    for (int q = 0; q < nPh; ++q) {
      const double c = phase_n_[q];
      if (n) n[q] = c;
      if (me) me[q] = phase_me_[q] / c;
      for (int k = 0; k < 3; ++k) {
        if (fv) fv[3 * q + k] = phase_fv_[3 * q + k] / c;
        if (bv) bv[3 * q + k] = phase_bv_[3 * q + k] / c;
      }
      for (int k = 0; k < 9; ++k) {
        if (fd) fd[9 * q + k] = phase_fd_[9 * q + k] / c;
        if (bd) bd[9 * q + k] = phase_bd_[9 * q + k] / c;
      }
    }
    return LGPU_OK;
  }

  long long series(int which, double* out, long long max_rows) {
    const std::vector<double>* v = nullptr;
    int w = 1;
    switch (which) {
      case 0: v = &ts_; break;
      case 1: v = &me_; break;
      case 2: v = &mp_; w = 3; break;
      case 3: v = &mv_; w = 3; break;
      case 4: v = &fd_; w = 9; break;
      case 5: v = &pc_; w = 9; break;
      case 6: v = &bv_; w = 3; break;
      case 7: v = &bd_; w = 9; break;
      default: return -fail(LGPU_ERR_BAD_ARG, "unknown series %d", which);
    }
    const long long rows = std::min<long long>(max_rows, (long long)(v->size() / w));
    if (out) std::copy(v->begin(), v->begin() + rows * w, out);
    return rows;
  }

  // lgpu_advance: n intervals with a sample after each
  int advance(int n, lgpu_step_report* rep) {
    if (!initialized_) return fail(LGPU_ERR_STATE, "init_ensemble comes first");
    for (int i = 0; i < n; ++i) {
      LGPU_TRY(step_interval(true));
      ++n_samp_;
      LGPU_TRY(process_sample());
    }
    if (rep) {
      LGPU_TRY(read_counters());
      rep->time = time_;
      rep->trial_freq = nu_trial_;
      rep->max_energy = cur_max_energy_;
      rep->mean_energy = me_.empty() ? 0.0 : me_.back();
      rep->real_collisions = (double)total_real_dev_;
      rep->null_collisions = (double)total_null_dev_;
      rep->sync_steps = (long long)interval_;
    }
    return LGPU_OK;
  }

  // ------------------------------------------- EEDF post-processing
  // The collisions behind the MC processes as the reference's end-of-job
  // routines read them (lgpu_set_twoterm): 6 int columns of P (kind, ion,
  // integral offset and length, momentum-transfer offset and length) and 4
  // double columns (density, threshold, mass ratio, statistical-weight
  // ratio); the raw tables back to back (integral energies, values,
  // momentum-transfer energies, values).
  int tt_n_ = 0;
  int* d_tt_i_ = nullptr;
  double* d_tt_d_ = nullptr;
  double* d_tt_raw_ = nullptr;
  size_t tt_int_total_ = 0, tt_mom_total_ = 0;
  double* d_post_ = nullptr;  // external EEDF, scratch, outputs
  size_t post_cap_ = 0;

  int set_twoterm(const lgpu_twoterm_process* q, int n) {
    if (P_ <= 0) return fail(LGPU_ERR_STATE, "set the processes before their two-term inputs");
    if (!q || n != P_) return fail(LGPU_ERR_BAD_ARG, "expected %d processes", P_);
    std::vector<int> vi(6 * (size_t)n);
    std::vector<double> vd(4 * (size_t)n), ie, iv, me, mv;
    for (int p = 0; p < n; ++p) {
      const lgpu_twoterm_process& c = q[p];
      if (c.kind < 0 || c.kind > 2 || c.ion < 0 || c.ion > 2)
        return fail(LGPU_ERR_BAD_ARG, "process %d: kind %d / ion %d out of range", p, c.kind, c.ion);
      if (c.kind == 2 && (p == 0 || q[p - 1].kind == 2))
        return fail(LGPU_ERR_BAD_ARG, "process %d: a superelastic copy follows its forward collision", p);
      if (c.n_int < 2 || !c.int_e || !c.int_v || (c.n_mom != 0 && (c.n_mom < 2 || !c.mom_e || !c.mom_v)))
        return fail(LGPU_ERR_BAD_ARG, "process %d: raw tables need at least 2 points", p);
      if (!(c.threshold >= 0) || !(c.density >= 0) || !(c.mass_ratio >= 0) || !(c.stat_ratio >= 0))
        return fail(LGPU_ERR_BAD_ARG, "process %d: negative or NaN threshold, density or ratio", p);
      // momentum transfer defaults to the integral cross section (isotropic scattering)
      const int nm = c.n_mom ? c.n_mom : c.n_int;
      const double* e2 = c.n_mom ? c.mom_e : c.int_e;
      const double* v2 = c.n_mom ? c.mom_v : c.int_v;
      for (int k = 1; k < c.n_int; ++k)
        if (!(c.int_e[k] > c.int_e[k - 1])) return fail(LGPU_ERR_BAD_ARG, "process %d: integral energies not increasing", p);
      for (int k = 1; k < nm; ++k)
        if (!(e2[k] > e2[k - 1])) return fail(LGPU_ERR_BAD_ARG, "process %d: momentum-transfer energies not increasing", p);
      vi[0 * (size_t)n + p] = c.kind;
      vi[1 * (size_t)n + p] = c.ion;
      vi[2 * (size_t)n + p] = (int)ie.size();
      vi[3 * (size_t)n + p] = c.n_int;
      vi[4 * (size_t)n + p] = (int)me.size();
      vi[5 * (size_t)n + p] = nm;
      vd[0 * (size_t)n + p] = c.density;
      vd[1 * (size_t)n + p] = c.threshold;
      vd[2 * (size_t)n + p] = c.mass_ratio;
      vd[3 * (size_t)n + p] = c.stat_ratio;
      ie.insert(ie.end(), c.int_e, c.int_e + c.n_int);
      iv.insert(iv.end(), c.int_v, c.int_v + c.n_int);
      me.insert(me.end(), e2, e2 + nm);
      mv.insert(mv.end(), v2, v2 + nm);
    }
    std::vector<double> raw;
    raw.reserve(2 * (ie.size() + me.size()));
    raw.insert(raw.end(), ie.begin(), ie.end());
    raw.insert(raw.end(), iv.begin(), iv.end());
    raw.insert(raw.end(), me.begin(), me.end());
    raw.insert(raw.end(), mv.begin(), mv.end());
    for (void* d : {(void*)d_tt_i_, (void*)d_tt_d_, (void*)d_tt_raw_})
      if (d) cudaFree(d);
    d_tt_i_ = nullptr;
    d_tt_d_ = nullptr;
    d_tt_raw_ = nullptr;
    tt_n_ = 0;
    LGPU_TRY(dalloc(&d_tt_i_, vi.size()));
    LGPU_TRY(dalloc(&d_tt_d_, vd.size()));
    LGPU_TRY(dalloc(&d_tt_raw_, raw.size()));
    LGPU_CU(copy(d_tt_i_, vi.data(), vi.size() * sizeof(int), cudaMemcpyHostToDevice));
    LGPU_CU(copy(d_tt_d_, vd.data(), vd.size() * sizeof(double), cudaMemcpyHostToDevice));
    LGPU_CU(copy(d_tt_raw_, raw.data(), raw.size() * sizeof(double), cudaMemcpyHostToDevice));
    tt_int_total_ = ie.size();
    tt_mom_total_ = me.size();
    tt_n_ = n;
    return LGPU_OK;
  }

  bool has_twoterm() const { return tt_n_ > 0 && tt_n_ == P_; }

  // the reference's end-of-job routines that read the EEDF
  // (Collision.C:355-397, BoltzmannMC.C:2186-2266), on the device
  int eedf_postprocess(const double* eedf, int nc, double max_e, lgpu_eedf_params* out, double* rate, int n) {
    if (!eedf) {
      nc = cfg_.n_energy_cells;
      max_e = max_eedf_;
      if (!(max_e > 0)) return fail(LGPU_ERR_STATE, "no EEDF yet: the distributions start at the steady state");
    }
    return run_post(eedf, eedf ? nullptr : d_eedf_, 1, nc, max_e, false, out, rate, n);
  }

  // the rate coefficients of several EEDFs, or (eedf null) of the per-phase
  // EEDFs of an AC run (BoltzmannMC.C:2276-2330, normalised as :1736-1740)
  int eedf_rates(const double* eedf, int n_eedf, int nc, double max_e, double* rate, int n) {
    if (!eedf) {
      if (omega_ == 0) return fail(LGPU_ERR_STATE, "per-phase EEDFs exist only under an AC field");
      nc = cfg_.n_energy_cells;
      max_e = max_eedf_;
      n_eedf = std::max(cfg_.n_phases, 1);
      if (!(max_e > 0)) return fail(LGPU_ERR_STATE, "no EEDF yet: the distributions start at the steady state");
    }
    if (n_eedf < 1) return fail(LGPU_ERR_BAD_ARG, "no EEDF given");
    return run_post(eedf, eedf ? nullptr : d_eedf_per_, n_eedf, nc, max_e, true, nullptr, rate, n);
  }

  int run_post(const double* eedf, const double* eeh, int n_eedf, int nc, double max_e, bool rates_only,
               lgpu_eedf_params* out, double* rate, int n) {
    if (!has_twoterm()) return fail(LGPU_ERR_STATE, "no two-term inputs: call lgpu_set_twoterm first");
    if (rate && n != P_) return fail(LGPU_ERR_BAD_ARG, "expected %d processes", P_);
    if (nc < 2 || !(max_e > 0))
      return fail(LGPU_ERR_BAD_ARG, "an EEDF needs at least 2 cells and a positive maximum energy");
    const size_t nn = (size_t)nc + 1;
    const size_t need = (size_t)n_eedf * ((size_t)nc + 5 * nn + (size_t)P_) + 16;
    if (need > post_cap_) {
      if (d_post_) cudaFree(d_post_);
      d_post_ = nullptr;
      post_cap_ = 0;
      LGPU_TRY(dalloc(&d_post_, need));
      post_cap_ = need;
    }
    EedfPostArgs a{};
    a.nc = nc;
    a.P = P_;
    a.n_eedf = n_eedf;
    a.rates_only = rates_only ? 1 : 0;
    a.max_energy = max_e;
    a.gas_density = Ngas_;
    a.omega = omega_;
    a.omega_c = omega_c_;
    a.eeh = eeh ? eeh : d_post_;  // unread when the EEDFs are given
    if (eedf) {
      LGPU_CU(cudaMemcpyAsync(d_post_, eedf, (size_t)n_eedf * nc * sizeof(double), cudaMemcpyHostToDevice, stream_));
      a.eedf_in = d_post_;
    }
    a.scratch = d_post_ + (size_t)n_eedf * nc;
    a.rates = a.scratch + (size_t)n_eedf * 5 * nn;
    a.params = a.rates + (size_t)n_eedf * P_;
    a.kind = d_tt_i_;
    a.ion = d_tt_i_ + P_;
    a.int_off = d_tt_i_ + 2 * P_;
    a.int_len = d_tt_i_ + 3 * P_;
    a.mom_off = d_tt_i_ + 4 * P_;
    a.mom_len = d_tt_i_ + 5 * P_;
    a.dens = d_tt_d_;
    a.thr = d_tt_d_ + P_;
    a.mass_ratio = d_tt_d_ + 2 * P_;
    a.stat = d_tt_d_ + 3 * P_;
    a.raw_ie = d_tt_raw_;
    a.raw_iv = d_tt_raw_ + tt_int_total_;
    a.raw_me = d_tt_raw_ + 2 * tt_int_total_;
    a.raw_mv = d_tt_raw_ + 2 * tt_int_total_ + tt_mom_total_;
    launch_eedf_post(a, stream_);
    ++launches_;
    LGPU_CU(cudaGetLastError());
    std::vector<double> res((size_t)n_eedf * P_ + 16);
    LGPU_CU(cudaMemcpyAsync(res.data(), a.rates, res.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    LGPU_TRY(sync("eedf post-processing"));
    if (rate) std::copy(res.begin(), res.begin() + (size_t)n_eedf * P_, rate);
    if (out) {
      const double* v = res.data() + (size_t)n_eedf * P_;
      *out = lgpu_eedf_params{v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], v[12],
                              v[13], v[14], v[15]};
    }
    return LGPU_OK;
  }

  // ------------------------------------------------------------ replay
  double* d_rp_in_ = nullptr;
  double* d_rp_out_ = nullptr;
  size_t rp_in_cap_ = 0, rp_out_cap_ = 0;
  int rp_reserve(size_t in, size_t out) {
    if (in > rp_in_cap_) {
      if (d_rp_in_) cudaFree(d_rp_in_);
      d_rp_in_ = nullptr;
      LGPU_TRY(dalloc(&d_rp_in_, in));
      rp_in_cap_ = in;
    }
    if (out > rp_out_cap_) {
      if (d_rp_out_) cudaFree(d_rp_out_);
      d_rp_out_ = nullptr;
      LGPU_TRY(dalloc(&d_rp_out_, out));
      rp_out_cap_ = out;
    }
    return LGPU_OK;
  }

  int replay_flights(int n, const double* t, const double* dt, const double* pos, const double* vel, double* po,
                     double* vo, double* eo, double* go) {
    if (n <= 0) return LGPU_OK;
    std::vector<double> in((size_t)n * 8);
    for (int i = 0; i < n; ++i) {
      double phi = 0.0;
      if (field_.mode == kFieldAC || field_.mode == kFieldACB) phi = std::fmod(omega_ * t[i], 2.0 * kPi);
      else if (field_.mode == kFieldECR) phi = std::fmod(omega_c_ * t[i], 2.0 * kPi);
      in[i] = phi;
      in[n + i] = dt[i];
      for (int k = 0; k < 3; ++k) {
        in[2 * (size_t)n + 3 * i + k] = pos[3 * i + k];
        in[5 * (size_t)n + 3 * i + k] = vel[3 * i + k];
      }
    }
    LGPU_TRY(rp_reserve(in.size(), (size_t)n * 8));
    LGPU_CU(copy(d_rp_in_, in.data(), in.size() * sizeof(double), cudaMemcpyHostToDevice));
    ReplayFlightArgs a{};
    a.n = n;
    a.phi0 = d_rp_in_;
    a.dt = d_rp_in_ + n;
    a.pos = d_rp_in_ + 2 * (size_t)n;
    a.vel = d_rp_in_ + 5 * (size_t)n;
    a.pos_out = d_rp_out_;
    a.vel_out = d_rp_out_ + 3 * (size_t)n;
    a.energy_out = d_rp_out_ + 6 * (size_t)n;
    a.gain_out = d_rp_out_ + 7 * (size_t)n;
    a.field = field_;
    a.half_me_over_e = (float)(0.5 * kMeD / kQeD);
    launch_replay_flight(a, stream_);
    ++launches_;
    std::vector<double> out((size_t)n * 8);
    LGPU_CU(copy(out.data(), d_rp_out_, out.size() * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_TRY(sync("replay_flights"));
    std::copy(out.begin(), out.begin() + 3 * (size_t)n, po);
    std::copy(out.begin() + 3 * (size_t)n, out.begin() + 6 * (size_t)n, vo);
    std::copy(out.begin() + 6 * (size_t)n, out.begin() + 7 * (size_t)n, eo);
    std::copy(out.begin() + 7 * (size_t)n, out.begin() + 8 * (size_t)n, go);
    return LGPU_OK;
  }

  int replay_collisions(int n, const double* nu, const double* vel, const double* energy, const double* u, int stride,
                        double* out, int* used, int coarse = 0) {
    if (n <= 0) return LGPU_OK;
    if (max_interp_ < 0) return fail(LGPU_ERR_STATE, "tables are not built");
    LGPU_TRY(upload_proc_consts());
    const size_t nin = (size_t)n * (5 + stride);
    LGPU_TRY(rp_reserve(nin, (size_t)n * 12));
    std::vector<double> in(nin);
    std::copy(nu, nu + n, in.begin());
    std::copy(vel, vel + 3 * (size_t)n, in.begin() + n);
    std::copy(energy, energy + n, in.begin() + 4 * (size_t)n);
    std::copy(u, u + (size_t)n * stride, in.begin() + 5 * (size_t)n);
    LGPU_CU(copy(d_rp_in_, in.data(), nin * sizeof(double), cudaMemcpyHostToDevice));
    ReplayCollArgs a{};
    a.n = n;
    a.nu = d_rp_in_;
    a.vel = d_rp_in_ + n;
    a.energy = d_rp_in_ + 4 * (size_t)n;
    a.u = d_rp_in_ + 5 * (size_t)n;
    a.u_stride = stride;
    a.out = d_rp_out_;
    a.used = reinterpret_cast<int*>(d_rp_out_ + 11 * (size_t)n);
    a.c = consts();
    a.t = tables();
    a.procs = d_procf_;
    a.gases = d_gasf_;
    a.coarse = coarse;
    launch_replay_collide(a, stream_);
    ++launches_;
    LGPU_CU(copy(out, d_rp_out_, (size_t)n * 11 * sizeof(double), cudaMemcpyDeviceToHost));
    LGPU_CU(copy(used, d_rp_out_ + 11 * (size_t)n, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost));
    return sync("replay_collisions");
  }

  int tables_out(double max_energy, double* nu_tot, double* nu_max, float* sig, float* cum) {
    if (!have_procs_ || !(Ngas_ > 0)) return fail(LGPU_ERR_STATE, "set_processes and set_conditions come first");
    max_interp_ = -1.0;
    LGPU_TRY(build_tables(max_energy));
    if (nu_tot) LGPU_CU(copy(nu_tot, d_nu_tot_, M_ * sizeof(double), cudaMemcpyDeviceToHost));
    if (nu_max) std::copy(h_nu_max_, h_nu_max_ + M_, nu_max);
    std::vector<float2> pairs((size_t)M_ * stride_);
    if (sig) {
      LGPU_CU(copy(pairs.data(), d_sig_pair_, pairs.size() * sizeof(float2), cudaMemcpyDeviceToHost));
      LGPU_TRY(sync("tables_out"));
      for (int i = 0; i < M_; ++i)
        for (int p = 0; p < P_; ++p) sig[(size_t)i * P_ + p] = pairs[(size_t)i * stride_ + p].x;
    }
    if (cum) {
      LGPU_CU(copy(pairs.data(), d_cum_pair_, pairs.size() * sizeof(float2), cudaMemcpyDeviceToHost));
      LGPU_TRY(sync("tables_out"));
      for (int i = 0; i < M_; ++i)
        for (int p = 0; p < P_; ++p) cum[(size_t)i * P_ + p] = pairs[(size_t)i * stride_ + p].x;
    }
    return sync("tables_out");
  }

  // ------------------------------------------------------------ state
  int N_ = 0, P_ = 0, M_ = 0, sec_cap_ = 0, sm_count_ = 1, stride_ = 2;
  size_t claim_words_ = 0;
  std::vector<lgpu_process> procs_;
  std::vector<lgpu_gas> gases_;
  bool have_procs_ = false, have_cond_ = false, have_ion_att_ = false, initialized_ = false, solved_ = false;
  double emax_elastic_ = 1e100;
  double Ngas_ = 0, Tg_ = 0, gas_energy_ = 0, red_field_ = 0, angle_ = 180;
  double E_[3] = {0, 0, 0}, freq_ = 0, omega_ = 0, red_mag_ = 0, omega_c_ = 0;
  bool cylindrical_ = true;
  FieldF field_{};
  double max_interp_ = -1, step_ = 0, nu_trial_ = 0;
  double* h_nu_max_ = nullptr;  // pinned: the asynchronous re-grid reads it back
  cudaEvent_t tables_ev_ = nullptr;
  bool tables_inflight_ = false;
  double time_ = 0, ss_time_ = kNonDef;
  uint64_t interval_ = 0;
  double origin_[3] = {0, 0, 0}, shift_[3] = {0, 0, 0};
  double cur_max_energy_ = 0, max_elec_energy_ = 0;
  // counters
  unsigned long long total_real_dev_ = 0, total_null_dev_ = 0;
  unsigned long long total_coll_ = 0, null_coll_ = 0, coll_at_ss_ = 0, null_at_ss_ = 0;
  double field_gain_ = 0, growth_ = 0;
  std::vector<unsigned long long> base_proc_count_;
  std::vector<double> base_proc_gain_, base_proc_loss_;
  unsigned long long base_null_ = 0;
  double base_field_gain_ = 0, base_growth_ = 0, base_time_adjust_ = 0;
  double pb_rel_err_ = 0;
  // series
  std::vector<double> ts_, me_, mp_, mv_, fd_, pc_, bv_, bd_;
  long long n_samp_ = 0, n_sync_ = 0, n_int_ = 0, first_int_ = 0;
  double total_int_time_ = 0;
  std::vector<double> phase_n_, phase_me_, phase_fv_, phase_bv_, phase_fd_, phase_bd_;
  // distributions
  double max_eedf_ = 0, eedf_step_ = 0, max_speed_ = 0, rad_step_ = 1, ax_step_ = 1;
  int status_ = LGPU_OK;
  // solve steps
  std::chrono::steady_clock::time_point solve_t0_;
  bool solve_good_ = false, sampling_ = false;
  int solve_capped_ = 0;
  long long solve_steps_ = 0;
  double pending_dt_ = 0;
  // batch mode
  bool batch_ = false, hist_pending_ = false, evdf_fused_ = false;
  BatchSlot slot_{};                            // cached argument blocks of this solve's batch slot
  long long solve_serial_ = 0, slot_built_ = -1;
  int sec_grown_ = 0;  // times the secondary buffers grew
  cudaStream_t own_stream_ = nullptr;
  HistArgs pending_hist_{};
  // timing
  double adv_ms_ = 0, adv_electron_steps_ = 0, h2d_bytes_ = 0, d2h_bytes_ = 0;
  long long adv_launches_ = 0, launches_ = 0;
  // device buffers (carved from d_core_, d_secbuf_ and d_procbuf_) and the pinned host block
  char *d_core_ = nullptr, *d_secbuf_ = nullptr, *d_procbuf_ = nullptr, *h_pinned_ = nullptr;
  float4* d_state_ = nullptr;
  int* d_alive_ = nullptr;
  float4* d_spill_ = nullptr;
  float4* d_sec_ = nullptr;
  int* d_att_ = nullptr;
  unsigned int* d_claim_ = nullptr;
  int *d_removed_ = nullptr, *d_pair_slot_ = nullptr, *d_pair_sec_ = nullptr;
  DevScalars* d_sc_ = nullptr;
  DevScalars* h_sc_ = nullptr;
  IntervalCtl* d_ctl_ = nullptr;
  IntervalCtl* h_ctl_ = nullptr;
  cudaGraphExec_t graph_[2] = {nullptr, nullptr};
  long long graph_launches_[2] = {0, 0};
  float2 *d_nu_pair_ = nullptr, *d_cum_pair_ = nullptr, *d_sig_pair_ = nullptr;
  double *d_nu_tot_ = nullptr, *d_nu_max_ = nullptr;
  float* d_nu_coarse_ = nullptr;
  int coarse_shift_ = 0, n_coarse_ = 1;
  ProcF* d_procf_ = nullptr;
  GasF* d_gasf_ = nullptr;
  int *d_is_super_ = nullptr, *d_raw_off_ = nullptr, *d_raw_len_ = nullptr;
  double *d_superw_ = nullptr, *d_emin_ = nullptr, *d_emax_ = nullptr, *d_rel_dens_ = nullptr, *d_raw_e_ = nullptr,
         *d_raw_v_ = nullptr;
  unsigned long long* d_proc_count_ = nullptr;
  double *d_proc_gain_ = nullptr, *d_proc_loss_ = nullptr;
  double *d_eedf_ = nullptr, *d_eedf_per_ = nullptr, *d_eadf_ = nullptr, *d_evdf_ = nullptr;
};

}  // namespace lgpu

// the C ABI's context handle
struct lgpu_ctx {
  lgpu::Engine* e;
};
