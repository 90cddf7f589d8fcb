// lgpu_engine.cpp - the C ABI of include/loki_gpu.h over lgpu::Engine
// (one swarm condition per context).
#include "lgpu_engine.h"

// ====================================================================== C ABI

extern "C" {

void lgpu_config_default(lgpu_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->device = 0;
  c->seed = 12345;
  c->n_electrons = 1e4;
  c->n_interp = 10000;                 // BoltzmannMC.h:104
  c->gas_temperature_effect = 0;
  c->sharing = 0;
  c->init_temp_ratio = 0.01;           // BoltzmannMC.h:74
  c->min_coll_before_ss = 0;           // BoltzmannMC.h:54
  c->max_coll_before_ss = 1e100;       // BoltzmannMC.h:55
  c->max_coll_after_ss = 1e100;        // BoltzmannMC.h:56
  c->req_integration_points = 200;     // BoltzmannMC.h:69
  c->req_ss_times = 0;
  c->req_abs_time = 0;
  c->errors_checked = 0;
  c->req_err_mean_energy = c->req_err_flux_v = c->req_err_flux_d = 1e100;
  c->req_err_bulk_v = c->req_err_bulk_d = c->req_err_power = 1e100;
  c->n_energy_cells = 1000;            // BoltzmannMC.h:59-62
  c->n_cos_cells = 100;
  c->n_radial_cells = 200;
  c->n_axial_cells = 200;
  c->n_phases = 100;                   // BoltzmannMC.h:75
  c->sync_x = 1.0;                     // BoltzmannMC.h:72
  c->sync_oversampling = 1;            // BoltzmannMC.h:73
  c->max_seconds = 0;
  c->max_sync_steps = 0;
  c->advance_real_batch = 0;
  c->advance_queue = 0;
}

#define CTX_CHECK(ctx)                          \
  do {                                          \
    if (!(ctx) || !(ctx)->e) return LGPU_ERR_BAD_ARG; \
  } while (0)

int lgpu_create(const lgpu_config* cfg, lgpu_ctx** out) {
  if (!cfg || !out) return LGPU_ERR_BAD_ARG;
  *out = nullptr;
  lgpu::Engine* e = new (std::nothrow) lgpu::Engine(*cfg);
  if (!e) return LGPU_ERR_OOM;
  lgpu_ctx* c = new (std::nothrow) lgpu_ctx{e};
  if (!c) {
    delete e;
    return LGPU_ERR_OOM;
  }
  *out = c;
  return e->init();
}

int lgpu_destroy(lgpu_ctx* ctx) {
  if (!ctx) return LGPU_OK;
  delete ctx->e;
  delete ctx;
  return LGPU_OK;
}

int lgpu_last_error(const lgpu_ctx* ctx, char* buf, size_t size) {
  if (!ctx || !ctx->e) return 0;
  const std::string& s = ctx->e->err_;
  if (buf && size) {
    std::snprintf(buf, size, "%s", s.c_str());
  }
  return (int)s.size();
}

void* lgpu_stream(lgpu_ctx* ctx) { return (ctx && ctx->e) ? (void*)ctx->e->stream_ : nullptr; }

int lgpu_set_processes(lgpu_ctx* ctx, const lgpu_process* procs, int n, const lgpu_gas* gases, int ng, double emax) {
  CTX_CHECK(ctx);
  if (!procs || !gases) return LGPU_ERR_BAD_ARG;
  return ctx->e->set_processes(procs, n, gases, ng, emax);
}

int lgpu_set_conditions(lgpu_ctx* ctx, const lgpu_conditions* c) {
  CTX_CHECK(ctx);
  if (!c) return LGPU_ERR_BAD_ARG;
  return ctx->e->set_conditions(*c);
}

int lgpu_init_ensemble(lgpu_ctx* ctx) {
  CTX_CHECK(ctx);
  return ctx->e->init_ensemble();
}

int lgpu_advance(lgpu_ctx* ctx, int n, lgpu_step_report* rep) {
  CTX_CHECK(ctx);
  if (n < 0) return LGPU_ERR_BAD_ARG;
  return ctx->e->advance(n, rep);
}

int lgpu_solve(lgpu_ctx* ctx, lgpu_result* r) {
  CTX_CHECK(ctx);
  if (!r) return LGPU_ERR_BAD_ARG;
  return ctx->e->solve(r);
}

int lgpu_get_process_results(lgpu_ctx* ctx, unsigned long long* counts, double* rate, double* gain, double* loss,
                             int n) {
  CTX_CHECK(ctx);
  return ctx->e->process_results(counts, rate, gain, loss, n);
}

int lgpu_get_distributions(lgpu_ctx* ctx, double* cells, double* eedf, double* efadf, double* esadf, double* eadf,
                           double* evdf, double* rcells, double* acells, double* eedf_per) {
  CTX_CHECK(ctx);
  return ctx->e->distributions(cells, eedf, efadf, esadf, eadf, evdf, rcells, acells, eedf_per);
}

int lgpu_set_twoterm(lgpu_ctx* ctx, const lgpu_twoterm_process* p, int n) {
  CTX_CHECK(ctx);
  return ctx->e->set_twoterm(p, n);
}

int lgpu_eedf_postprocess(lgpu_ctx* ctx, const double* eedf, int n_cells, double max_energy, lgpu_eedf_params* out,
                          double* rate, int n) {
  CTX_CHECK(ctx);
  return ctx->e->eedf_postprocess(eedf, n_cells, max_energy, out, rate, n);
}

int lgpu_eedf_rates(lgpu_ctx* ctx, const double* eedf, int n_eedf, int n_cells, double max_energy, double* rate,
                    int n) {
  CTX_CHECK(ctx);
  return ctx->e->eedf_rates(eedf, n_eedf, n_cells, max_energy, rate, n);
}

int lgpu_get_periodic(lgpu_ctx* ctx, double* n, double* me, double* fv, double* bv, double* fd, double* bd) {
  CTX_CHECK(ctx);
  return ctx->e->periodic(n, me, fv, bv, fd, bd);
}

long long lgpu_get_series(lgpu_ctx* ctx, int which, double* out, long long max_rows) {
  if (!ctx || !ctx->e) return -LGPU_ERR_BAD_ARG;
  return ctx->e->series(which, out, max_rows);
}

int lgpu_get_timing(lgpu_ctx* ctx, lgpu_timing* t) {
  CTX_CHECK(ctx);
  if (!t) return LGPU_ERR_BAD_ARG;
  t->advance_ms = ctx->e->adv_ms_;
  t->advance_launches = ctx->e->adv_launches_;
  t->electron_steps = ctx->e->adv_electron_steps_;
  t->kernel_launches = ctx->e->launches_;
  t->h2d_bytes = ctx->e->h2d_bytes_;
  t->d2h_bytes = ctx->e->d2h_bytes_;
  return LGPU_OK;
}

int lgpu_build_tables(lgpu_ctx* ctx, double max_energy, double* nu_tot, double* nu_max, float* sig, float* cum) {
  CTX_CHECK(ctx);
  if (!(max_energy > 0)) return LGPU_ERR_BAD_ARG;
  return ctx->e->tables_out(max_energy, nu_tot, nu_max, sig, cum);
}

int lgpu_set_field_raw(lgpu_ctx* ctx, const double e[3], double freq_hz, double red_mag, double cyclotron) {
  CTX_CHECK(ctx);
  if (!e) return LGPU_ERR_BAD_ARG;
  return ctx->e->set_field_raw(e, freq_hz, red_mag, cyclotron);
}

int lgpu_replay_flights(lgpu_ctx* ctx, int n, const double* t, const double* dt, const double* pos, const double* vel,
                        double* po, double* vo, double* eo, double* go) {
  CTX_CHECK(ctx);
  if (n < 0 || (n > 0 && (!t || !dt || !pos || !vel || !po || !vo || !eo || !go))) return LGPU_ERR_BAD_ARG;
  return ctx->e->replay_flights(n, t, dt, pos, vel, po, vo, eo, go);
}

int lgpu_replay_collisions(lgpu_ctx* ctx, int n, const double* nu, const double* vel, const double* energy,
                           const double* u, int stride, double* out, int* used) {
  CTX_CHECK(ctx);
  if (n < 0 || stride < 1 || (n > 0 && (!nu || !vel || !energy || !u || !out || !used))) return LGPU_ERR_BAD_ARG;
  return ctx->e->replay_collisions(n, nu, vel, energy, u, stride, out, used);
}

int lgpu_replay_collisions_coarse(lgpu_ctx* ctx, int n, const double* nu, const double* vel, const double* energy,
                                  const double* u, int stride, double* out, int* used) {
  CTX_CHECK(ctx);
  if (n < 0 || stride < 1 || (n > 0 && (!nu || !vel || !energy || !u || !out || !used))) return LGPU_ERR_BAD_ARG;
  return ctx->e->replay_collisions(n, nu, vel, energy, u, stride, out, used, 1);
}

}  // extern "C"
