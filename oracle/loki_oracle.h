/*
 * loki_oracle.h - CPU restatement of LoKI-MC's electron Monte Carlo engine.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT. Only the tests, the smoke check and the
 * CPU-baseline leg of the benchmark may load this library, and only for the
 * results the GPU path is compared with or as the timed CPU baseline. The GPU product never links it.
 *
 * Every function restates one routine of the reference engine
 * (Code/LoKI-MC/Sources/BoltzmannMC.C, Code/LoKI-MC/Sources/MathFunctions.C,
 * Code/LoKI-MC/Headers/AngularScatteringFunctions.h) in FP64 with the same
 * operation order, so that, fed the same uniforms, it reproduces the
 * reference's per-electron results. The restatement is pinned against the
 * reference built from its own sources (oracle/ref) through golden vectors in
 * tests/golden/.
 */
#ifndef LOKI_ORACLE_H
#define LOKI_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Random stream: replay of recorded uniforms, or xoshiro256** when replay is NULL. */
typedef struct lo_rng {
  uint64_t s[4];
  const double* replay;
  size_t n, pos;
  int overrun;
} lo_rng;

void lo_rng_seed(lo_rng* r, uint64_t seed, uint64_t stream);
void lo_rng_replay(lo_rng* r, const double* u, size_t n);
double lo_uniform(lo_rng* r, int include_zero, int include_one);

/* Flattened processes and interpolated tables (BoltzmannMC.h:86-118). */
typedef struct lo_procs {
  int P, G;
  const int* ptype;          /* 0 conservative, 1 ionization, 2 attachment */
  const int* is_super;
  const int* sampler;        /* 0 iso, 1 fwd, 2 bornDipole, 3 surendra, 4 coulombScreen, 5 momentum conservation */
  const double* sampler_p0;
  const double* sampler_p1;
  const double* superw;
  const double* emin;
  const double* emax;
  const double* rel_dens;
  const double* mass;
  const double* red_mass;
  const double* eloss;
  const double* wparam;
  const int* raw_off;        /* offset of each process' raw table in raw_e/raw_v */
  const int* raw_len;
  const double* raw_e;
  const double* raw_v;
  const int* gas_first;
  const int* gas_last;
  const double* gas_frac;
  double energy_max_elastic;
  /* tables (owned by the caller, sizes M and M*P) */
  int M;
  double max_interp, step;
  double* grid;
  double* sig;               /* [i*P + p] */
  double* cum;               /* [i*P + p] */
  double* nu_tot;
  double* nu_max;
} lo_procs;

typedef struct lo_fields {
  double N;            /* total gas density, m^-3 */
  double Tg;           /* gas temperature, K */
  double gas_energy;   /* 1.5 k Tg / e, eV */
  double E[3];         /* electric field vector, V/m (amplitude for AC) */
  double acc[3];       /* -e E / m */
  double freq_hz;      /* excitation frequency, Hz */
  double omega;        /* 2 pi f */
  double red_mag;      /* B/N, Hx (only compared with zero) */
  double omega_c;      /* cyclotron frequency e B / m */
  int gas_temp_effect; /* 0 false, 1 true, 2 smartActivation */
  int sharing;         /* 0 equal, 1 oneTakesAll, 2 SDCS, 3 randomUniform */
  double sharing_factor;
} lo_fields;

/* Per-collision result (performCollision and the kinematics routines). */
typedef struct lo_coll_out {
  int chosen;           /* process id, -1 null */
  double vel[3];
  double energy;
  double dE;            /* electronEnergyChanges */
  double dE_over_E;     /* electronEnergyChangesOverIncidEnergies */
  double ej_vel[3];
  double ej_energy;
} lo_coll_out;

/* GSL-style linear interpolation on the raw table of process p. */
double lo_interp(const lo_procs* pr, int p, double x);
/* BoltzmannMC.C:561-615 */
void lo_build_tables(lo_procs* pr, const lo_fields* f, double max_energy);
/* BoltzmannMC.C:804-905 */
void lo_accelerate(const lo_fields* f, double t, double dt, double* pos, double* vel, double* energy,
                   double* gain);
/* BoltzmannMC.C:907-1280 (one collision event at the end of a free flight) */
void lo_collide(const lo_procs* pr, const lo_fields* f, double nu_trial, const double* vel_in, double energy_in,
                lo_rng* rng, lo_coll_out* out);
/* BoltzmannMC.C:765-802 */
double lo_max_accel_energy(const lo_fields* f, double initial_energy, double dt);

/* MathFunctions.C:211-231 */
double lo_statistical_error(const double* a, int n, double nbins);

/* ---- full solve (BoltzmannMC.C:299-426 and what it calls) ---- */
typedef struct lo_run_config {
  int n_electrons;
  int n_threads;
  uint64_t seed;
  double init_temp_ratio;          /* initialElecTempOverGasTemp */
  double sync_x;                   /* synchronizationTimeXMaxCollisionFrequency */
  int sync_oversampling;
  double min_coll_before_ss;       /* absolute counts (already x nElectrons) */
  double max_coll_before_ss;
  double max_coll_after_ss;
  double req_integration_points;
  double req_ss_times;
  double req_abs_time;
  int errors_checked;
  double req_err_energy, req_err_flux_v, req_err_flux_d, req_err_bulk_v, req_err_bulk_d, req_err_power;
  int n_energy_cells, n_cos_cells, n_radial_cells, n_axial_cells, n_phases;
  int cylindrical;                 /* angle == 180 */
  double max_seconds;              /* wall-clock cap (<=0: none); used to bound baseline samples */
  long long max_sync_steps;        /* cap on synchronisation intervals (<=0: none) */
  long long mark_sync_step;        /* record collisions and wall time after this many intervals (<=0: none) */
  double mark_seconds;             /* or at the first interval that starts after this wall time (<=0: none) */
} lo_run_config;

typedef struct lo_run_result {
  double mean_energy, mean_energy_err;
  double flux_v[3], flux_v_err[3];
  double flux_d[9], flux_d_err[9];
  double bulk_v[3], bulk_v_err[3];
  double bulk_d[9], bulk_d_err[9];
  double real_collisions, null_collisions, coll_at_ss, null_at_ss;
  double ss_time, final_time, integration_points, trial_freq;
  double power_field, power_growth, power_balance_rel_err;
  double max_eedf_energy;
  double elapsed;
  long long sync_steps;
  double mark_real_collisions, mark_null_collisions, mark_elapsed;
  long long mark_sync_steps;       /* intervals begun before the mark */
  int status;                      /* 0 ok, 1 energy above elastic table, 2 capped by time/steps */
} lo_run_result;

/* rate (P), power_gain (P), power_loss (P), eedf (n_energy_cells), eedf_cells (n_energy_cells) may be NULL */
int lo_run(const lo_procs* pr, lo_fields* f, const lo_run_config* cfg, lo_run_result* res, double* rate,
           double* power_gain, double* power_loss, double* eedf, double* eedf_cells);

#ifdef __cplusplus
}
#endif
#endif
