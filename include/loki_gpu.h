/*
 * loki_gpu.h - C ABI of the GB300 electron Monte Carlo backend.
 *
 * The backend replaces the numerical core of LoKI-MC's BoltzmannMC engine
 * (Code/LoKI-MC/Sources/BoltzmannMC.C, Code/LoKI-MC/Headers/BoltzmannMC.h).
 * The reference has no foreign-function interface: the engine is a template
 * parameter of Setup<T> and Output<T> (Code/LoKI-MC/Sources/lokimc.C:14-41,
 * 78-80). Each entry point below names the reference routine or data it
 * stands in for; a C++ adapter class (BoltzmannMCGPU,
 * loki-mc_gb300/adapter/BoltzmannMCGPU.h) calls them from the reference's host
 * code.
 *
 * Conventions: plain C types, host pointers with explicit sizes, int status
 * returns (LGPU_OK = 0). A context owns all device memory; no pointer passed
 * in is retained after a call returns. One host thread per context.
 */
#ifndef LOKI_GPU_H
#define LOKI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference's failures call Message::error
 * (Code/LoKI-MC/Sources/Message.C:6-16), which logs and exits; the host maps
 * a non-zero status onto it. */
#define LGPU_OK 0
#define LGPU_ERR_BAD_ARG 1
#define LGPU_ERR_OOM 2
#define LGPU_ERR_ENERGY_ABOVE_TABLE 3 /* BoltzmannMC.C:1426-1430 */
#define LGPU_ERR_TIMEOUT 4
#define LGPU_ERR_CUDA 5
#define LGPU_ERR_STATE 6              /* call out of order */
#define LGPU_ERR_OVERFLOW 7           /* a device buffer or bounded loop ran out */
#define LGPU_ERR_NO_DEVICE 8

typedef struct lgpu_ctx lgpu_ctx;

/* Numerical settings of one context: the electronKinetics.numericsMC keys the
 * reference reads in its constructor (BoltzmannMC.h:262-376) plus the device
 * and seed. Collision-count limits are given as in the setup file, i.e. in
 * multiples of nElectrons (BoltzmannMC.h:295-303). */
typedef struct lgpu_config {
  int device;
  uint64_t seed;
  double n_electrons;               /* nElectrons */
  int n_interp;                     /* nInterpPoints (default 1e4) */
  int gas_temperature_effect;       /* 0 false, 1 true, 2 smartActivation */
  int sharing;                      /* ionizationOperatorType: 0 equalSharing, 1 oneTakesAll, 2 usingSDCS, 3 randomUniform */
  double init_temp_ratio;           /* initialElecTempOverGasTemp (default 0.01) */
  double min_coll_before_ss;        /* minCollisionsBeforeSteadyState (x nElectrons) */
  double max_coll_before_ss;        /* maxCollisionsBeforeSteadyState (x nElectrons) */
  double max_coll_after_ss;         /* maxCollisionsAfterSteadyState (x nElectrons) */
  double req_integration_points;    /* nIntegrationPoints (default 200) */
  double req_ss_times;              /* nIntegratedSSTimes */
  double req_abs_time;              /* integratedAbsoluteTime */
  int errors_checked;               /* relError present */
  double req_err_mean_energy, req_err_flux_v, req_err_flux_d, req_err_bulk_v, req_err_bulk_d, req_err_power;
  int n_energy_cells, n_cos_cells, n_radial_cells, n_axial_cells, n_phases;
  double sync_x;                    /* synchronizationTimeXMaxCollisionFrequency */
  int sync_oversampling;            /* synchronizationOverSampling */
  double max_seconds;               /* wall-clock cap of one solve (<= 0: none) */
  long long max_sync_steps;         /* interval cap of one solve (<= 0: none) */
  int advance_real_batch;           /* lanes of a warp with a pending real collision that start its
                                       collision turn (1..32); 0: 20 alone, tuned on line in a batch.
                                       Scheduling only: no result depends on it */
  int advance_queue;                /* secondaries a warp keeps in its own queue before it spills them to
                                       the global buffer the drain launch works off (1..32; 0: 32).
                                       Scheduling only: a small value exercises the spill path */
} lgpu_config;

/* Fills the reference's defaults (BoltzmannMC.h:50-76). */
void lgpu_config_default(lgpu_config* cfg);

/* One Monte Carlo process, flattened as BoltzmannMC::allocateEvaluateVariablesFirstTime
 * does (BoltzmannMC.C:29-271): every non-Effective collision once, a reversible
 * one followed immediately by its superelastic copy. */
typedef struct lgpu_process {
  int type;             /* 0 conservative, 1 ionization, 2 attachment (GeneralDefinitions.h:34-36) */
  int is_super;         /* superelastic copy of the process before it */
  int is_elastic;       /* Elastic collision (power bookkeeping) */
  int sampler;          /* 0 isotropic, 1 forward, 2 bornDipole, 3 surendra, 4 coulombScreen, 5 momentumConservationIonization */
  double sampler_p0, sampler_p1;
  double superw;        /* g_target / g_product (superelastic), else 0 */
  double emin, emax;    /* energyMinLimits / energyMaxLimits (eV) */
  double rel_dens;      /* relDensities */
  double mass;          /* targetMasses (kg) */
  double eloss;         /* energyLosses (eV), negative for superelastic */
  double wparam;        /* wParameters (eV) */
  int raw_len;          /* threshold-clipped raw cross section (crossSectionEnergies/Values) */
  const double* raw_e;
  const double* raw_v;
} lgpu_process;

typedef struct lgpu_gas {
  int first, last;      /* firstProcessIndexPerGas / lastProcessIndexPerGas */
  double fraction;      /* gasFractions */
} lgpu_gas;

/* Working conditions of one job (WorkingConditions.h:55-132). */
typedef struct lgpu_conditions {
  double gas_density;            /* m^-3 */
  double gas_temperature;        /* K */
  double reduced_field_td;       /* E/N (Td) */
  double field_angle_deg;        /* elecFieldAngle */
  double excitation_freq_hz;     /* excitationFrequency */
  double reduced_mag_field_hx;   /* B/N (Hx) */
} lgpu_conditions;

/* Results of one solve (BoltzmannMC.C:1484-1649 and the public members that
 * Output.h reads). */
typedef struct lgpu_result {
  double mean_energy, mean_energy_err;
  double flux_v[3], flux_v_err[3];
  double flux_d[9], flux_d_err[9];
  double bulk_v[3], bulk_v_err[3];
  double bulk_d[9], bulk_d_err[9];
  double power_field, power_growth, power_balance_rel_err;
  double ss_time, final_time;
  double trial_freq;
  double max_eedf_energy;
  double real_collisions, null_collisions;     /* totalCollisionCounter, nullCollisionCounter */
  double coll_at_ss, null_at_ss;               /* collisionCounterAtSS, nullCollisionCounterAtSS */
  long long integration_points;                /* nIntegrationPoints */
  long long sampling_points;                   /* nSamplingPoints */
  long long first_integration_index;
  long long sync_steps;
  double elapsed;                              /* seconds */
  int capped;                                  /* stopped by max_seconds / max_sync_steps */
} lgpu_result;

/* Progress report of lgpu_advance. */
typedef struct lgpu_step_report {
  double time;                /* absolute simulation time (s) */
  double trial_freq;          /* trialCollisionFrequency */
  double max_energy;          /* largest electron energy (eV) */
  double mean_energy;         /* ensemble mean at the last sample (eV) */
  double real_collisions;     /* cumulative */
  double null_collisions;     /* cumulative */
  long long sync_steps;       /* cumulative */
} lgpu_step_report;

/* Device-time accounting of the main advance kernel (CUDA events on the
 * context's stream). */
typedef struct lgpu_timing {
  double advance_ms;          /* summed duration of the main advance launches */
  long long advance_launches;
  double electron_steps;      /* electrons advanced by those launches */
  long long kernel_launches;  /* every kernel this context launched */
  double h2d_bytes;           /* host-to-device bytes copied by this context */
  double d2h_bytes;           /* device-to-host bytes copied by this context */
} lgpu_timing;

/* Context lifetime (replaces `new BoltzmannMC(setup)`, BoltzmannMC.h:244-380). */
int lgpu_create(const lgpu_config* cfg, lgpu_ctx** out);
int lgpu_destroy(lgpu_ctx* ctx);
/* Last error message of the context (empty when none). Returns the length. */
int lgpu_last_error(const lgpu_ctx* ctx, char* buf, size_t size);
/* The context's CUDA stream (a cudaStream_t), for callers that order work around it. */
void* lgpu_stream(lgpu_ctx* ctx);

/* Process set: the per-process arrays of BoltzmannMC.C:29-271 plus
 * energyMaxElastic (BoltzmannMC.C:157-159). Uploads the raw tables once. */
int lgpu_set_processes(lgpu_ctx* ctx, const lgpu_process* procs, int n_procs, const lgpu_gas* gases, int n_gases,
                       double energy_max_elastic);

/* Field and gas state of the next job (BoltzmannMC.C:428-489): E vector from
 * E/N and the angle, sqrt(2) for AC, cyclotron frequency from B/N. */
int lgpu_set_conditions(lgpu_ctx* ctx, const lgpu_conditions* cond);

/* Start ensemble (BoltzmannMC.C:491-516): positions zero, Maxwellian
 * velocities at initialElecTempOverGasTemp * Tg, first tables at twice the
 * largest energy, trial frequency at their maximum. Resets every tally. */
int lgpu_init_ensemble(lgpu_ctx* ctx);

/* n synchronisation intervals of the plain method (BoltzmannMC.C:617-688),
 * each followed by an ensemble sample; no steady-state logic. */
int lgpu_advance(lgpu_ctx* ctx, int n_intervals, lgpu_step_report* report);

/* The whole evaluateEEDF loop (BoltzmannMC.C:299-426): stepping, sampling,
 * steady-state detection, error control and the time averages. */
int lgpu_solve(lgpu_ctx* ctx, lgpu_result* result);

/* Per-process MC results after a solve: collisionCounters, averagedRateCoeffs
 * (BoltzmannMC.C:1627-1638), averagedPowerGain/LossProcesses
 * (BoltzmannMC.C:1640-1649). Any pointer may be NULL; each has n_procs entries. */
int lgpu_get_process_results(lgpu_ctx* ctx, unsigned long long* counts, double* rate, double* power_gain,
                             double* power_loss, int n_procs);

/* Time-averaged distributions after a solve (BoltzmannMC.C:1574-1605,
 * 1728-1741). Sizes follow the config; NULL skips an output.
 * eedf_cells/eedf/efadf/esadf: n_energy_cells; eadf: n_energy_cells x n_cos_cells;
 * evdf: n_radial_cells x n_axial_cells (row-major), radial/axial cell centres;
 * eedf_periodic: n_phases x n_energy_cells. */
int lgpu_get_distributions(lgpu_ctx* ctx, double* eedf_cells, double* eedf, double* efadf, double* esadf,
                           double* eadf, double* evdf, double* radial_cells, double* axial_cells,
                           double* eedf_periodic);

/* Phase-resolved averages of an AC solve (BoltzmannMC.C:1468-1481, 1728-1734):
 * per integration phase the number of samples and the averages of the mean
 * energy, flux and bulk velocity (x3) and flux and bulk diffusion (x9).
 * Arrays have n_phases rows; any pointer may be NULL. */
int lgpu_get_periodic(lgpu_ctx* ctx, double* n_points, double* mean_energy, double* flux_v, double* bulk_v,
                      double* flux_d, double* bulk_d);

/* Sampled time series (BoltzmannMC.h:124-175). which: 0 samplingTimes,
 * 1 meanEnergies, 2 meanPositions (x3), 3 meanVelocities (x3),
 * 4 fluxDiffusionCoeffs (x9), 5 positionCovariances (x9), 6 bulkVelocities (x3),
 * 7 bulkDiffusionCoeffs (x9). Returns the number of rows written (<= max_rows),
 * or a negative status. */
long long lgpu_get_series(lgpu_ctx* ctx, int which, double* out, long long max_rows);

int lgpu_get_timing(lgpu_ctx* ctx, lgpu_timing* timing);

/* ---- parity entry points: the production device functions on given inputs ---- */

/* Rebuilds the tables at a given maximum energy (BoltzmannMC.C:561-615) and
 * optionally returns them: grid/nu_tot/nu_max [M] in FP64, sig/cum [M*P] as the
 * FP32 values the kernels use. Any output may be NULL. */
int lgpu_build_tables(lgpu_ctx* ctx, double max_energy, double* nu_tot, double* nu_max, float* sig, float* cum);

/* Overrides the field the kernels use (the reference harness sets
 * electricField, excitationFrequency, reducedMagField and cyclotronFrequency
 * directly): E in V/m (amplitude), f in Hz, B/N in Hx (only compared with
 * zero), cyclotron frequency in rad/s. */
int lgpu_set_field_raw(lgpu_ctx* ctx, const double e_field[3], double freq_hz, double red_mag_hx,
                       double cyclotron);

/* n free flights (BoltzmannMC.C:804-905): start time t (s, absolute), length
 * dt, position and velocity [n x 3]. Outputs position, velocity, energy and
 * field energy gain. */
int lgpu_replay_flights(lgpu_ctx* ctx, int n, const double* t, const double* dt, const double* pos,
                        const double* vel, double* pos_out, double* vel_out, double* energy_out, double* gain_out);

/* n collision events (BoltzmannMC.C:907-1280) driven by recorded uniforms
 * (u_stride per event, used in order). out: n x 11 = chosen process (-1
 * null), velocity (3), energy, energy change, change / incident energy,
 * secondary velocity (3), secondary energy. used: uniforms consumed. */
int lgpu_replay_collisions(lgpu_ctx* ctx, int n, const double* nu_trial, const double* vel, const double* energy,
                           const double* uniforms, int u_stride, double* out, int* used);

/* The same events through the null test the advance kernels run
 * (BoltzmannMC.C:1033-1052 with a shortcut of this backend): the random
 * frequency is compared first with an upper bound of the total frequency over
 * a block of table rows, and the table row is read only when it lies below.
 * A bound below an interpolated frequency would turn a real collision into a
 * null one, so the outputs must equal lgpu_replay_collisions'. */
int lgpu_replay_collisions_coarse(lgpu_ctx* ctx, int n, const double* nu_trial, const double* vel,
                                  const double* energy, const double* uniforms, int u_stride, double* out, int* used);

/* ---- free flights without device allocation ----
 *
 * No counterpart in the reference. For callers that cannot allocate device
 * memory - a serving process that reserved the device up front, a host
 * application whose allocator owns the device, a pipeline stage that must not
 * allocate or synchronise on an allocation - this runs the same free-flight
 * kernel as lgpu_replay_flights without a context: inputs and outputs are the
 * caller's host arrays, staged through a static device array of at most 4096
 * flights (512 KiB, held on every GPU that loads the library until exit).
 * More than 4096 flights, or a device index outside [0, device count),
 * return LGPU_ERR_BAD_ARG. The first call on a device looks the array's
 * address up (cudaGetSymbolAddress) and keeps it for the process, so make that
 * call before any stream capture, and do not call this on a device after a
 * cudaDeviceReset there. Calls share the array: calls that overlap on the GPU
 * (from several host threads or streams) race. The caller's current device is
 * restored before returning. Synchronous: returns when the outputs are
 * written. The field arguments are those of lgpu_set_field_raw. */
int lgpu_replay_flights_noalloc(int device, const double e_field[3], double freq_hz, double red_mag_hx,
                                double cyclotron, int n, const double* t, const double* dt, const double* pos,
                                const double* vel, double* pos_out, double* vel_out, double* energy_out,
                                double* gain_out);

/* ---- batches: many swarm conditions per launch sequence ----
 *
 * No counterpart in the reference, which solves one condition per run
 * (lokimc.C:78-80); a sweep there is one run per setup. A batch solves many
 * contexts together: each context keeps its own ensemble, tables, tallies and
 * host control flow (the steps of lgpu_solve, BoltzmannMC.C:299-426), while
 * each synchronisation interval of all of them is one launch sequence (a CUDA
 * graph) over every context's electrons. Contexts are created on the batch's
 * device with processes and conditions set, and may differ in everything
 * (mixture, field, electron count, numerics). When more contexts are added
 * than the batch has slots, the rest start as running ones finish. After
 * lgpu_batch_run every lgpu_get_* call on a context works as after lgpu_solve;
 * lgpu_solve and lgpu_advance refuse a context while a batch holds it. */
typedef struct lgpu_batch lgpu_batch;

typedef struct lgpu_batch_report {
  long long intervals;          /* batched launch sequences */
  long long kernel_launches;    /* kernels launched for them */
  double elapsed;               /* wall time of the run (s) */
  double real_collisions;       /* summed over the contexts */
  double null_collisions;
  double advance_ms;            /* device time of the advance launches */
  double electron_steps;        /* electrons x intervals advanced */
  double h2d_bytes, d2h_bytes;  /* host<->device copies of the batched intervals */
  double host_ms;               /* host time of the intervals outside the wait for the device */
  double secondaries;           /* ionization secondaries created */
  double spilled;               /* of those, the ones a warp queue could not hold */
  double attached;              /* electrons removed by attachment */
  double real_batch;            /* collision-turn threshold in use (0 while it is being tuned) */
  double coarse_null_test;      /* 1: null tests try the block bounds first, 0: not, -1: being tuned */
  double regrids;               /* energy-grid re-builds, each overlapped with a batched interval the
                                   context sat out */
  double advance_threads;       /* launch shape of the advance chosen by the on-line tuner (0 while it is
                                   being tuned): threads per block, */
  double advance_blocks_per_sm; /* blocks per SM (the register budget), */
  double advance_chunk;         /* electrons a warp takes at a time, */
  double advance_stash;         /* records of a warp's collision stash (0: none; -1 while being tuned) */
} lgpu_batch_report;

int lgpu_batch_create(int device, int max_slots, lgpu_batch** out);
int lgpu_batch_destroy(lgpu_batch* batch);
int lgpu_batch_last_error(const lgpu_batch* batch, char* buf, size_t size);
/* Queues a context for the next lgpu_batch_run (not owned by the batch). */
int lgpu_batch_add(lgpu_batch* batch, lgpu_ctx* ctx);
/* Solves every queued context; results[i] and status[i] (an LGPU_* code) are
 * those of the i-th added context (n = number added). The batch is empty
 * afterwards. Returns LGPU_OK when the batch itself ran, whatever the
 * contexts' own status. */
int lgpu_batch_run(lgpu_batch* batch, lgpu_result* results, int* status, int n, lgpu_batch_report* report);
/* Interval-level control (benchmarks, callers with their own loop):
 * lgpu_batch_start starts the queued contexts that fit the slots (their
 * lgpu_init_ensemble), lgpu_batch_step runs n batched intervals (a context
 * whose stop criteria hold finishes and leaves its slot to a waiting one;
 * *running counts those still running), and a later lgpu_batch_run completes
 * what is left. report counts only this call. A context whose energy grid
 * must be re-built (the trial-frequency check, BoltzmannMC.C:617-688) sits
 * one batched interval out while the re-build runs beside it, so n batched
 * intervals advance it by n or fewer of its own; its own sequence of
 * intervals, and so its results, do not change. */
int lgpu_batch_start(lgpu_batch* batch);
int lgpu_batch_step(lgpu_batch* batch, int n, int* running, lgpu_batch_report* report);
/* The cudaStream_t all of the batch's work runs on. */
void* lgpu_batch_stream(lgpu_batch* batch);
/* Pins the advance's schedule instead of tuning it on line: launch shape
 * 0..5 (lgpu_batch_report's advance_threads .. advance_stash name it), the
 * collision-turn threshold (12, 16, 20, 24 or 28; a stash shape always takes
 * 32) and the coarse null test (0 or 1). shape -1 returns to on-line tuning.
 * The schedule changes no result: what an electron draws and decides does
 * not depend on it. */
int lgpu_batch_set_schedule(lgpu_batch* batch, int shape, int real_batch, int coarse);

/* ---- EEDF post-processing on the device ----
 *
 * The reference's end-of-job routines that read the EEDF, run in FP64 on the
 * device: the EEDF-convolved rate coefficient of every collision
 * (Collision::evaluateRateCoeff, Collision.C:355-397; called from
 * BoltzmannMC::evaluateRateCoeff, BoltzmannMC.C:2268-2384) and the two-term
 * swarm parameters (BoltzmannMC::evaluateSwarmParameters,
 * BoltzmannMC.C:2186-2266). They read each collision's own cross sections as
 * the reference's Collision holds them (the raw LXCat table, and the
 * momentum-transfer one its angular law gives, Collision.C:127-199), which
 * lgpu_set_twoterm takes per MC process, in the lgpu_set_processes order. */
typedef struct lgpu_twoterm_process {
  int kind;          /* 0 elastic, 1 inelastic (excitation, ionization, attachment, ...), 2 superelastic copy */
  int ion;           /* 1 ionization, 2 attachment, 0 otherwise */
  double density;    /* relative density of the target (of the product, for a superelastic copy) */
  double threshold;  /* eV (the forward collision's, for a superelastic copy) */
  double mass_ratio; /* m_e / M of the target gas (used for elastic collisions) */
  double stat_ratio; /* g_target / g_product of a reversible collision (used by its superelastic copy) */
  int n_int, n_mom;  /* points of the raw integral and momentum-transfer tables (n_mom 0: the integral one) */
  const double* int_e; /* eV, increasing */
  const double* int_v; /* m^2 */
  const double* mom_e;
  const double* mom_v;
} lgpu_twoterm_process;
int lgpu_set_twoterm(lgpu_ctx* ctx, const lgpu_twoterm_process* p, int n);

/* The two-term swarm parameters, named as the reference's swarmParam keys. */
typedef struct lgpu_eedf_params {
  double tot_ion_rate, tot_att_rate;       /* totalIonRateCoeff, totalAttRateCoeff (m^3/s) */
  double mom_transf_freq;                  /* momTransfFreq (1/s) */
  double energy_relax_freq;                /* energyRelaxFreq */
  double energy_relax_freq_classic;        /* energyRelaxFreqClassic */
  double red_diff_energy, red_mob_energy;  /* redDiffCoeffEnergy_eedf, redMobCoeffEnergy_eedf */
  double red_diff, red_mob_dc;             /* redDiffCoeff_eedf, redMobCoeff_DC_eedf */
  double charac_energy;                    /* characEnergy_eedf (eV) */
  double red_mob_xx_re, red_mob_xx_im;     /* redMobCoeff_xx_{real,imag}_eedf */
  double red_mob_xy_re, red_mob_xy_im;     /* redMobCoeff_xy_{real,imag}_eedf */
  double red_mob_zz_re, red_mob_zz_im;     /* redMobCoeff_zz_{real,imag}_eedf */
} lgpu_eedf_params;
/* eedf NULL: the context's own time-averaged EEDF (after lgpu_solve or a
 * batch); else n_cells values on cells of width max_energy / n_cells (the
 * grid of Grid::updateMaxValue, Grid.C:44-53). The field frequencies and the
 * gas density are the context's conditions. rate[n] (n = the process count;
 * may be NULL): each MC process's EEDF-convolved rate coefficient (m^3/s),
 * the superelastic one for a superelastic copy. */
int lgpu_eedf_postprocess(lgpu_ctx* ctx, const double* eedf, int n_cells, double max_energy, lgpu_eedf_params* out,
                          double* rate, int n);
/* The EEDF-convolved rate coefficients alone, of n_eedf EEDFs given as rows
 * of n_cells (rate[n_eedf * n]); eedf NULL: the context's per-phase EEDFs of
 * an AC run (n_eedf = config.n_phases; BoltzmannMC.C:2276-2330, each phase's
 * EEDF normalised as BoltzmannMC.C:1736-1740). */
int lgpu_eedf_rates(lgpu_ctx* ctx, const double* eedf, int n_eedf, int n_cells, double max_energy, double* rate,
                    int n);

/* ---- serving: continuous batching of swarm jobs ----
 *
 * No counterpart in the reference. A server owns one device and one thread
 * that runs a batch without pause: submitted jobs wait in arrival order and
 * are admitted while a slot is free and their device footprint (ensemble,
 * secondary buffers, tables, tallies) fits the memory budget; every
 * synchronisation interval advances all admitted jobs in one launch sequence;
 * a job leaves when its own stop criteria hold, its results are copied to the
 * host and its device memory is freed for the next admission. Jobs are
 * independent: each result is that of lgpu_solve on the same input, within
 * the statistical tolerance of a Monte Carlo run. Submission is thread-safe. */
typedef struct lgpu_server lgpu_server;

typedef struct lgpu_job {
  lgpu_config config;             /* config.device is ignored: the server's device */
  const lgpu_process* procs;      /* copied at submission, raw cross sections included */
  int n_procs;
  const lgpu_gas* gases;
  int n_gases;
  double emax_elastic;            /* as lgpu_set_processes */
  lgpu_conditions conditions;
  const lgpu_twoterm_process* twoterm; /* n_procs entries, copied at submission, or NULL: with them the
                                          server post-processes the job's EEDF on the device at its end
                                          (lgpu_server_job_eedf) */
} lgpu_job;

#define LGPU_JOB_QUEUED 0
#define LGPU_JOB_RUNNING 1
#define LGPU_JOB_DONE 2
#define LGPU_JOB_FAILED 3
#define LGPU_JOB_CANCELLED 4

typedef struct lgpu_job_status {
  int state;                      /* LGPU_JOB_* */
  int status;                     /* LGPU_* code of a failed job */
  double submit_time;             /* seconds since the server started */
  double start_time;              /* admission */
  double end_time;                /* results available */
  double footprint_bytes;         /* device memory the job held */
  lgpu_result result;
  char error[256];                /* message of a failed job */
} lgpu_job_status;

typedef struct lgpu_server_report {
  long long submitted, completed, failed, running, queued;
  long long intervals;            /* batched launch sequences so far */
  double real_collisions;         /* of completed jobs */
  double null_collisions;
  double busy_seconds;            /* wall time with at least one job admitted */
  double peak_footprint_bytes;
} lgpu_server_report;

/* max_slots: jobs advanced together; memory_budget_bytes: device memory the
 * admitted jobs may hold (0: 80% of the free memory at start). */
int lgpu_server_start(int device, int max_slots, double memory_budget_bytes, lgpu_server** out);
int lgpu_server_submit(lgpu_server* server, const lgpu_job* job, long long* job_id);
int lgpu_server_poll(lgpu_server* server, long long job_id, lgpu_job_status* status);
/* Blocks until the job is done, failed or cancelled, or timeout_s passes
 * (LGPU_ERR_TIMEOUT; timeout_s <= 0 waits without limit). */
int lgpu_server_wait(lgpu_server* server, long long job_id, double timeout_s, lgpu_job_status* status);
/* Per-process collision counts and rate coefficients of a finished job
 * (as lgpu_get_process_results; n = the job's process count). */
int lgpu_server_job_rates(lgpu_server* server, long long job_id, unsigned long long* counts, double* rate, int n);
/* The EEDF post-processing of a finished job submitted with two-term inputs
 * (lgpu_job.twoterm; a request's jobs carry them): its two-term swarm
 * parameters and each process's EEDF-convolved rate coefficient, computed on
 * the device at the job's end. LGPU_ERR_STATE for other jobs. */
int lgpu_server_job_eedf(lgpu_server* server, long long job_id, lgpu_eedf_params* params, double* rate, int n);
/* A queued job is dropped; a running one stops at its next interval. */
int lgpu_server_cancel(lgpu_server* server, long long job_id);
/* Drops the record of a finished (done, failed or cancelled) job: its status,
 * results and rates are no longer available (LGPU_ERR_STATE for a job still
 * queued or running). A long-running server keeps the records of its last
 * 65536 finished jobs in any case and drops older ones. */
int lgpu_server_forget(lgpu_server* server, long long job_id);
int lgpu_server_report_get(lgpu_server* server, lgpu_server_report* report);
int lgpu_server_last_error(const lgpu_server* server, char* buf, size_t size);
/* Cancels what is left, joins the thread, frees the device memory. */
int lgpu_server_stop(lgpu_server* server);

/* ---- requests: jobs from the reference's own input files ----
 *
 * The reference reads a setup file (.in) and the LXCat files it names
 * (Parse.C:43-295, Setup.h:229-459) and flattens the collisions into its MC
 * processes (BoltzmannMC.C:29-271). lgpu_request_parse does the same on the
 * files' texts, with no file access and no reference code, so that a server
 * can admit a request as a user of the reference writes it: working
 * conditions (one of E/N, B/N, field angle, frequency may be a vector: one job
 * per entry), numericsMC keys, gas masses, fractions and OPB parameters,
 * state energies, statistical weights and populations (values or
 * boltzmannPopulation@T over a family "G(X,v=*)"), anisotropic scattering
 * "group;gas;type;law;params" lines. Values are arithmetic expressions as in
 * the reference's setup files. An input it does not read (for instance a
 * momentum-transfer cross section with an anisotropic law) fails with
 * LGPU_ERR_BAD_ARG and a message in err. */
typedef struct lgpu_request lgpu_request;
int lgpu_request_parse(const char* setup_text, int n_files, const char* const* file_names,
                       const char* const* file_texts, lgpu_request** out, char* err, size_t err_size);
/* Number of jobs of the request. */
int lgpu_request_jobs(const lgpu_request* req);
/* The k-th job, ready for lgpu_server_submit (its pointers stay valid while
 * the request lives). */
int lgpu_request_job(const lgpu_request* req, int k, lgpu_job* job);
void lgpu_request_free(lgpu_request* req);
/* Submits every job of the request; job_ids has room for lgpu_request_jobs. */
int lgpu_server_submit_request(lgpu_server* server, const lgpu_request* req, long long* job_ids, int max_ids);

#ifdef __cplusplus
}
#endif
#endif
