/*
 * loki_oracle.c - CPU restatement of LoKI-MC's electron Monte Carlo engine.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT: the results the GPU path is compared with
 * and the CPU baseline of the benchmark. Compiled with -ffp-contract=off so that, like
 * the reference built on x86-64, no a*b+c is fused.
 *
 * Each routine cites the reference routine it restates (file:line under the
 * reference's Code/ directory) and keeps its operation order.
 */
#include "loki_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Constant.h:6-8, 23 */
#define LO_KB 1.38064852e-23
#define LO_QE 1.6021766208e-19
#define LO_ME 9.10938356e-31
#define LO_NON_DEF (-123456789.0)
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ RNG */

static uint64_t splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

void lo_rng_seed(lo_rng* r, uint64_t seed, uint64_t stream) {
  uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ULL);
  for (int i = 0; i < 4; ++i) r->s[i] = splitmix64(&x);
  r->replay = NULL;
  r->n = r->pos = 0;
  r->overrun = 0;
}

void lo_rng_replay(lo_rng* r, const double* u, size_t n) {
  r->replay = u;
  r->n = n;
  r->pos = 0;
  r->overrun = 0;
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static double raw_uniform(lo_rng* r) {
  if (r->replay) {
    if (r->pos < r->n) return r->replay[r->pos++];
    r->overrun = 1;
    return 0.5;
  }
  uint64_t* s = r->s;
  uint64_t result = rotl(s[1] * 5, 7) * 9;
  uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
  return (double)(result >> 11) * 0x1.0p-53; /* [0, 1) */
}

/* MathFunctions.C:31-43: redraw excluded endpoints */
double lo_uniform(lo_rng* r, int include_zero, int include_one) {
  double u = raw_uniform(r);
  while ((!include_zero && u == 0) || (!include_one && u == 1)) u = raw_uniform(r);
  return u;
}

/* MathFunctions.C:54-59: Box-Muller on four uniforms */
static void normal3(lo_rng* r, double* out) {
  double r1 = lo_uniform(r, 0, 1), r2 = lo_uniform(r, 0, 1), r3 = lo_uniform(r, 0, 1), r4 = lo_uniform(r, 0, 1);
  double a = sqrt(-2.0 * log(r1)), b = 2.0 * M_PI * r2;
  out[0] = a * cos(b);
  out[1] = a * sin(b);
  out[2] = sqrt(-2.0 * log(r3)) * cos(2.0 * M_PI * r4);
}

/* Eigen's squaredNorm of a 3-vector sums (x^2 + y^2) + z^2 */
static inline double sqnorm3(const double* v) { return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]; }

/* --------------------------------------------------------- interpolation */

/* Linear interpolant of GSL's gsl_interp_linear over the raw table: the
 * bracketing index by bisection (largest i with x_i <= x, clamped to n-2),
 * then y_i + (x - x_i)/(x_{i+1} - x_i)*(y_{i+1} - y_i). Callers guarantee
 * x_0 <= x <= x_{n-1} (BoltzmannMC.C:585, 597). */
double lo_interp(const lo_procs* pr, int p, double x) {
  const double* xs = pr->raw_e + pr->raw_off[p];
  const double* ys = pr->raw_v + pr->raw_off[p];
  size_t n = (size_t)pr->raw_len[p];
  size_t lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    size_t mid = (hi + lo) / 2;
    if (xs[mid] > x) hi = mid; else lo = mid;
  }
  double dx = xs[lo + 1] - xs[lo];
  return ys[lo] + (x - xs[lo]) / dx * (ys[lo + 1] - ys[lo]);
}

/* BoltzmannMC.C:561-615 */
void lo_build_tables(lo_procs* pr, const lo_fields* f, double max_energy) {
  if (max_energy == pr->max_interp) return;
  const int M = pr->M, P = pr->P;
  pr->max_interp = max_energy;
  pr->step = max_energy / (double)(M - 1);
  double max_freq = 0;
  for (int i = 0; i < M; ++i) {
    double energy = i * pr->step;
    pr->grid[i] = energy;
    double cur = 0;
    for (int p = 0; p < P; ++p) {
      double value;
      if (pr->is_super[p]) {
        if (energy > pr->emin[p] && energy <= pr->emax[p]) {
          /* Klein-Rosseland: (g_i/g_f)(1 + thr/u) sigma_{i,f}(u + thr) */
          value = pr->superw[p] * (1.0 + pr->emin[p - 1] / energy) * lo_interp(pr, p - 1, energy + pr->emin[p - 1]) *
                  pr->rel_dens[p];
        } else {
          value = 0;
        }
      } else {
        if (energy >= pr->emin[p] && energy <= pr->emax[p]) {
          value = lo_interp(pr, p, energy) * pr->rel_dens[p];
        } else {
          value = 0;
        }
      }
      pr->sig[(size_t)i * P + p] = value;
      cur += value;
      pr->cum[(size_t)i * P + p] = cur;
    }
    cur *= f->N * sqrt(energy * 2.0 * LO_QE / LO_ME);
    pr->nu_tot[i] = cur;
    max_freq = fmax(cur, max_freq);
    pr->nu_max[i] = max_freq;
  }
}

/* ------------------------------------------------------------ free flight */

/* BoltzmannMC.C:804-905 */
void lo_accelerate(const lo_fields* f, double t, double dt, double* pos, double* vel, double* energy, double* gain) {
  double previous = *energy;
  const double e = LO_QE, me = LO_ME;
  const double* E = f->E;
  if (f->red_mag == 0) {
    if (f->freq_hz == 0) {
      for (int k = 0; k < 3; ++k) pos[k] = pos[k] + (vel[k] * dt + f->acc[k] * (0.5 * dt * dt));
      for (int k = 0; k < 3; ++k) vel[k] = vel[k] + f->acc[k] * dt;
    } else {
      double w = f->omega;
      double phi = w * t;
      double sinPhi = sin(phi), cosPhi = cos(phi);
      double wdt = w * dt;
      double phase = wdt + phi;
      double sinPhase = sin(phase), cosPhase = cos(phase);
      double e_me_w = e / (me * w);
      double aux1 = e_me_w / w * (cosPhase + wdt * sinPhi - cosPhi);
      double aux2 = e_me_w * (sinPhi - sinPhase);
      pos[0] += vel[0] * dt + E[0] * aux1;
      pos[1] += vel[1] * dt;
      pos[2] += vel[2] * dt + E[2] * aux1;
      vel[0] += E[0] * aux2;
      vel[2] += E[2] * aux2;
    }
  } else {
    double vx0 = vel[0], vy0 = vel[1], vz0 = vel[2];
    if (f->freq_hz == 0) {
      double W = f->omega_c;
      double Wdt = W * dt;
      double sinW = sin(Wdt), cosW = cos(Wdt);
      double sinW_W = sinW / W;
      double aux2 = (cosW - 1.0) / W;
      double vExCyc = e * E[0] / (me * W);
      double az = e * E[2] / me;
      pos[0] += vx0 * sinW_W + (vy0 + vExCyc) * aux2;
      pos[1] += -vx0 * aux2 + vy0 * sinW_W + vExCyc * (sinW_W - dt);
      pos[2] += vz0 * dt - 0.5 * az * dt * dt;
      vel[0] = vx0 * cosW - vy0 * sinW - vExCyc * sinW;
      vel[1] = vx0 * sinW + vy0 * cosW + vExCyc * (cosW - 1.0);
      vel[2] = vz0 - az * dt;
    } else if (fabs(f->omega - f->omega_c) / f->omega < 1E-6) {
      /* electron cyclotron resonance */
      double W = f->omega_c;
      double phi = W * t;
      double sinPhi = sin(phi), cosPhi = cos(phi);
      double Wdt = W * dt;
      double sinW = sin(Wdt), cosW = cos(Wdt);
      double phase = Wdt + phi;
      double sinPhase = sin(phase), cosPhase = cos(phase);
      double cosOpp = cos(phi - Wdt);
      double e_me_W = e / (me * W);
      double vExCyc = e_me_W * E[0];
      double vEzAC = e_me_W * E[2];
      double sinW_W = sinW / W;
      double cosWm1_W = (cosW - 1.0) / W;
      double cosPhase_W = cosPhase / W;
      pos[0] += vx0 * sinW_W + vy0 * cosWm1_W - 0.25 * vExCyc * (cosPhase_W - cosOpp / W + 2.0 * dt * sinPhase);
      pos[1] += -vx0 * cosWm1_W + vy0 * sinW_W + 0.5 * vExCyc * (dt * cosPhase_W - 2.0 * cosWm1_W * sinPhi - cosPhi * sinW_W);
      pos[2] += vz0 * dt + vEzAC * (cosPhase_W - cosPhi / W + dt * sinPhi);
      vel[0] = vx0 * cosW - vy0 * sinW - 0.5 * vExCyc * (Wdt * cosPhase + cosPhi * sinW);
      vel[1] = vx0 * sinW + vy0 * cosW - 0.5 * vExCyc * (Wdt * cosW * sinPhi + (Wdt * cosPhi - sinPhi) * sinW);
      vel[2] = vz0 + vEzAC * (sinPhi - sinPhase);
    } else {
      double w = f->omega, W = f->omega_c;
      double phi = w * t;
      double sinPhi = sin(phi), cosPhi = cos(phi);
      double wdt = w * dt;
      double sinw = sin(wdt), cosw = cos(wdt);
      double phase = wdt + phi;
      double sinPhase = sin(phase), cosPhase = cos(phase);
      double Wdt = W * dt;
      double sinW = sin(Wdt), cosW = cos(Wdt);
      double w2 = w * w, W2 = W * W, w2mW2 = w2 - W2;
      double vExCyc = e / (me * W) * E[0];
      double vEzAC = e / (me * w) * E[2];
      double vExCyc_d = vExCyc / w2mW2;
      double WvExCyc_d = W * vExCyc_d;
      double sinW_W = sinW / W;
      double cosWm1_W = (cosW - 1.0) / W;
      double wSinPhi = w * sinPhi;
      pos[0] += vx0 * sinW_W + vy0 * cosWm1_W + WvExCyc_d * (cosPhi * (cosw - cosW) + (wSinPhi * sinW_W - sinPhi * sinw));
      pos[1] += -vx0 * cosWm1_W + vy0 * sinW_W - vExCyc_d / w * ((W2 + w2 * cosW - w2) * sinPhi + W2 * (w * cosPhi * sinW_W - sinPhase));
      pos[2] += vz0 * dt + vEzAC * ((cosPhase - cosPhi) / w + dt * sinPhi);
      vel[0] = vx0 * cosW - vy0 * sinW + WvExCyc_d * w * (cosW * sinPhi - sinPhase + cosPhi / w * W * sinW);
      vel[1] = vx0 * sinW + vy0 * cosW + vExCyc_d * W2 * (cosPhase - cosPhi * cosW + wSinPhi * sinW_W);
      vel[2] = vz0 + vEzAC * (sinPhi - sinPhase);
    }
  }
  *energy = 0.5 * LO_ME * sqnorm3(vel) / LO_QE;
  *gain = *energy - previous;
}

/* BoltzmannMC.C:765-802 */
double lo_max_accel_energy(const lo_fields* f, double initial_energy, double dt) {
  double e = LO_QE, me = LO_ME, e_me = e / me;
  double Ex0 = fabs(f->E[0]), Ez0 = fabs(f->E[2]);
  double Ex02 = Ex0 * Ex0, Ez02 = Ez0 * Ez0, E02 = Ex02 + Ez02, E0 = sqrt(E02);
  double v0 = sqrt(initial_energy * e * 2.0 / me);
  double w = f->omega, W = f->omega_c;
  double gain = (E0 * v0 + 0.5 * e_me * E02 * dt) * dt;
  if (W == 0) {
    if (w != 0) gain = fmin(gain, 2.0 / w * (e_me * E02 / w + v0 * (Ex0 + Ez0)));
  } else {
    if (w == 0) {
      gain = fmin(gain, 0.5 * e_me * Ez02 * dt * dt + (2.0 * e_me * Ex02 / W + 3.0 * v0 * Ex0) / W + v0 * dt * Ez0);
    } else if (fabs(w - W) / w < 1E-6) {
      double W2 = W * W;
      gain = fmin(gain, 2.0 * e_me * Ez02 / W2 + e_me * Ex02 / (8.0 * W2) * (4.0 + W * dt * (2.0 + W * dt)) +
                            (v0 * dt + v0 / W) * Ex0 + 2.0 * v0 * Ez0 / W);
    } else {
      double w2 = w * w, W2 = W * W, d = w2 - W2;
      gain = fmin(gain, 2.0 * e_me * Ez02 / w2 + 0.5 * e_me * Ex02 / (d * d) * (5.0 * w2 + 8.0 * w * W + 5.0 * W * W) +
                            3.0 * v0 * Ex0 / fabs(w - W) + 2.0 * v0 * Ez0 / w);
    }
  }
  return initial_energy + gain;
}

/* ---------------------------------------------------------------- kinematics */

/* MathFunctions.C:143-163 */
static void cart2sph(const double* v, double* norm, double* sT, double* cT, double* sP, double* cP) {
  double x = v[0], y = v[1], z = v[2];
  double x2y2 = x * x + y * y;
  double nxy = sqrt(x2y2);
  *norm = sqrt(x2y2 + z * z);
  *sT = nxy / *norm;
  *cT = z / *norm;
  if (nxy != 0) {
    *sP = y / nxy;
    *cP = x / nxy;
  } else {
    *sP = 1;
    *cP = 0;
  }
}

/* MathFunctions.C:129-141 (Yousfi 1994) */
static void euler(double sinChi, double cosChi, double sinEta, double cosEta, double sinTheta, double cosTheta,
                  double sinPhi, double cosPhi, double* out) {
  double sCsE = sinChi * sinEta;
  double aux = sinChi * cosEta * cosTheta + cosChi * sinTheta;
  out[0] = -sCsE * sinPhi + aux * cosPhi;
  out[1] = sCsE * cosPhi + aux * sinPhi;
  out[2] = -sinChi * cosEta * sinTheta + cosChi * cosTheta;
}

/* AngularScatteringFunctions.h:27-74 */
static double sample_cos_chi(const lo_procs* pr, int p, double energy, double energy_after, lo_rng* rng) {
  switch (pr->sampler[p]) {
    case 0:
      return 1.0 - 2.0 * lo_uniform(rng, 1, 1);
    case 1:
      return 1;
    case 2: {
      double eloss = pr->eloss[p];
      double s = sqrt(energy_after) + sqrt(energy);
      double ratio = eloss / pow(s, 2);
      double r2 = ratio * ratio;
      return 1.0 + 2.0 * r2 / (1.0 - r2) * (1.0 - pow(r2, -lo_uniform(rng, 1, 1)));
    }
    case 3:
      return (2.0 + energy - 2.0 * pow(1.0 + energy, lo_uniform(rng, 1, 1))) / energy;
    case 4: {
      double eps = (pr->sampler_p0[p] == 0) ? energy : energy_after;
      double sp = pr->sampler_p1[p] / eps;
      double R = lo_uniform(rng, 1, 1);
      return (sp + 1.0 - (2.0 * sp + 1.0) * R) / (sp + 1.0 - R);
    }
    default:
      return 1.0 - 2.0 * lo_uniform(rng, 1, 1);
  }
}

static inline int thermal_branch(const lo_fields* f, double energy) {
  return f->gas_temp_effect == 1 || (f->gas_temp_effect == 2 && energy < 20.0 * f->gas_energy);
}

/* BoltzmannMC.C:1115-1193 */
static void conservative(const lo_procs* pr, const lo_fields* f, int p, const double* tv, double* vel, double* energy,
                         lo_rng* rng, lo_coll_out* out) {
  double M = pr->mass[p], rm = pr->red_mass[p], eloss = pr->eloss[p];
  double incident = *energy;
  if (thermal_branch(f, incident)) {
    double rel[3] = {vel[0] - tv[0], vel[1] - tv[1], vel[2] - tv[2]};
    double rs, sT, cT, sP, cP;
    cart2sph(rel, &rs, &sT, &cT, &sP, &cP);
    double relE = 0.5 * rm * rs * rs / LO_QE;
    double relEA = relE - eloss;
    if (relEA <= 0) {
      out->chosen = -1;
      return;
    }
    double cosChi = sample_cos_chi(pr, p, relE, relEA, rng);
    double sinChi = sqrt(1.0 - cosChi * cosChi);
    double eta = 2.0 * M_PI * lo_uniform(rng, 0, 1);
    double sE = sin(eta), cE = cos(eta);
    double ver[3];
    euler(sinChi, cosChi, sE, cE, sT, cT, sP, cP, ver);
    double s = sqrt(rs * rs - 2.0 / rm * eloss * LO_QE);
    for (int k = 0; k < 3; ++k) {
      double relA = s * ver[k];
      vel[k] = M / (LO_ME + M) * relA + (LO_ME * vel[k] + M * tv[k]) / (LO_ME + M);
    }
  } else {
    double speed, sT, cT, sP, cP;
    cart2sph(vel, &speed, &sT, &cT, &sP, &cP);
    double eA = incident - eloss;
    if (eA <= 0) {
      out->chosen = -1;
      return;
    }
    double cosChi = sample_cos_chi(pr, p, incident, eA, rng);
    double sinChi = sqrt(1.0 - cosChi * cosChi);
    double eta = 2.0 * M_PI * lo_uniform(rng, 0, 1);
    double sE = sin(eta), cE = cos(eta);
    double ver[3];
    euler(sinChi, cosChi, sE, cE, sT, cT, sP, cP, ver);
    double s = sqrt((speed * speed - 2.0 / LO_ME * eloss * LO_QE) * (1.0 - 2.0 * rm / (LO_ME + M) * (1.0 - cosChi)));
    for (int k = 0; k < 3; ++k) vel[k] = s * ver[k];
  }
  *energy = 0.5 * LO_ME * sqnorm3(vel) / LO_QE;
  out->dE = *energy - incident;
  out->dE_over_E = out->dE / incident;
}

/* BoltzmannMC.C:1195-1272 */
static void ionization(const lo_procs* pr, const lo_fields* f, int p, double* vel, double* energy, lo_rng* rng,
                       lo_coll_out* out) {
  double incident = *energy;
  double thr = pr->eloss[p];
  if (incident < thr) {
    out->chosen = -1;
    return;
  }
  double speed, sT, cT, sP, cP;
  cart2sph(vel, &speed, &sT, &cT, &sP, &cP);
  double net = incident - thr;
  double ej;
  if (f->sharing == 2) {
    double w = pr->wparam[p];
    ej = w * tan(lo_uniform(rng, 1, 1) * atan(net / (2.0 * w)));
  } else if (f->sharing == 3) {
    ej = lo_uniform(rng, 1, 1) * net;
  } else {
    ej = f->sharing_factor * net;
  }
  double scat = net - ej;
  double sinChiS, cosChiS, sinChiE, cosChiE, sinEtaS, cosEtaS, sinEtaE, cosEtaE;
  if (pr->sampler[p] == 5) {
    cosChiS = sqrt(scat / net);
    sinChiS = sqrt(1.0 - cosChiS * cosChiS);
    double eta = 2.0 * M_PI * lo_uniform(rng, 0, 1);
    sinEtaS = sin(eta);
    cosEtaS = cos(eta);
    cosChiE = sqrt(ej / net);
    sinChiE = sqrt(1.0 - cosChiE * cosChiE);
    sinEtaE = -sinEtaS;
    cosEtaE = -cosEtaS;
  } else {
    cosChiS = sample_cos_chi(pr, p, incident, scat, rng);
    sinChiS = sqrt(1.0 - cosChiS * cosChiS);
    double eta = 2.0 * M_PI * lo_uniform(rng, 0, 1);
    sinEtaS = sin(eta);
    cosEtaS = cos(eta);
    cosChiE = sample_cos_chi(pr, p, incident, ej, rng);
    sinChiE = sqrt(1.0 - cosChiE * cosChiE);
    double etaE = 2.0 * M_PI * lo_uniform(rng, 0, 1);
    sinEtaE = sin(etaE);
    cosEtaE = cos(etaE);
  }
  double ver[3];
  euler(sinChiS, cosChiS, sinEtaS, cosEtaS, sT, cT, sP, cP, ver);
  double s = sqrt(2.0 * scat * LO_QE / LO_ME);
  for (int k = 0; k < 3; ++k) vel[k] = s * ver[k];
  euler(sinChiE, cosChiE, sinEtaE, cosEtaE, sT, cT, sP, cP, ver);
  double se = sqrt(2.0 * ej * LO_QE / LO_ME);
  for (int k = 0; k < 3; ++k) out->ej_vel[k] = se * ver[k];
  out->ej_energy = ej;
  *energy = scat;
  out->dE = -thr;
  out->dE_over_E = -thr / incident;
}

/* BoltzmannMC.C:907-1113 */
void lo_collide(const lo_procs* pr, const lo_fields* f, double nu_trial, const double* vel_in, double energy_in,
                lo_rng* rng, lo_coll_out* out) {
  const int M = pr->M, P = pr->P;
  double vel[3] = {vel_in[0], vel_in[1], vel_in[2]};
  double energy = energy_in;
  double tv[3] = {0, 0, 0};
  int chosen = -1;
  out->dE = 0;
  out->dE_over_E = 0;
  out->ej_vel[0] = out->ej_vel[1] = out->ej_vel[2] = 0;
  out->ej_energy = 0;

  if (thermal_branch(f, energy)) {
    double versor[3];
    normal3(rng, versor);
    double rcs = nu_trial * lo_uniform(rng, 0, 1) / f->N;
    double prev = 0;
    for (int g = 0; g < pr->G && chosen == -1; ++g) {
      if (pr->gas_frac[g] == 0) continue;
      int L = pr->gas_first[g], R = pr->gas_last[g];
      double sd = sqrt(LO_KB * f->Tg / pr->mass[L]);
      for (int k = 0; k < 3; ++k) tv[k] = versor[k] * sd;
      double rel[3] = {vel[0] - tv[0], vel[1] - tv[1], vel[2] - tv[2]};
      double rs = sqrt(sqnorm3(rel));
      double reos = 0.5 * pr->red_mass[L] * rs * rs / LO_QE / pr->step;
      int i1 = (int)fmin(reos, M - 1);
      int i2 = (int)fmin(i1 + 1, M - 1);
      double w1 = (double)i2 - reos;
      w1 = (w1 < 0) ? 0.0 : 1.0; /* BoltzmannMC.C:959-967: 0/1 row weights */
      double w2 = 1.0 - w1;
      const double* c1 = pr->cum + (size_t)i1 * P;
      const double* c2 = pr->cum + (size_t)i2 * P;
      const double* s1 = pr->sig + (size_t)i1 * P;
      const double* s2 = pr->sig + (size_t)i2 * P;
      double ref = 0;
      if (L > 0) ref = w1 * c1[L - 1] + w2 * c2[L - 1];
      double lim = prev + (w1 * c1[R] + w2 * c2[R] - ref) * rs;
      if (rcs > lim) {
        prev = lim;
        continue;
      }
      while (L != R) {
        int t = (L + R) / 2;
        double tvl = prev + (w1 * c1[t] + w2 * c2[t] - ref) * rs;
        if (rcs < tvl) R = t;
        else if (rcs > tvl) L = t + 1;
        else { chosen = t; break; }
      }
      if (L == R) chosen = L;
      while (w1 * s1[chosen] == 0 && w2 * s2[chosen] == 0) --chosen;
    }
    if (chosen == -1) {
      out->chosen = -1;
      goto finish;
    }
  } else {
    double r = nu_trial * lo_uniform(rng, 0, 1);
    double eos = energy / pr->step;
    int i1 = (int)fmin(eos, M - 1);
    int i2 = (int)fmin(i1 + 1, M - 1);
    double w1 = (double)i2 - eos;
    if (w1 < 0) w1 = 0.0;
    double w2 = 1.0 - w1;
    if (r > w1 * pr->nu_tot[i1] + w2 * pr->nu_tot[i2]) {
      out->chosen = -1;
      goto finish;
    }
    const double* c1 = pr->cum + (size_t)i1 * P;
    const double* c2 = pr->cum + (size_t)i2 * P;
    const double* s1 = pr->sig + (size_t)i1 * P;
    const double* s2 = pr->sig + (size_t)i2 * P;
    double rcs = r / f->N / sqrt(sqnorm3(vel));
    int L = 0, R = P - 1;
    while (L != R) {
      int t = (L + R) / 2;
      double tvl = w1 * c1[t] + w2 * c2[t];
      if (rcs < tvl) R = t;
      else if (rcs > tvl) L = t + 1;
      else { chosen = t; break; }
    }
    if (L == R) chosen = L;
    while (w1 * s1[chosen] == 0 && w2 * s2[chosen] == 0) --chosen;
  }

  out->chosen = chosen;
  if (pr->ptype[chosen] == 0) {
    conservative(pr, f, chosen, tv, vel, &energy, rng, out);
  } else if (pr->ptype[chosen] == 1) {
    ionization(pr, f, chosen, vel, &energy, rng, out);
  } else {
    out->dE = -energy; /* BoltzmannMC.C:1274-1280 */
    out->dE_over_E = -1;
  }
finish:
  for (int k = 0; k < 3; ++k) out->vel[k] = vel[k];
  out->energy = energy;
}

/* ---------------------------------------------------------------- statistics */

/* MathFunctions.C:211-231: 50-block batch means */
double lo_statistical_error(const double* a, int n, double nbins) {
  if (n == 0) return 0;
  if (n < nbins) return NAN;
  int np = (int)(n / nbins);
  double mean = 0;
  for (int i = 0; i < n; ++i) mean += a[i];
  mean /= n;
  double sum = 0;
  int nb = (int)nbins;
  for (int b = 0; b < nb; ++b) {
    double m = 0;
    for (int i = 0; i < np; ++i) m += a[b * np + i];
    m /= np;
    sum += pow(m - mean, 2);
  }
  return sqrt(sum) / nbins;
}

/* ------------------------------------------------------------------ full run */

typedef struct {
  /* time series (sample index) */
  double *t, *me, *mp, *mv, *fd, *pc, *bv, *bd;
  int cap;
} series;

static void series_grow(series* s, int need) {
  if (need < s->cap) return;
  int nc = s->cap ? s->cap : 100;
  while (nc <= need) nc *= 2;
  s->t = realloc(s->t, sizeof(double) * nc);
  s->me = realloc(s->me, sizeof(double) * nc);
  s->mp = realloc(s->mp, sizeof(double) * nc * 3);
  s->mv = realloc(s->mv, sizeof(double) * nc * 3);
  s->bv = realloc(s->bv, sizeof(double) * nc * 3);
  s->fd = realloc(s->fd, sizeof(double) * nc * 9);
  s->pc = realloc(s->pc, sizeof(double) * nc * 9);
  s->bd = realloc(s->bd, sizeof(double) * nc * 9);
  s->cap = nc;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* column-wise batch-mean errors of a block of rows [first, first+n) */
static void col_stats(const double* data, int ncol, int first, int n, double* mean, double* err) {
  double* col = malloc(sizeof(double) * (n > 0 ? n : 1));
  for (int c = 0; c < ncol; ++c) {
    double m = 0;
    for (int i = 0; i < n; ++i) {
      col[i] = data[(size_t)(first + i) * ncol + c];
      m += col[i];
    }
    mean[c] = n ? m / n : NAN;
    err[c] = lo_statistical_error(col, n, 50);
  }
  free(col);
}

int lo_run(const lo_procs* pr_in, lo_fields* f, const lo_run_config* cfg, lo_run_result* res, double* rate,
           double* power_gain, double* power_loss, double* eedf_out, double* eedf_cells_out) {
  lo_procs pr = *pr_in;
  const int P = pr.P, M = pr.M;
  const int N = cfg->n_electrons;
  const double t_start = now_s();
  int nthreads = cfg->n_threads > 0 ? cfg->n_threads : 1;
#ifdef _OPENMP
  omp_set_num_threads(nthreads);
#else
  nthreads = 1;
#endif
  memset(res, 0, sizeof(*res));
  pr.max_interp = -1.0;

  lo_rng* rngs = malloc(sizeof(lo_rng) * nthreads);
  for (int i = 0; i < nthreads; ++i) lo_rng_seed(&rngs[i], cfg->seed, (uint64_t)i + 1);
  lo_rng* r0 = &rngs[0];

  double* pos = calloc((size_t)N * 3, sizeof(double));
  double* vel = malloc(sizeof(double) * N * 3);
  double* en = malloc(sizeof(double) * N);
  double* et = calloc(N, sizeof(double));
  double* tau = malloc(sizeof(double) * N);
  double* nui = malloc(sizeof(double) * N);
  int* chosen = malloc(sizeof(int) * N);
  double* ejp = malloc(sizeof(double) * N * 3);
  double* ejv = malloc(sizeof(double) * N * 3);
  double* eje = malloc(sizeof(double) * N);
  double* dE = malloc(sizeof(double) * N);
  double* gainf = malloc(sizeof(double) * N);
  char* adv = malloc(N);
  char* attached = malloc(N);
  int* ej_ids = malloc(sizeof(int) * N);
  int* att_ids = malloc(sizeof(int) * N);
  unsigned long long* counters = calloc(P, sizeof(unsigned long long));
  double* egp = calloc(P, sizeof(double));
  double* elp = calloc(P, sizeof(double));

  /* BoltzmannMC.C:428-559 */
  double time = 0, ss_time = LO_NON_DEF;
  const double gas_energy = 1.5 * LO_KB * f->Tg / LO_QE;
  f->gas_energy = gas_energy;
  double sd_e = sqrt(LO_KB * cfg->init_temp_ratio * f->Tg / LO_ME);
  for (int i = 0; i < N; ++i) {
    double n3[3];
    normal3(r0, n3);
    for (int k = 0; k < 3; ++k) vel[i * 3 + k] = n3[k] * sd_e;
    en[i] = 0.5 * LO_ME * sqnorm3(vel + i * 3) / LO_QE;
    tau[i] = LO_NON_DEF;
  }
  double maxE0 = 0;
  for (int i = 0; i < N; ++i) maxE0 = (i == 0 || en[i] > maxE0) ? en[i] : maxE0;
  lo_build_tables(&pr, f, 2.0 * maxE0);
  double nu_trial = pr.nu_max[M - 1];
  for (int i = 0; i < N; ++i) nui[i] = nu_trial;

  series S = {0};
  series_grow(&S, 100);
  int nPh = cfg->n_phases;
  int periodic = f->omega != 0;
  double phase_step = 2.0 * M_PI / nPh;
  double* nppp = calloc(nPh, sizeof(double));
  double* me_per = calloc(nPh, sizeof(double));
  double* fv_per = calloc((size_t)nPh * 3, sizeof(double));
  double* bv_per = calloc((size_t)nPh * 3, sizeof(double));
  double* fd_per = calloc((size_t)nPh * 9, sizeof(double));
  double* bd_per = calloc((size_t)nPh * 9, sizeof(double));
  double max_elec_energy = maxE0;

  double energy_gain_field = 0, energy_growth = 0;
  unsigned long long total_coll = 0, null_coll = 0, coll_at_ss = 0, null_at_ss = 0, coll_after_ss = 0;
  int nEC = cfg->n_energy_cells;
  double max_eedf = 0, eedf_step = 0;
  double* eeh_sum = calloc(nEC, sizeof(double));
  double* eeh_sum_per = calloc((size_t)nPh * nEC, sizeof(double));
  double* eeh = calloc(nEC, sizeof(double));
  double* tmp_sum = calloc(nEC, sizeof(double));
  double* tmp_per = calloc((size_t)nPh * nEC, sizeof(double));

  int nSamp = 1, nSync = 1, cur = 0, first_int = 0, nInt = 0;
  double total_int_time = 0, time_int = 0;
  int good_err = 0;
  int status = 0;
  double pb_rel_err = 0;
  long long sync_steps = 0;

  /* calculateMeanDataForSwarmParams (BoltzmannMC.C:1410-1482) */
#define MEAN_DATA()                                                                                         \
  do {                                                                                                      \
    series_grow(&S, nSamp);                                                                                 \
    double mx = en[0];                                                                                      \
    for (int i = 1; i < N; ++i) mx = en[i] > mx ? en[i] : mx;                                               \
    max_elec_energy = fmax(max_elec_energy, mx);                                                            \
    if (max_elec_energy > pr.energy_max_elastic) status = 1;                                                \
    double se = 0, sp[3] = {0, 0, 0}, sv[3] = {0, 0, 0}, pc[9] = {0}, fd[9] = {0};                           \
    for (int i = 0; i < N; ++i) {                                                                           \
      se += en[i];                                                                                          \
      for (int a = 0; a < 3; ++a) {                                                                         \
        sp[a] += pos[i * 3 + a];                                                                            \
        sv[a] += vel[i * 3 + a];                                                                            \
        for (int b = 0; b < 3; ++b) {                                                                       \
          pc[a * 3 + b] += pos[i * 3 + a] * pos[i * 3 + b];                                                 \
          fd[a * 3 + b] += pos[i * 3 + a] * vel[i * 3 + b];                                                 \
        }                                                                                                   \
      }                                                                                                     \
    }                                                                                                       \
    S.me[cur] = se / N;                                                                                     \
    for (int a = 0; a < 3; ++a) {                                                                           \
      S.mp[cur * 3 + a] = sp[a] / N;                                                                        \
      S.mv[cur * 3 + a] = sv[a] / N;                                                                        \
    }                                                                                                       \
    for (int a = 0; a < 3; ++a)                                                                             \
      for (int b = 0; b < 3; ++b) {                                                                         \
        S.pc[cur * 9 + a * 3 + b] = pc[a * 3 + b] / N - S.mp[cur * 3 + a] * S.mp[cur * 3 + b];              \
        S.fd[cur * 9 + a * 3 + b] = fd[a * 3 + b] / N - S.mp[cur * 3 + a] * S.mv[cur * 3 + b];              \
      }                                                                                                     \
    if (cur != 0) {                                                                                         \
      double dt_s = S.t[cur] - S.t[cur - 1];                                                                \
      for (int a = 0; a < 3; ++a) S.bv[cur * 3 + a] = (S.mp[cur * 3 + a] - S.mp[(cur - 1) * 3 + a]) / dt_s;\
      for (int a = 0; a < 9; ++a) S.bd[cur * 9 + a] = 0.5 * (S.pc[cur * 9 + a] - S.pc[(cur - 1) * 9 + a]) / dt_s; \
    } else {                                                                                                \
      for (int a = 0; a < 3; ++a) S.bv[a] = S.mv[a];                                                        \
      for (int a = 0; a < 9; ++a) S.bd[a] = S.fd[a];                                                        \
    }                                                                                                       \
    if (periodic && ss_time != LO_NON_DEF) {                                                                \
      double ph = fmod(f->omega * time, 2.0 * M_PI);                                                        \
      int pi = (int)fmin(floor(ph / phase_step), nPh - 1);                                                  \
      nppp[pi] += 1.0;                                                                                      \
      me_per[pi] += S.me[cur];                                                                              \
      for (int a = 0; a < 3; ++a) {                                                                         \
        fv_per[pi * 3 + a] += S.mv[cur * 3 + a];                                                            \
        bv_per[pi * 3 + a] += S.bv[cur * 3 + a];                                                            \
      }                                                                                                     \
      for (int a = 0; a < 9; ++a) {                                                                         \
        fd_per[pi * 9 + a] += S.fd[cur * 9 + a];                                                            \
        bd_per[pi * 9 + a] += S.bd[cur * 9 + a];                                                            \
      }                                                                                                     \
    }                                                                                                       \
  } while (0)

  /* EEDF part of getTimeDependDistributions (BoltzmannMC.C:1492-1560) */
#define EEDF_ACCUM()                                                                                        \
  do {                                                                                                      \
    if (max_elec_energy > max_eedf) {                                                                       \
      double old_step = eedf_step, old_max = max_eedf;                                                      \
      memcpy(tmp_sum, eeh_sum, sizeof(double) * nEC);                                                       \
      memcpy(tmp_per, eeh_sum_per, sizeof(double) * nPh * nEC);                                             \
      max_eedf = 1.2 * max_elec_energy;                                                                     \
      eedf_step = max_eedf / nEC;                                                                           \
      memset(eeh_sum, 0, sizeof(double) * nEC);                                                             \
      for (int o = 0; o < nEC; ++o) {                                                                       \
        double lo_e = o * old_step, hi_e = (o + 1 == nEC) ? old_max : (o + 1) * old_step;                  \
        int nl = (int)(lo_e / eedf_step), nr = (int)(hi_e / eedf_step);                                     \
        if (nl == nr) {                                                                                     \
          eeh_sum[nl] += tmp_sum[o];                                                                        \
          if (periodic)                                                                                     \
            for (int rep = 0; rep < nPh; ++rep)                                                             \
              for (int q = 0; q < nPh; ++q) eeh_sum_per[q * nEC + nl] += tmp_per[q * nEC + o];              \
        } else {                                                                                            \
          double lf = (nr * eedf_step - lo_e) / old_step;                                                   \
          eeh_sum[nl] += lf * tmp_sum[o];                                                                   \
          eeh_sum[nr] += (1.0 - lf) * tmp_sum[o];                                                           \
          if (periodic)                                                                                     \
            for (int rep = 0; rep < nPh; ++rep)                                                             \
              for (int q = 0; q < nPh; ++q) {                                                               \
                eeh_sum_per[q * nEC + nl] += lf * tmp_per[q * nEC + o];                                     \
                eeh_sum_per[q * nEC + nr] += (1.0 - lf) * tmp_per[q * nEC + o];                             \
              }                                                                                             \
        }                                                                                                   \
      }                                                                                                     \
    }                                                                                                       \
    memset(eeh, 0, sizeof(double) * nEC);                                                                   \
    for (int i = 0; i < N; ++i) {                                                                           \
      int c = (int)((en[i] - 0.0) / eedf_step);                                                             \
      if (c < nEC) eeh[c] += 1;                                                                             \
    }                                                                                                       \
    for (int c = 0; c < nEC; ++c) eeh_sum[c] += eeh[c];                                                     \
    if (periodic) {                                                                                         \
      double ph = fmod(f->omega * time, 2.0 * M_PI);                                                        \
      int pi = (int)fmin(floor(ph / phase_step), nPh - 1);                                                  \
      for (int c = 0; c < nEC; ++c) eeh_sum_per[pi * nEC + c] += eeh[c];                                    \
    }                                                                                                       \
  } while (0)

  S.t[0] = 0;
  MEAN_DATA();

  while ((!good_err && cfg->errors_checked) || nInt < cfg->req_integration_points ||
         total_int_time / ss_time < cfg->req_ss_times || total_int_time < cfg->req_abs_time) {
    if (coll_after_ss >= cfg->max_coll_after_ss && nInt > 100) break;
    if (status == 1) break;
    if ((cfg->max_seconds > 0 && now_s() - t_start > cfg->max_seconds) ||
        (cfg->max_sync_steps > 0 && sync_steps >= cfg->max_sync_steps)) {
      status = 2;
      break;
    }

    /* electronDynamicsUntilSynchronization (BoltzmannMC.C:617-688) */
    /* checkMaxCollisionFrequency (BoltzmannMC.C:716-763) */
#define CHECK_MAX_FREQ()                                                                                    \
  do {                                                                                                      \
    double mb = en[0];                                                                                      \
    for (int i = 1; i < N; ++i) mb = en[i] > mb ? en[i] : mb;                                               \
    double thermal = (f->gas_temp_effect == 1 || f->gas_temp_effect == 2) ? 10.0 * gas_energy : 0;          \
    int upd = 1;                                                                                            \
    while (upd) {                                                                                           \
      upd = 0;                                                                                              \
      double maxEn = lo_max_accel_energy(f, mb, 10.0 / nu_trial) + thermal;                                 \
      if (maxEn > pr.max_interp || 2.5 * maxEn < pr.max_interp) {                                           \
        if (2.0 * maxEn < pr.energy_max_elastic) lo_build_tables(&pr, f, 2.0 * maxEn);                      \
        else lo_build_tables(&pr, f, pr.energy_max_elastic);                                                \
      }                                                                                                     \
      int ei = (int)fmin(ceil(maxEn / pr.step), M - 1);                                                     \
      if (nu_trial < pr.nu_max[ei]) {                                                                       \
        upd = 1;                                                                                            \
        nu_trial *= 1.1;                                                                                    \
      }                                                                                                     \
    }                                                                                                       \
  } while (0)

    CHECK_MAX_FREQ();
    double dt_sync = cfg->sync_x / nu_trial;
    double t_sync = time + dt_sync;
    ++nSync;
    ++sync_steps;
    if ((cfg->mark_sync_step > 0 && sync_steps == cfg->mark_sync_step + 1) ||
        (cfg->mark_seconds > 0 && res->mark_elapsed == 0 && now_s() - t_start > cfg->mark_seconds)) {
      res->mark_real_collisions = (double)(total_coll);
      res->mark_null_collisions = (double)null_coll;
      res->mark_elapsed = now_s() - t_start;
      res->mark_sync_steps = sync_steps - 1;
    }
    memset(adv, 1, N);
    int any = 1;
    while (any) {
      any = 0;
      memset(adv, 0, N);
      CHECK_MAX_FREQ();
      const double nu_now = nu_trial;
#pragma omp parallel for schedule(static)
      for (int i = 0; i < N; ++i) {
#ifdef _OPENMP
        lo_rng* rr = &rngs[omp_get_thread_num()];
#else
        lo_rng* rr = r0;
#endif
        double ti = et[i];
        if (ti == t_sync) {
          chosen[i] = (int)LO_NON_DEF;
          continue;
        }
        double p3[3] = {pos[i * 3], pos[i * 3 + 1], pos[i * 3 + 2]};
        double v3[3] = {vel[i * 3], vel[i * 3 + 1], vel[i * 3 + 2]};
        double e = en[i];
        double ft = tau[i];
        double g;
        if (ft == LO_NON_DEF) {
          ft = -log(lo_uniform(rr, 0, 0)) / nu_now;
          nui[i] = nu_now;
        }
        if (ti + ft > t_sync) {
          double dta = t_sync - ti;
          lo_accelerate(f, ti, dta, p3, v3, &e, &g);
          gainf[i] = g;
          ti = t_sync;
          ft -= dta;
          chosen[i] = -2;
        } else {
          lo_accelerate(f, ti, ft, p3, v3, &e, &g);
          gainf[i] = g;
          ti += ft;
          lo_coll_out co;
          lo_collide(&pr, f, nui[i], v3, e, rr, &co);
          chosen[i] = co.chosen;
          v3[0] = co.vel[0];
          v3[1] = co.vel[1];
          v3[2] = co.vel[2];
          e = co.energy;
          dE[i] = co.dE;
          if (co.chosen >= 0 && pr.ptype[co.chosen] == 1) {
            for (int k = 0; k < 3; ++k) {
              ejv[i * 3 + k] = co.ej_vel[k];
              ejp[i * 3 + k] = p3[k];
            }
            eje[i] = co.ej_energy;
          }
          ft = -log(lo_uniform(rr, 0, 0)) / nu_now;
          nui[i] = nu_now;
          adv[i] = 1;
        }
        for (int k = 0; k < 3; ++k) {
          pos[i * 3 + k] = p3[k];
          vel[i * 3 + k] = v3[k];
        }
        en[i] = e;
        et[i] = ti;
        tau[i] = ft;
      }
      for (int i = 0; i < N; ++i) any |= adv[i];

      /* nonParallelCollisionTasks (BoltzmannMC.C:1282-1408) */
      int nEj = 0, nAt = 0;
      memset(attached, 0, N);
      for (int i = 0; i < N; ++i) {
        int c = chosen[i];
        if (c == (int)LO_NON_DEF) continue;
        energy_gain_field += gainf[i];
        if (c == -1) { ++null_coll; continue; }
        if (c == -2) continue;
        ++counters[c];
        ++total_coll;
        if (dE[i] >= 0) egp[c] += dE[i];
        else elp[c] += dE[i];
        if (pr.ptype[c] == 1) ej_ids[nEj++] = i;
        else if (pr.ptype[c] == 2) {
          attached[i] = 1;
          att_ids[nAt++] = i;
        }
      }
      for (int a = 0; a < nAt; ++a) {
        int id = att_ids[a];
        if (nEj > 0) {
          int s = ej_ids[nEj - 1];
          for (int k = 0; k < 3; ++k) {
            pos[id * 3 + k] = ejp[s * 3 + k];
            vel[id * 3 + k] = ejv[s * 3 + k];
          }
          en[id] = eje[s];
          et[id] = et[s];
          tau[id] = LO_NON_DEF;
          nui[id] = nu_trial;
          attached[id] = 0;
          --nEj;
        } else {
          int r = (int)fmin(lo_uniform(r0, 1, 0) * N, N - 1);
          while (attached[r]) r = (int)fmin(lo_uniform(r0, 1, 0) * N, N - 1);
          energy_growth += en[r];
          for (int k = 0; k < 3; ++k) {
            pos[id * 3 + k] = pos[r * 3 + k];
            vel[id * 3 + k] = vel[r * 3 + k];
          }
          en[id] = en[r];
          et[id] = et[r];
          tau[id] = tau[r];
          nui[id] = nui[r];
        }
      }
      while (nEj > 0) {
        int r = (int)fmin(lo_uniform(r0, 1, 0) * (N + nEj), N + nEj - 1);
        if (r < N) {
          int s = ej_ids[nEj - 1];
          energy_growth -= en[r];
          for (int k = 0; k < 3; ++k) {
            pos[r * 3 + k] = ejp[s * 3 + k];
            vel[r * 3 + k] = ejv[s * 3 + k];
          }
          en[r] = eje[s];
          et[r] = et[s];
          tau[r] = LO_NON_DEF;
          nui[r] = nu_trial;
        } else {
          r -= N;
          energy_growth -= eje[ej_ids[r]];
          int tmp = ej_ids[r];
          ej_ids[r] = ej_ids[nEj - 1];
          ej_ids[nEj - 1] = tmp;
        }
        --nEj;
      }
    }
    time = t_sync;

    /* sampling (BoltzmannMC.C:331-381) */
    if (nSync % cfg->sync_oversampling == 0) {
      ++nSamp;
      cur = nSamp - 1;
      series_grow(&S, nSamp);
      S.t[cur] = time;
      MEAN_DATA();
      if (status == 1) break;
      int dec = (int)fmax(log((double)nSamp) / log(2.0) - 11, 6);
      int between_ss = (int)pow(2, dec);
      if (ss_time != LO_NON_DEF) {
        ++nInt;
        coll_after_ss = total_coll - coll_at_ss;
        time_int = time - total_int_time;
        total_int_time = time - ss_time;
        EEDF_ACCUM();
      } else if (nSamp >= 100 && nSamp % between_ss == 0 && total_coll > cfg->min_coll_before_ss) {
        /* checkSteadyState (BoltzmannMC.C:1787-1893) */
        double t1 = 0.5 * time, t2 = 0.75 * time, a1 = 0, a2 = 0, rs = 0;
        int n1 = 0, n2 = 0;
        for (int i = 0; i < nSamp; ++i) {
          double st = S.t[i];
          if (st >= t1 && st <= t2) { a1 += S.me[i]; ++n1; }
          else if (st > t2) { double v = S.me[i]; a2 += v; rs += v * v; ++n2; }
        }
        a1 /= n1;
        a2 /= n2;
        rs = sqrt((rs / n2 - a2 * a2) / n2);
        if ((a1 >= a2 && rs < 0.01) || total_coll >= cfg->max_coll_before_ss) {
          first_int = cur;
          nInt = 1;
          ss_time = time;
          coll_at_ss = total_coll;
          null_at_ss = null_coll;
          energy_gain_field = 0;
          memset(counters, 0, sizeof(unsigned long long) * P);
          memset(egp, 0, sizeof(double) * P);
          memset(elp, 0, sizeof(double) * P);
          energy_growth = 0;
          total_int_time = 0;
          max_eedf = 1.2 * max_elec_energy;
          eedf_step = max_eedf / nEC;
          memset(eeh_sum, 0, sizeof(double) * nEC);
          memset(eeh_sum_per, 0, sizeof(double) * nPh * nEC);
          EEDF_ACCUM();
        }
      }
      dec = (int)fmax(log((double)nInt) / log(2.0) - 9, 7);
      int between_err = (int)pow(2, dec);
      if (ss_time != LO_NON_DEF && nInt > 200 && nInt % between_err == 0 && cfg->errors_checked) {
        /* checkStatisticalErrors (BoltzmannMC.C:1743-1767) */
        double m, e1, fv[3], fve[3], fdm[9], fde[9], bvm[3], bve[3], bdm[9], bde[9];
        col_stats(S.me, 1, first_int, nInt, &m, &e1);
        col_stats(S.mv, 3, first_int, nInt, fv, fve);
        col_stats(S.fd, 9, first_int, nInt, fdm, fde);
        col_stats(S.bv, 3, first_int, nInt, bvm, bve);
        col_stats(S.bd, 9, first_int, nInt, bdm, bde);
        double tg = energy_gain_field, tl = 0;
        if (energy_growth > 0) tg += energy_growth; else tl += energy_growth;
        for (int p = 0; p < P; ++p) { tg += egp[p]; tl += elp[p]; }
        pb_rel_err = fabs(tg + tl) / tg;
        double rf = (fabs(fv[0]) * fve[0] + fabs(fv[1]) * fve[1] + fabs(fv[2]) * fve[2]) / sqnorm3(fv);
        double rb = (fabs(bvm[0]) * bve[0] + fabs(bvm[1]) * bve[1] + fabs(bvm[2]) * bve[2]) / sqnorm3(bvm);
        if (e1 / m <= cfg->req_err_energy && rf <= cfg->req_err_flux_v && fde[0] / fdm[0] <= cfg->req_err_flux_d &&
            fde[4] / fdm[4] <= cfg->req_err_flux_d && fde[8] / fdm[8] <= cfg->req_err_flux_d &&
            rb <= cfg->req_err_bulk_v && bde[0] / bdm[0] <= cfg->req_err_bulk_d && bde[4] / bdm[4] <= cfg->req_err_bulk_d &&
            bde[8] / bdm[8] <= cfg->req_err_bulk_d && pb_rel_err <= cfg->req_err_power)
          good_err = 1;
      }
    }
  }

  /* finals (BoltzmannMC.C:386-396, 1484-1649) */
  total_int_time = time - ss_time;
  if (nInt > 0) {
    col_stats(S.me, 1, first_int, nInt, &res->mean_energy, &res->mean_energy_err);
    col_stats(S.mv, 3, first_int, nInt, res->flux_v, res->flux_v_err);
    col_stats(S.fd, 9, first_int, nInt, res->flux_d, res->flux_d_err);
    col_stats(S.bv, 3, first_int, nInt, res->bulk_v, res->bulk_v_err);
    col_stats(S.bd, 9, first_int, nInt, res->bulk_d, res->bulk_d_err);
  }
  double denom = (double)N * total_int_time * f->N;
  if (rate)
    for (int p = 0; p < P; ++p)
      rate[p] = pr.rel_dens[p] != 0 ? (double)counters[p] / (total_int_time * N * pr.rel_dens[p] * f->N) : 0;
  if (power_gain) for (int p = 0; p < P; ++p) power_gain[p] = egp[p] / denom;
  if (power_loss) for (int p = 0; p < P; ++p) power_loss[p] = elp[p] / denom;
  {
    double tg = energy_gain_field, tl = 0;
    if (energy_growth > 0) tg += energy_growth; else tl += energy_growth;
    for (int p = 0; p < P; ++p) { tg += egp[p]; tl += elp[p]; }
    res->power_balance_rel_err = fabs(tg + tl) / tg;
  }
  res->power_field = energy_gain_field / denom;
  res->power_growth = energy_growth / denom;
  if (eedf_out && eedf_cells_out) {
    double norm = 0;
    for (int c = 0; c < nEC; ++c) norm += eeh_sum[c];
    for (int c = 0; c < nEC; ++c) {
      double cell = eedf_step / 2.0 + c * eedf_step;
      eedf_cells_out[c] = cell;
      eedf_out[c] = eeh_sum[c] / (sqrt(cell) * norm * eedf_step);
    }
  }
  res->real_collisions = (double)total_coll;
  res->null_collisions = (double)null_coll;
  res->coll_at_ss = (double)coll_at_ss;
  res->null_at_ss = (double)null_at_ss;
  res->ss_time = ss_time;
  res->final_time = time;
  res->integration_points = nInt;
  res->trial_freq = nu_trial;
  res->max_eedf_energy = max_eedf;
  res->sync_steps = sync_steps;
  res->status = status;
  res->elapsed = now_s() - t_start;
  (void)time_int;

  free(rngs); free(pos); free(vel); free(en); free(et); free(tau); free(nui); free(chosen);
  free(ejp); free(ejv); free(eje); free(dE); free(gainf); free(adv); free(attached);
  free(ej_ids); free(att_ids); free(counters); free(egp); free(elp);
  free(S.t); free(S.me); free(S.mp); free(S.mv); free(S.fd); free(S.pc); free(S.bv); free(S.bd);
  free(nppp); free(me_per); free(fv_per); free(bv_per); free(fd_per); free(bd_per);
  free(eeh_sum); free(eeh_sum_per); free(eeh); free(tmp_sum); free(tmp_per);
  return status;
}
