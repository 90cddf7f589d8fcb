// Test infrastructure for the oracle build of the reference (never shipped).
//
// Replaces the reference's random-number entry points
// (Code/LoKI-MC/Sources/MathFunctions.C:31-59: unitUniformRand, unitNormalRand,
// unitNormalRand3) in the oracle build so that the reference engine can be
// driven either by a recorded stream of uniforms (replay) or by a seeded,
// reproducible generator. The reference's own object file for
// MathFunctions.C is linked with these three symbols weakened, so every call
// made by BoltzmannMC.C resolves here.
//
// Semantics kept from the reference:
//  * unitUniformRand(includeZero, includeOne) redraws while the value is an
//    excluded endpoint (MathFunctions.C:38-41).
//  * unitNormalRand3 is Box-Muller on four uniforms drawn with (false, true):
//    (a cos b, a sin b, sqrt(-2 ln r3) cos(2 pi r4)), a = sqrt(-2 ln r1),
//    b = 2 pi r2 (MathFunctions.C:54-59).
//  * The seeded generator is the same family as the reference's
//    (std::mt19937_64 + uniform_real_distribution<double>(0, 1)), one per
//    OpenMP thread, seeded from (seed, thread index) instead of random_device.
#include "LoKI-MC/Headers/MathFunctions.h"

#include <omp.h>

#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <random>

namespace {
const double* g_replay = nullptr;
size_t g_replay_n = 0;
size_t g_replay_pos = 0;
bool g_replay_on = false;
int g_replay_overrun = 0;
uint64_t seed_from_env() {
  const char* s = std::getenv("LOKI_ORACLE_SEED");
  return s ? std::strtoull(s, nullptr, 10) : 12345ULL;
}
std::atomic<uint64_t> g_seed{seed_from_env()};
std::atomic<uint64_t> g_epoch{1};

struct ThreadGen {
  uint64_t epoch = 0;
  std::mt19937_64 gen;
  std::uniform_real_distribution<double> uni{0.0, 1.0};
  std::normal_distribution<double> nrm{0.0, 1.0};
};
thread_local ThreadGen t_gen;

double draw_raw() {
  if (g_replay_on) {
    if (g_replay_pos < g_replay_n) return g_replay[g_replay_pos++];
    g_replay_overrun = 1;
    return 0.5;
  }
  ThreadGen& t = t_gen;
  const uint64_t e = g_epoch.load();
  if (t.epoch != e) {
    const uint64_t s = g_seed.load() ^ (0x9E3779B97F4A7C15ULL * (uint64_t)(omp_get_thread_num() + 1));
    t.gen.seed(s);
    t.uni.reset();
    t.nrm.reset();
    t.epoch = e;
  }
  return t.uni(t.gen);
}
}  // namespace

double MathFunctions::unitUniformRand(bool includeZero, bool includeOne) {
  double u = draw_raw();
  while ((!includeZero && u == 0) || (!includeOne && u == 1)) u = draw_raw();
  return u;
}

double MathFunctions::unitNormalRand() {
  // not used on the electron Monte Carlo path; kept for link completeness
  double r1 = unitUniformRand(false, true), r2 = unitUniformRand(false, true);
  return std::sqrt(-2.0 * std::log(r1)) * std::cos(2.0 * M_PI * r2);
}

Eigen::Array3d MathFunctions::unitNormalRand3() {
  double r1 = unitUniformRand(false, true), r2 = unitUniformRand(false, true),
         r3 = unitUniformRand(false, true), r4 = unitUniformRand(false, true);
  double a = std::sqrt(-2.0 * std::log(r1)), b = 2.0 * M_PI * r2;
  return Eigen::Array3d(a * std::cos(b), a * std::sin(b), std::sqrt(-2.0 * std::log(r3)) * std::cos(2.0 * M_PI * r4));
}

extern "C" {
void ref_rng_replay(const double* u, size_t n) {
  g_replay = u;
  g_replay_n = n;
  g_replay_pos = 0;
  g_replay_on = true;
  g_replay_overrun = 0;
}
void ref_rng_replay_off() { g_replay_on = false; }
size_t ref_rng_consumed() { return g_replay_pos; }
int ref_rng_overrun() { return g_replay_overrun; }
void ref_rng_seed(uint64_t seed) {
  g_seed.store(seed);
  g_epoch.fetch_add(1);
}
}
