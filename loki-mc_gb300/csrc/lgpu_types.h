// lgpu_types.h - plain data shared by the host runtime and the kernels of the
// electron Monte Carlo path. Integer codes follow the reference
// (Code/LoKI-MC/Headers/GeneralDefinitions.h:34-51).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lgpu {

enum FieldMode : int { kFieldDC = 0, kFieldAC = 1, kFieldB = 2, kFieldECR = 3, kFieldACB = 4 };
enum ProcType : int { kConservative = 0, kIonization = 1, kAttachment = 2 };
enum Sampler : int {
  kSamplerIsotropic = 0,
  kSamplerForward = 1,
  kSamplerBornDipole = 2,
  kSamplerSurendra = 3,
  kSamplerCoulombScreen = 4,
  kSamplerMomentumConservation = 5
};
enum Sharing : int { kSharingEqual = 0, kSharingOneTakesAll = 1, kSharingSDCS = 2, kSharingRandom = 3 };
enum GasTemp : int { kGasTempFalse = 0, kGasTempTrue = 1, kGasTempSmart = 2 };

// Field of one swarm condition, FP32 (the phase origin is passed per launch).
struct FieldF {
  int mode;
  float ax, ay, az;  // -e E / m (DC)
  float Ex, Ez;      // E amplitude (V/m), x and z components
  float w, W;        // excitation and cyclotron angular frequencies (rad/s)
  float e_me;        // e / m
};

// One process, FP32 copy of the flattened arrays (BoltzmannMC.h:86-113).
struct ProcF {
  int type;
  int sampler;
  float sp0, sp1;       // sampler parameters
  float eloss;          // eV, negative for superelastic
  float mass;           // target mass (kg)
  float red_mass;       // reduced mass (kg)
  float mass_factor;    // 2 m_r / (m_e + M)
  float wparam;         // SDCS w (eV)
  int pad;
};

// One target gas (per-gas process range for the thermal choice).
struct GasF {
  int first, last;
  float fraction;
  float thermal_sd;  // sqrt(k Tg / M)
  float red_mass;    // reduced mass of the gas' first process
  int pad[3];
};

// Interpolated tables of one condition: row pairs (row i, row min(i+1,M-1))
// so that each interpolation is one 8-byte load.
struct TablesF {
  const float2* nu_pair;   // [M] total collision frequency
  const float2* cum_pair;  // [M*P] cumulative sigma*n
  const float2* sig_pair;  // [M*P] sigma*n
  int M, P;
  int stride;              // row stride in pairs: P rounded up to even (16-byte rows), padded with +inf / 0
  float inv_step;          // 1 / energy step (1/eV)
  float inv_N;             // 1 / gas density
  // bound of the total frequency over blocks of 2^coarse_shift rows (one
  // block also covers the row after it), slightly raised so that rounding in
  // the interpolation cannot exceed it: r above it is a null collision
  const float* nu_coarse;  // [n_coarse], or null
  int coarse_shift, n_coarse;
};
constexpr int kMaxCoarse = 256;

// Per-condition constants used by the kernels.
struct Consts {
  float qe, me, inv_qe;
  float half_me_over_e;    // 0.5 m / e: energy (eV) = v^2 * this
  float two_qe_over_me;    // 2 e / m
  int sharing;
  float sharing_factor;
  int gas_temp;
  float smart_energy;      // 20 * (3/2) k Tg / e (eV)
  int G;
};

// Per-interval parameters, written by the host into device memory before each
// synchronisation interval so that one captured CUDA graph serves every interval.
struct IntervalCtl {
  float dt_sync;          // interval length (s)
  float phi0;             // phase at the interval start (rad), reduced in FP64 on the host
  float phase_rate;       // w (AC, AC+B) or W (resonance)
  float nu;               // trial collision frequency (1/s)
  float inv_step;         // 1 / table energy step (1/eV)
  float shift_x, shift_y, shift_z;  // origin shift subtracted from every position on load
  unsigned long long interval;      // interval index (random-number counter)
};

// Per-block tallies written by the advance kernels (reduced on the device).
struct StepTally {
  unsigned long long null_count;
  unsigned long long real_count;
  double field_gain;
};

}  // namespace lgpu
