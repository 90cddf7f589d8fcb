// lgpu_device.cuh - per-electron device physics of the electron Monte Carlo
// path: counter-based random numbers, closed-form free flights, the
// null-collision test and process choice on interpolated tables, and the
// collision kinematics. Everything here runs in FP32; the FP64 parts of the
// method (absolute time, phase origin, position origin, tallies) live in the
// host runtime and the reduction kernels.
//
// Each function names the reference routine whose physics it implements
// (paths relative to the reference's Code/ directory).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lgpu_types.h"

namespace lgpu {

// ------------------------------------------------------------ records
// An electron record is two float4 in one 32-byte sector: (x, y, z, s) and
// (vx, vy, vz, flag). Every record buffer (ensemble, secondaries, spill) comes
// from cudaMalloc, so record i starts at a multiple of 32 bytes and moves with
// one 256-bit access (sm_100 and later) instead of two 128-bit ones: half the
// load/store instructions and L1 wavefronts of the passes over the ensemble.
__device__ __forceinline__ void load_record(const float4* rec, float4& A, float4& B) {
  asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=f"(A.x), "=f"(A.y), "=f"(A.z), "=f"(A.w), "=f"(B.x), "=f"(B.y), "=f"(B.z), "=f"(B.w)
               : "l"(rec));
}
__device__ __forceinline__ void store_record(float4* rec, float4 A, float4 B) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(rec), "f"(A.x), "f"(A.y),
               "f"(A.z), "f"(A.w), "f"(B.x), "f"(B.y), "f"(B.z), "f"(B.w)
               : "memory");
}

// Constant.h:6-8
constexpr double kQe = 1.6021766208e-19;
constexpr double kMe = 9.10938356e-31;
constexpr double kKb = 1.38064852e-23;
constexpr float kTwoPiF = 6.28318530717958647692f;

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon et al., SC'11): counter (4 x u32) and key (2 x u32)
// give four independent 32-bit words.
struct Philox {
  uint4 ctr;
  uint2 key;
  __device__ __forceinline__ static uint4 round(uint4 c, uint2 k) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    return make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  __device__ __forceinline__ uint4 next() {
    uint4 c = ctr;
    uint2 k = key;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      c = round(c, k);
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
    c = round(c, k);
    ctr.w += 1u;  // the per-electron event counter lives in the last word
    return c;
  }
};

// Uniform in (0, 1]: 24-bit lattice (k + 1) * 2^-24.
__device__ __forceinline__ float u01_oc(uint32_t x) { return (float)((x >> 8) + 1u) * 5.9604644775390625e-8f; }
// Uniform in (0, 1): 23-bit lattice (k + 0.5) * 2^-23.
__device__ __forceinline__ float u01_oo(uint32_t x) { return ((float)(x >> 9) + 0.5f) * 1.1920928955078125e-7f; }

// A stream of uniforms for one electron: four words per Philox call, used in
// order. Counter = (electron id, interval index low, interval index high,
// event word); key = the run seed.
struct PhiloxStream {
  Philox ph;
  uint4 buf;
  int left;
  __device__ __forceinline__ void init(uint32_t electron, uint64_t interval, uint64_t seed, uint32_t salt) {
    ph.ctr = make_uint4(electron, (uint32_t)interval, (uint32_t)(interval >> 32) ^ (salt << 16), 0u);
    ph.key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    left = 0;
  }
  __device__ __forceinline__ uint32_t word() {
    if (left == 0) {
      buf = ph.next();
      left = 4;
    }
    uint32_t w = buf.x;
    buf.x = buf.y;
    buf.y = buf.z;
    buf.z = buf.w;
    --left;
    return w;
  }
  // (0,1] for choices and samplers whose reference draw allows one
  __device__ __forceinline__ float oc() { return u01_oc(word()); }
  // (0,1) for the free-flight exponential (reference excludes 0 and 1)
  __device__ __forceinline__ float oo() { return u01_oo(word()); }
  // [0,1]-semantics draws take the (0,1] lattice
  __device__ __forceinline__ float cc() { return u01_oc(word()); }
};

// The per-electron stream of the advance kernels: PCG32 (XSH-RR output of a
// 64-bit LCG, O'Neill 2014), seeded for each (electron, interval, pass) by one
// Philox4x32-10 block, so results stay reproducible from the run seed while
// each uniform costs a handful of integer instructions and no divergent
// buffer refills.
struct PcgStream {
  uint64_t state, inc;
  // `tag` is the counter's last word: 0x5EED for ensemble electrons, the
  // creating warp's index for secondaries (whose salt differs)
  __device__ __forceinline__ void init(uint32_t electron, uint64_t interval, uint64_t seed, uint32_t salt,
                                       uint32_t tag = 0x5EEDu) {
    Philox ph;
    ph.ctr = make_uint4(electron, (uint32_t)interval, (uint32_t)(interval >> 32) ^ (salt << 16), tag);
    ph.key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    const uint4 w = ph.next();
    state = ((uint64_t)w.x << 32) | w.y;
    inc = ((((uint64_t)w.z << 32) | w.w) << 1) | 1ull;
  }
  __device__ __forceinline__ uint32_t word() {
    const uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    return __funnelshift_r(xs, xs, (uint32_t)(old >> 59));
  }
  __device__ __forceinline__ float oc() { return u01_oc(word()); }
  __device__ __forceinline__ float oo() { return u01_oo(word()); }
  __device__ __forceinline__ float cc() { return u01_oc(word()); }
};

// Replay of recorded uniforms (parity tests): values are taken in order.
struct ReplayStream {
  const double* u;
  int n, pos;
  __device__ __forceinline__ float take() { return pos < n ? (float)u[pos++] : (pos++, 0.5f); }
  __device__ __forceinline__ float oc() { return take(); }
  __device__ __forceinline__ float oo() { return take(); }
  __device__ __forceinline__ float cc() { return take(); }
};

// ------------------------------------------------------------ free flight

// Closed-form free flight (BoltzmannMC.C:804-905). `phi0` is the phase
// w*t (AC, AC+B) or W*t (resonance) at the flight start, reduced to [0, 2pi)
// by the caller in FP64. Position is an FP32 offset. Returns nothing; the
// caller recomputes the energy from the new velocity.
// MODE >= 0 selects the branch at compile time, -1 at run time from f.mode
template <int MODE = -1>
__device__ __forceinline__ void free_flight(const FieldF& f, float phi0, float dt, float3& p, float3& v) {
  switch (MODE >= 0 ? MODE : f.mode) {
    case kFieldDC: {
      // x += v dt + a dt^2/2 ; v += a dt. The DC, AC and B branches spell out
      // every rounding (explicit _rn operations) so that each kernel that
      // inlines them computes the same bits, whatever the compiler's choice
      // of multiply-add contraction in the surrounding code.
      const float hdt2 = __fmul_rn(__fmul_rn(0.5f, dt), dt);
      p.x = __fadd_rn(p.x, __fmaf_rn(v.x, dt, __fmul_rn(f.ax, hdt2)));
      p.y = __fadd_rn(p.y, __fmaf_rn(v.y, dt, __fmul_rn(f.ay, hdt2)));
      p.z = __fadd_rn(p.z, __fmaf_rn(v.z, dt, __fmul_rn(f.az, hdt2)));
      v.x = __fmaf_rn(f.ax, dt, v.x);
      v.y = __fmaf_rn(f.ay, dt, v.y);
      v.z = __fmaf_rn(f.az, dt, v.z);
      break;
    }
    case kFieldAC: {
      // harmonic E(t) = E cos(w t): BoltzmannMC.C:816-831
      const float w = f.w;
      float sPhi, cPhi, sPh, cPh;
      sincosf(phi0, &sPhi, &cPhi);
      const float wdt = __fmul_rn(w, dt);
      sincosf(__fadd_rn(phi0, wdt), &sPh, &cPh);
      const float k = __fdiv_rn(f.e_me, w);  // e/(m w)
      const float aux1 = __fmul_rn(__fdiv_rn(k, w), __fsub_rn(__fmaf_rn(wdt, sPhi, cPh), cPhi));
      const float aux2 = __fmul_rn(k, __fsub_rn(sPhi, sPh));
      p.x = __fadd_rn(p.x, __fmaf_rn(v.x, dt, __fmul_rn(f.Ex, aux1)));
      p.y = __fmaf_rn(v.y, dt, p.y);
      p.z = __fadd_rn(p.z, __fmaf_rn(v.z, dt, __fmul_rn(f.Ez, aux1)));
      v.x = __fmaf_rn(f.Ex, aux2, v.x);
      v.z = __fmaf_rn(f.Ez, aux2, v.z);
      break;
    }
    case kFieldB: {
      // DC E in the x-z plane, B along z: BoltzmannMC.C:835-849
      const float W = f.W;
      const float Wdt = __fmul_rn(W, dt);
      float sW, cW;
      sincosf(Wdt, &sW, &cW);
      const float sh = sinf(__fmul_rn(0.5f, Wdt));
      const float cWm1 = __fmul_rn(__fmul_rn(-2.0f, sh), sh);  // cos(W dt) - 1 without cancellation
      const float sW_W = __fdiv_rn(sW, W);
      const float aux2 = __fdiv_rn(cWm1, W);
      const float vEx = __fdiv_rn(__fmul_rn(f.e_me, f.Ex), W);
      const float az = __fmul_rn(f.e_me, f.Ez);
      const float vx0 = v.x, vy0 = v.y, vz0 = v.z;
      p.x = __fadd_rn(p.x, __fmaf_rn(vx0, sW_W, __fmul_rn(__fadd_rn(vy0, vEx), aux2)));
      p.y = __fadd_rn(p.y, __fmaf_rn(vEx, __fsub_rn(sW_W, dt), __fmaf_rn(vy0, sW_W, __fmul_rn(-vx0, aux2))));
      p.z = __fadd_rn(p.z, __fsub_rn(__fmul_rn(vz0, dt), __fmul_rn(__fmul_rn(__fmul_rn(0.5f, az), dt), dt)));
      v.x = __fsub_rn(__fmaf_rn(vx0, cW, __fmul_rn(-vy0, sW)), __fmul_rn(vEx, sW));
      v.y = __fmaf_rn(vEx, cWm1, __fmaf_rn(vx0, sW, __fmul_rn(vy0, cW)));
      v.z = __fsub_rn(vz0, __fmul_rn(az, dt));
      break;
    }
    case kFieldECR: {
      // w == W (cyclotron resonance): BoltzmannMC.C:850-872
      const float W = f.W;
      float sPhi, cPhi, sW, cW, sPh, cPh;
      sincosf(phi0, &sPhi, &cPhi);
      const float Wdt = W * dt;
      sincosf(Wdt, &sW, &cW);
      sincosf(phi0 + Wdt, &sPh, &cPh);
      const float cOpp = cosf(phi0 - Wdt);
      const float sh = sinf(0.5f * Wdt);
      const float cWm1 = -2.0f * sh * sh;
      const float k = f.e_me / W;
      const float vEx = k * f.Ex, vEz = k * f.Ez;
      const float sW_W = sW / W, cWm1_W = cWm1 / W, cPh_W = cPh / W;
      const float vx0 = v.x, vy0 = v.y, vz0 = v.z;
      p.x += vx0 * sW_W + vy0 * cWm1_W - 0.25f * vEx * (cPh_W - cOpp / W + 2.0f * dt * sPh);
      p.y += -vx0 * cWm1_W + vy0 * sW_W + 0.5f * vEx * (dt * cPh_W - 2.0f * cWm1_W * sPhi - cPhi * sW_W);
      p.z += vz0 * dt + vEz * (cPh_W - cPhi / W + dt * sPhi);
      v.x = vx0 * cW - vy0 * sW - 0.5f * vEx * (Wdt * cPh + cPhi * sW);
      v.y = vx0 * sW + vy0 * cW - 0.5f * vEx * (Wdt * cW * sPhi + (Wdt * cPhi - sPhi) * sW);
      v.z = vz0 + vEz * (sPhi - sPh);
      break;
    }
    default: {
      // general AC E + DC B: BoltzmannMC.C:873-897
      const float w = f.w, W = f.W;
      float sPhi, cPhi, sw, cw, sPh, cPh, sW, cW;
      sincosf(phi0, &sPhi, &cPhi);
      const float wdt = w * dt;
      sincosf(wdt, &sw, &cw);
      sincosf(phi0 + wdt, &sPh, &cPh);
      const float Wdt = W * dt;
      sincosf(Wdt, &sW, &cW);
      const float sh = sinf(0.5f * Wdt);
      const float cWm1 = -2.0f * sh * sh;
      const float w2 = w * w, W2 = W * W, d = w2 - W2;
      const float vEx = f.e_me / W * f.Ex;
      const float vEz = f.e_me / w * f.Ez;
      const float vEx_d = vEx / d;
      const float WvEx_d = W * vEx_d;
      const float sW_W = sW / W, cWm1_W = cWm1 / W;
      const float wsPhi = w * sPhi;
      const float vx0 = v.x, vy0 = v.y, vz0 = v.z;
      p.x += vx0 * sW_W + vy0 * cWm1_W + WvEx_d * (cPhi * (cw - cW) + (wsPhi * sW_W - sPhi * sw));
      p.y += -vx0 * cWm1_W + vy0 * sW_W - vEx_d / w * ((W2 + w2 * cW - w2) * sPhi + W2 * (w * cPhi * sW_W - sPh));
      p.z += vz0 * dt + vEz * ((cPh - cPhi) / w + dt * sPhi);
      v.x = vx0 * cW - vy0 * sW + WvEx_d * w * (cW * sPhi - sPh + cPhi / w * W * sW);
      v.y = vx0 * sW + vy0 * cW + vEx_d * W2 * (cPh - cPhi * cW + wsPhi * sW_W);
      v.z = vz0 + vEz * (sPhi - sPh);
      break;
    }
  }
}

// ------------------------------------------------------------ kinematics

// Spherical angles without trigonometry (MathFunctions.C:143-163).
struct Sph {
  float speed, sT, cT, sP, cP;
};
__device__ __forceinline__ Sph cart2sph(float3 v) {
  Sph s;
  const float xy2 = v.x * v.x + v.y * v.y;
  const float nxy = sqrtf(xy2);
  s.speed = sqrtf(xy2 + v.z * v.z);
  const float inv = 1.0f / s.speed;
  s.sT = nxy * inv;
  s.cT = v.z * inv;
  if (nxy != 0.0f) {
    const float ixy = 1.0f / nxy;
    s.sP = v.y * ixy;
    s.cP = v.x * ixy;
  } else {
    s.sP = 1.0f;
    s.cP = 0.0f;
  }
  return s;
}

// Rotation of the scattering angles into the laboratory frame
// (Yousfi 1994; MathFunctions.C:129-141).
__device__ __forceinline__ float3 euler(float sChi, float cChi, float sEta, float cEta, const Sph& s) {
  const float sCsE = sChi * sEta;
  const float aux = sChi * cEta * s.cT + cChi * s.sT;
  return make_float3(-sCsE * s.sP + aux * s.cP, sCsE * s.cP + aux * s.sP, -sChi * cEta * s.sT + cChi * s.cT);
}

// cos(chi) samplers (AngularScatteringFunctions.h:27-74). Each returns
// (cos chi, 1 - cos chi, 1 + cos chi), the last two formed without
// cancellation, so that sin chi = sqrt((1-c)(1+c)) keeps FP32 accuracy for
// forward and backward scattering alike.
template <class Rng>
__device__ __forceinline__ float3 sample_cos_chi(const ProcF& pr, float energy, float energy_after, Rng& rng) {
  switch (pr.sampler) {
    case kSamplerForward:
      return make_float3(1.0f, 0.0f, 2.0f);
    case kSamplerBornDipole: {
      // Vialetto 2021, eq. 25: c = 1 + 2 r2/(1-r2) (1 - r2^-U)
      // 1 - c = 2 r2 (r2^-U - 1)/(1-r2), 1 + c = 2 (1 - r2^(1-U))/(1-r2)
      const float s = sqrtf(energy_after) + sqrtf(energy);
      const float ratio = pr.eloss / (s * s);
      const float r2 = ratio * ratio;
      const float u = rng.cc();
      const float lr = logf(r2);
      const float inv = 1.0f / (1.0f - r2);
      const float om = 2.0f * r2 * inv * expm1f(-u * lr);
      const float op = -2.0f * inv * expm1f((1.0f - u) * lr);
      return make_float3(1.0f - om, om, op);
    }
    case kSamplerSurendra: {
      // Vahedi 1995, eq. 9: c = (2 + e - 2 (1+e)^U) / e
      // 1 - c = 2((1+e)^U - 1)/e, 1 + c = -2 (1+e) ((1+e)^(U-1) - 1)/e
      const float u = rng.cc();
      const float l = log1pf(energy);
      const float om = 2.0f * expm1f(u * l) / energy;
      const float op = -2.0f * (1.0f + energy) * expm1f((u - 1.0f) * l) / energy;
      return make_float3(1.0f - om, om, op);
    }
    case kSamplerCoulombScreen: {
      // Hagelaar 2000, eqs. 21-23: c = (sp + 1 - (2 sp + 1) R) / (sp + 1 - R)
      // 1 - c = 2 sp R / d, 1 + c = 2 (sp + 1)(1 - R) / d, d = sp + (1 - R)
      const float eps = (pr.sp0 == 0.0f) ? energy : energy_after;
      const float sp = pr.sp1 / eps;
      const float R = rng.cc();
      const float omr = 1.0f - R;
      const float inv = 1.0f / (sp + omr);
      const float om = 2.0f * sp * R * inv;
      const float op = 2.0f * (sp + 1.0f) * omr * inv;
      return make_float3((sp + 1.0f - (2.0f * sp + 1.0f) * R) * inv, om, op);
    }
    default: {  // isotropic: c = 1 - 2U
      const float u = rng.cc();
      return make_float3(1.0f - 2.0f * u, 2.0f * u, 2.0f * (1.0f - u));
    }
  }
}

__device__ __forceinline__ float sin_from(float3 c) { return sqrtf(fmaxf(0.0f, c.y * c.z)); }

// Result of one collision event.
struct CollResult {
  int chosen;         // process id, -1 null
  float dE;           // energy change (eV) of the incident electron
  int ionized;        // a secondary was created
  float3 ej_v;        // secondary velocity
};

// (rounding spelled out, as in the flights)
__device__ __forceinline__ float energy_of(float3 v, float half_me_over_e) {
  return __fmul_rn(__fmaf_rn(v.z, v.z, __fmaf_rn(v.y, v.y, __fmul_rn(v.x, v.x))), half_me_over_e);
}

// Collision kinematics of the chosen process (BoltzmannMC.C:1115-1280).
// `tv` is the target velocity (zero for a cold gas). Returns false when the
// event turns into a null collision (energy below the threshold after
// interpolation, BoltzmannMC.C:1137-1140, 1169-1172, 1202-1205).
template <class Rng>
__device__ __forceinline__ bool apply_collision(const Consts& c, const ProcF& pr, bool thermal, float3 tv, float3& v,
                                                float& energy, Rng& rng, CollResult& out) {
  const float incident = energy;
  if (pr.type == kConservative) {
    if (thermal) {
      // centre-of-mass kinematics with a moving target (BoltzmannMC.C:1125-1158)
      const float3 rel = make_float3(v.x - tv.x, v.y - tv.y, v.z - tv.z);
      const Sph s = cart2sph(rel);
      const float relE = 0.5f * pr.red_mass * s.speed * s.speed * c.inv_qe;
      const float relEA = relE - pr.eloss;
      if (relEA <= 0.0f) return false;
      const float3 cc = sample_cos_chi(pr, relE, relEA, rng);
      const float cChi = cc.x, sChi = sin_from(cc);
      float sEta, cEta;
      sincosf(kTwoPiF * rng.oc(), &sEta, &cEta);
      const float3 ver = euler(sChi, cChi, sEta, cEta, s);
      const float sa = sqrtf(fmaxf(0.0f, s.speed * s.speed - 2.0f / pr.red_mass * pr.eloss * c.qe));
      const float inv_tot = 1.0f / (c.me + pr.mass);
      const float fa = pr.mass * inv_tot;
      v.x = fa * (sa * ver.x) + (c.me * v.x + pr.mass * tv.x) * inv_tot;
      v.y = fa * (sa * ver.y) + (c.me * v.y + pr.mass * tv.y) * inv_tot;
      v.z = fa * (sa * ver.z) + (c.me * v.z + pr.mass * tv.z) * inv_tot;
    } else {
      // target at rest (BoltzmannMC.C:1160-1187)
      const Sph s = cart2sph(v);
      const float eA = incident - pr.eloss;
      if (eA <= 0.0f) return false;
      const float3 cc = sample_cos_chi(pr, incident, eA, rng);
      const float cChi = cc.x, sChi = sin_from(cc);
      float sEta, cEta;
      sincosf(kTwoPiF * rng.oc(), &sEta, &cEta);
      const float3 ver = euler(sChi, cChi, sEta, cEta, s);
      const float sp = sqrtf(fmaxf(0.0f, (s.speed * s.speed - c.two_qe_over_me * pr.eloss) *
                                             (1.0f - pr.mass_factor * cc.y)));
      v = make_float3(sp * ver.x, sp * ver.y, sp * ver.z);
    }
    energy = energy_of(v, c.half_me_over_e);
    out.dE = energy - incident;
    out.ionized = 0;
    return true;
  }
  if (pr.type == kIonization) {
    // BoltzmannMC.C:1195-1272
    const float thr = pr.eloss;
    if (incident < thr) return false;
    const Sph s = cart2sph(v);
    const float net = incident - thr;
    float ej;
    if (c.sharing == kSharingSDCS) {
      ej = pr.wparam * tanf(rng.cc() * atanf(net / (2.0f * pr.wparam)));
    } else if (c.sharing == kSharingRandom) {
      ej = rng.cc() * net;
    } else {
      ej = c.sharing_factor * net;
    }
    const float scat = net - ej;
    float cChiS, sChiS, cChiE, sChiE, sEtaS, cEtaS, sEtaE, cEtaE;
    if (pr.sampler == kSamplerMomentumConservation) {
      cChiS = sqrtf(scat / net);
      sChiS = sqrtf(ej / net);  // sqrt(1 - cos^2) with cos^2 = scat/net
      sincosf(kTwoPiF * rng.oc(), &sEtaS, &cEtaS);
      cChiE = sqrtf(ej / net);
      sChiE = sqrtf(scat / net);
      sEtaE = -sEtaS;
      cEtaE = -cEtaS;
    } else {
      const float3 cs = sample_cos_chi(pr, incident, scat, rng);
      cChiS = cs.x;
      sChiS = sin_from(cs);
      sincosf(kTwoPiF * rng.oc(), &sEtaS, &cEtaS);
      const float3 ce = sample_cos_chi(pr, incident, ej, rng);
      cChiE = ce.x;
      sChiE = sin_from(ce);
      sincosf(kTwoPiF * rng.oc(), &sEtaE, &cEtaE);
    }
    const float3 vs = euler(sChiS, cChiS, sEtaS, cEtaS, s);
    const float3 ve = euler(sChiE, cChiE, sEtaE, cEtaE, s);
    const float ss = sqrtf(c.two_qe_over_me * scat), se = sqrtf(c.two_qe_over_me * ej);
    v = make_float3(ss * vs.x, ss * vs.y, ss * vs.z);
    out.ej_v = make_float3(se * ve.x, se * ve.y, se * ve.z);
    energy = scat;
    out.dE = -thr;
    out.ionized = 1;
    return true;
  }
  // attachment (BoltzmannMC.C:1274-1280)
  out.dE = -incident;
  out.ionized = 0;
  return true;
}

// Row weights of the linear interpolation between table rows
// (BoltzmannMC.C:1036-1047).
__device__ __forceinline__ void row_weights(float eos, int M, int& i1, float& w1, float& w2) {
  i1 = (int)fminf(eos, (float)(M - 1));
  const int i2 = min(i1 + 1, M - 1);
  w1 = (float)i2 - eos;
  if (w1 < 0.0f) w1 = 0.0f;
  w2 = 1.0f - w1;
}

// Index of the first cumulative value >= x in one table row, i.e. the result
// of the reference's bisection (BoltzmannMC.C:1066-1088), which returns the
// smallest p with C_p >= x (or P-1). Instead of a chain of dependent loads it
// counts the entries below x with independent 16-byte loads: the whole row
// for up to 64 processes, otherwise every 16th entry first and then the 16
// entries of the selected block.
__device__ __forceinline__ int row_count_below(const float2* row, int P, int stride, float w1, float w2, float x) {
  const float4* r4 = reinterpret_cast<const float4*>(row);
  int cnt = 0;
  if (P <= 64) {
#pragma unroll 8
    for (int q = 0; q < (stride >> 1); ++q) {
      const float4 c = __ldg(&r4[q]);
      cnt += (w1 * c.x + w2 * c.y < x) + (w1 * c.z + w2 * c.w < x);
    }
  } else {
    const int nb = (P + 15) >> 4;
    int blk = 0;
#pragma unroll 4
    for (int b = 0; b < nb; ++b) {
      const int last = min((b << 4) + 15, P - 1);
      const float2 c = __ldg(&row[last]);
      blk += (w1 * c.x + w2 * c.y < x);
    }
    blk = min(blk, nb - 1);
    cnt = blk << 4;
    const float4* b4 = r4 + (blk << 3);
    const int nq = min(8, (stride >> 1) - (blk << 3));
#pragma unroll 8
    for (int q = 0; q < nq; ++q) {
      const float4 c = __ldg(&b4[q]);
      cnt += (w1 * c.x + w2 * c.y < x) + (w1 * c.z + w2 * c.w < x);
    }
  }
  return min(cnt, P - 1);
}

// Null test of a cold gas (BoltzmannMC.C:1033-1052): r = U nu_trial against
// the interpolated total frequency. False for a null collision; r is kept
// for the process choice.
// With `coarse` (a copy of the table's block bounds, e.g. in shared memory)
// most null collisions are decided without loading the table row: r above the
// bound of the row's block is above the interpolated frequency too.
template <class Rng>
__device__ __forceinline__ bool cold_real(const TablesF& t, float nu_trial, float energy, Rng& rng, float& r,
                                          const float* coarse = nullptr) {
  r = nu_trial * rng.oc();
  int i1;
  float w1, w2;
  row_weights(energy * t.inv_step, t.M, i1, w1, w2);
  if (coarse && r > coarse[i1 >> t.coarse_shift]) return false;
  const float2 nt = __ldg(&t.nu_pair[i1]);
  return !(r > w1 * nt.x + w2 * nt.y);
}

// Process of a real cold collision whose null test drew r (BoltzmannMC.C:1053-1097):
// the first interpolated cumulative sum that reaches r/(N|v|), backward skip of
// zero-rate processes.
__device__ __forceinline__ int cold_choice(const TablesF& t, float energy, float speed, float r) {
  int i1;
  float w1, w2;
  row_weights(energy * t.inv_step, t.M, i1, w1, w2);
  const float rcs = r * t.inv_N / speed;
  int chosen = row_count_below(t.cum_pair + (size_t)i1 * t.stride, t.P, t.stride, w1, w2, rcs);
  const float2* sig = t.sig_pair + (size_t)i1 * t.stride;
  while (chosen > 0) {
    const float2 s2 = __ldg(&sig[chosen]);
    if (!(w1 * s2.x == 0.0f && w2 * s2.y == 0.0f)) break;
    --chosen;
  }
  return chosen;
}

// Process choice for a cold gas: -1 for null.
template <class Rng>
__device__ __forceinline__ int choose_cold(const TablesF& t, float nu_trial, float energy, float speed, Rng& rng) {
  float r;
  if (!cold_real(t, nu_trial, energy, rng, r)) return -1;
  return cold_choice(t, energy, speed, r);
}

// Process choice with thermal targets, gas by gas (BoltzmannMC.C:916-1031):
// Maxwellian target velocity from three normals (Box-Muller on four
// uniforms, MathFunctions.C:54-59), 0/1 row weights, per-gas bisection.
template <class Rng>
__device__ __forceinline__ int choose_thermal(const TablesF& t, const GasF* gases, int G, float nu_trial, float3 v,
                                              Rng& rng, float3& tv, float inv_qe) {
  float n0, n1, n2;
  {
    const float r1 = rng.oc(), r2 = rng.oc(), r3 = rng.oc(), r4 = rng.oc();
    const float a = sqrtf(-2.0f * __logf(r1));
    float sb, cb;
    sincosf(kTwoPiF * r2, &sb, &cb);
    n0 = a * cb;
    n1 = a * sb;
    n2 = sqrtf(-2.0f * __logf(r3)) * cosf(kTwoPiF * r4);
  }
  const float rcs = nu_trial * rng.oc() * t.inv_N;
  float prev = 0.0f;
  int chosen = -1;
  for (int g = 0; g < G && chosen == -1; ++g) {
    const GasF gs = gases[g];
    if (gs.fraction == 0.0f) continue;
    int L = gs.first, R = gs.last;
    tv = make_float3(n0 * gs.thermal_sd, n1 * gs.thermal_sd, n2 * gs.thermal_sd);
    const float rx = v.x - tv.x, ry = v.y - tv.y, rz = v.z - tv.z;
    const float rs = sqrtf(rx * rx + ry * ry + rz * rz);
    const float reos = 0.5f * gs.red_mass * rs * rs * inv_qe * t.inv_step;
    int i1 = (int)fminf(reos, (float)(t.M - 1));
    const int i2 = min(i1 + 1, t.M - 1);
    // BoltzmannMC.C:959-967: the weight is 0 or 1
    const float w1 = ((float)i2 - reos < 0.0f) ? 0.0f : 1.0f;
    const float w2 = 1.0f - w1;
    const float2* cum = t.cum_pair + (size_t)i1 * t.stride;
    float ref = 0.0f;
    if (L > 0) {
      const float2 c2 = __ldg(&cum[L - 1]);
      ref = w1 * c2.x + w2 * c2.y;
    }
    const float2 cr = __ldg(&cum[R]);
    const float lim = prev + (w1 * cr.x + w2 * cr.y - ref) * rs;
    if (rcs > lim) {
      prev = lim;
      continue;
    }
    while (L != R) {
      const int m = (L + R) >> 1;
      const float2 c2 = __ldg(&cum[m]);
      const float tvl = prev + (w1 * c2.x + w2 * c2.y - ref) * rs;
      if (rcs < tvl) R = m;
      else if (rcs > tvl) L = m + 1;
      else { chosen = m; break; }
    }
    if (L == R) chosen = L;
    const float2* sig = t.sig_pair + (size_t)i1 * t.stride;
    while (chosen > 0) {
      const float2 s2 = __ldg(&sig[chosen]);
      if (!(w1 * s2.x == 0.0f && w2 * s2.y == 0.0f)) break;
      --chosen;
    }
  }
  return chosen;
}

// Whether the event samples a thermal target (BoltzmannMC.C:916).
__device__ __forceinline__ bool is_thermal(const Consts& c, float energy) {
  return (c.gas_temp == kGasTempTrue) || (c.gas_temp == kGasTempSmart && energy < c.smart_energy);
}

// The rest of a collision event once a cold gas's null test said real (with
// its r), or the whole event for a thermal target (r unused).
template <class Rng>
__device__ __forceinline__ void collide_pending(const Consts& c, const TablesF& t, const ProcF* procs,
                                                const GasF* gases, float nu_trial, float r, float3& v,
                                                float& energy, Rng& rng, CollResult& out) {
  out.chosen = -1;
  out.dE = 0.0f;
  out.ionized = 0;
  const bool thermal = is_thermal(c, energy);
  float3 tv = make_float3(0.f, 0.f, 0.f);
  int ch;
  if (thermal) {
    ch = choose_thermal(t, gases, c.G, nu_trial, v, rng, tv, c.inv_qe);
  } else {
    const float speed = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    ch = cold_choice(t, energy, speed, r);
  }
  if (ch < 0) return;
  const ProcF pr = procs[ch];
  if (!apply_collision(c, pr, thermal, tv, v, energy, rng, out)) return;
  out.chosen = ch;
}

// One collision event at the end of a free flight (BoltzmannMC.C:907-1113).
template <class Rng>
__device__ __forceinline__ void collide(const Consts& c, const TablesF& t, const ProcF* procs, const GasF* gases,
                                        float nu_trial, float3& v, float& energy, Rng& rng, CollResult& out) {
  float r = 0.0f;
  if (!is_thermal(c, energy) && !cold_real(t, nu_trial, energy, rng, r)) {
    out.chosen = -1;
    out.dE = 0.0f;
    out.ionized = 0;
    return;
  }
  collide_pending(c, t, procs, gases, nu_trial, r, v, energy, rng, out);
}

}  // namespace lgpu
