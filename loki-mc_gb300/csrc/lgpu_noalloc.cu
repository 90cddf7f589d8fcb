// lgpu_noalloc.cu - free flights without any device allocation.
//
// Some callers cannot call cudaMalloc: a serving process that reserved the
// device's memory up front and hands out nothing more, a host application
// whose own allocator owns every device byte, or a code path that must not
// allocate (and so must not risk the implicit synchronisation an allocation
// can cause) between two stages of its own pipeline. For them this file gives
// one entry point, lgpu_replay_flights_noalloc, that runs the free-flight
// kernel of the library (the closed-form push of BoltzmannMC.C:804-905, the
// same device code as lgpu_replay_flights) with its staging memory in a
// file-scope device array instead of buffers of a context.
//
// The array is static device memory: every GPU that loads the library holds
// it (512 KiB) until the process exits. Its host-side name is only a handle;
// the device address is looked up once per device with cudaGetSymbolAddress
// (the first call on a device does it, so that first call should come before
// any stream capture) and kept for the life of the process, so the entry point
// must not be used on a device after cudaDeviceReset there. The caller's
// current device is restored before the call returns. Every call shares the array and leaves its contents
// behind; calls whose work overlaps on the GPU (two host threads, or two
// streams) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/loki_gpu.h"
#include "lgpu_device.cuh"

namespace {

constexpr int kNoAllocMaxFlights = 4096;
constexpr int kNoAllocDoubles = 16 * kNoAllocMaxFlights;  // 8 inputs + 8 outputs per flight
constexpr int kMaxDevices = 64;
constexpr double kPiD = 3.14159265358979323846;

// staging: [t | dt | pos x3 | vel x3] then [pos x3 | vel x3 | energy | gain], n entries each
static __device__ __align__(256) double g_flight_scratch[kNoAllocDoubles];

double* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

__global__ void k_replay_flight_noalloc(int n, const double* in, double* out, lgpu::FieldF field, double phase_rate,
                                        float hme) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* t = in;
  const double* dt = in + n;
  const double* pos = in + 2 * (size_t)n;
  const double* vel = in + 5 * (size_t)n;
  // phase at the flight start, reduced in FP64 (fmod is exact)
  const double phi0 = phase_rate != 0.0 ? fmod(phase_rate * t[i], 2.0 * kPiD) : 0.0;
  float3 p = make_float3((float)pos[3 * i], (float)pos[3 * i + 1], (float)pos[3 * i + 2]);
  float3 v = make_float3((float)vel[3 * i], (float)vel[3 * i + 1], (float)vel[3 * i + 2]);
  const float e0 = lgpu::energy_of(v, hme);
  lgpu::free_flight(field, (float)phi0, (float)dt[i], p, v);
  const float e1 = lgpu::energy_of(v, hme);
  out[3 * i] = p.x;
  out[3 * i + 1] = p.y;
  out[3 * i + 2] = p.z;
  out[3 * (size_t)n + 3 * i] = v.x;
  out[3 * (size_t)n + 3 * i + 1] = v.y;
  out[3 * (size_t)n + 3 * i + 2] = v.z;
  out[6 * (size_t)n + i] = e1;
  out[7 * (size_t)n + i] = e1 - e0;
}

// Device address of the staging array on the current device, looked up once
// per device (with that device current).
int scratch_for_device(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return LGPU_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_flight_scratch);
    if (e != cudaSuccess) {
      std::fprintf(stderr, "lgpu_replay_flights_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return LGPU_ERR_CUDA;
    }
    g_scratch_ptr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[device];
  return LGPU_OK;
}

int run_flights(int device, const double e_field[3], double freq_hz, double red_mag_hx, double cyclotron, int n,
                const double* t, const double* dt, const double* pos, const double* vel, double* pos_out,
                double* vel_out, double* energy_out, double* gain_out);

}  // namespace

extern "C" int lgpu_replay_flights_noalloc(int device, const double e_field[3], double freq_hz, double red_mag_hx,
                                           double cyclotron, int n, const double* t, const double* dt,
                                           const double* pos, const double* vel, double* pos_out, double* vel_out,
                                           double* energy_out, double* gain_out) {
  if (n < 0 || !e_field) return LGPU_ERR_BAD_ARG;
  if (n > kNoAllocMaxFlights) {
    std::fprintf(stderr, "lgpu_replay_flights_noalloc: %d flights requested, the static staging holds at most %d\n", n,
                 kNoAllocMaxFlights);
    return LGPU_ERR_BAD_ARG;
  }
  if (n == 0) return LGPU_OK;
  if (!t || !dt || !pos || !vel || !pos_out || !vel_out || !energy_out || !gain_out) return LGPU_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return LGPU_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return LGPU_ERR_BAD_ARG;
  // the caller's current device is put back on every return path
  int prev_device = 0;
  if (cudaGetDevice(&prev_device) != cudaSuccess) return LGPU_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return LGPU_ERR_CUDA;
  const int rc = run_flights(device, e_field, freq_hz, red_mag_hx, cyclotron, n, t, dt, pos, vel, pos_out, vel_out,
                             energy_out, gain_out);
  if (cudaSetDevice(prev_device) != cudaSuccess && rc == LGPU_OK) return LGPU_ERR_CUDA;
  return rc;
}

namespace {

int run_flights(int device, const double e_field[3], double freq_hz, double red_mag_hx, double cyclotron, int n,
                const double* t, const double* dt, const double* pos, const double* vel, double* pos_out,
                double* vel_out, double* energy_out, double* gain_out) {
  double* scratch = nullptr;
  const int rc = scratch_for_device(device, &scratch);
  if (rc != LGPU_OK) return rc;

  // the field branch of BoltzmannMC.C:811-897, as lgpu_set_field_raw selects it
  const double qe = 1.6021766208e-19, me = 9.10938356e-31;
  const double omega = freq_hz * 2.0 * kPiD;
  lgpu::FieldF f{};
  f.ax = (float)(-qe / me * e_field[0]);
  f.ay = (float)(-qe / me * e_field[1]);
  f.az = (float)(-qe / me * e_field[2]);
  f.Ex = (float)e_field[0];
  f.Ez = (float)e_field[2];
  f.w = (float)omega;
  f.W = (float)cyclotron;
  f.e_me = (float)(qe / me);
  if (red_mag_hx == 0) f.mode = (freq_hz == 0) ? lgpu::kFieldDC : lgpu::kFieldAC;
  else if (freq_hz == 0) f.mode = lgpu::kFieldB;
  else if (std::abs(omega - cyclotron) / omega < 1E-6) f.mode = lgpu::kFieldECR;
  else f.mode = lgpu::kFieldACB;
  double phase_rate = 0.0;
  if (f.mode == lgpu::kFieldAC || f.mode == lgpu::kFieldACB) phase_rate = omega;
  else if (f.mode == lgpu::kFieldECR) phase_rate = cyclotron;

  // inputs straight from the caller's arrays into the static array, outputs
  // straight back: no other memory is used
  double* d_in = scratch;
  double* d_out = scratch + 8 * (size_t)kNoAllocMaxFlights;
  const size_t nb = (size_t)n * sizeof(double);
  if (cudaMemcpy(d_in, t, nb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_in + n, dt, nb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_in + 2 * (size_t)n, pos, 3 * nb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_in + 5 * (size_t)n, vel, 3 * nb, cudaMemcpyHostToDevice) != cudaSuccess)
    return LGPU_ERR_CUDA;
  k_replay_flight_noalloc<<<(n + 127) / 128, 128>>>(n, d_in, d_out, f, phase_rate, (float)(0.5 * me / qe));
  if (cudaGetLastError() != cudaSuccess) return LGPU_ERR_CUDA;
  if (cudaMemcpy(pos_out, d_out, 3 * nb, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(vel_out, d_out + 3 * (size_t)n, 3 * nb, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(energy_out, d_out + 6 * (size_t)n, nb, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(gain_out, d_out + 7 * (size_t)n, nb, cudaMemcpyDeviceToHost) != cudaSuccess)
    return LGPU_ERR_CUDA;
  return LGPU_OK;
}

}  // namespace
