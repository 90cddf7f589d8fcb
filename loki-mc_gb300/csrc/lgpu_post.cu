// lgpu_post.cu - the reference's end-of-job routines that read the EEDF, on
// the device in FP64: the EEDF-convolved rate coefficient of every MC process
// (Collision::evaluateRateCoeff, Collision.C:355-397) and the two-term swarm
// parameters (BoltzmannMC::evaluateSwarmParameters, BoltzmannMC.C:2186-2266).
//
// Built with -fmad=false: every elementwise step rounds as the reference's
// (whose build contracts nothing), so the per-node totals of the
// momentum-transfer and energy-relaxation cross sections come out bit for
// bit; the sums over cells run as a fixed-order block reduction, so they
// agree with the reference's to rounding.
#include "lgpu_kernels.cuh"

namespace lgpu {

namespace {

constexpr int kPostThreads = 512;
constexpr double kQeP = 1.6021766208e-19;  // C (Constant.h:7)
constexpr double kMeP = 9.10938356e-31;    // kg (Constant.h:8)

// Sum over the block in a fixed order (every thread calls it; the result on
// every thread).
__device__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();  // red[] free again
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
  return s;
}

// The grid of Grid::updateMaxValue (Grid.C:44-53) as Eigen's LinSpaced lays
// it out: node i = i * step with the last node the maximum itself; cell l =
// step/2 + l * cell step with the last cell max - step/2.
struct PostGrid {
  double max, step, lo, hi, cstep;
  int nc;
  __device__ double node(int i) const { return i == nc ? max : (double)i * step; }
  __device__ double cell(int l) const { return l == nc - 1 ? hi : lo + (double)l * cstep; }
};

// Collision::interpolatedCrossSection (Collision.C:229-288) at one energy:
// linear between the bracketing raw points (largest lower point by
// bisection), zero outside the table.
__device__ double raw_at(const double* e, const double* v, int n, double x) {
  if (n < 2 || x < e[0] || x > e[n - 1]) return 0.0;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (hi + lo) >> 1;
    if (e[mid] > x) hi = mid;
    else lo = mid;
  }
  return v[lo] + (x - e[lo]) / (e[lo + 1] - e[lo]) * (v[lo + 1] - v[lo]);
}

// sum over cells l = lmin .. nc-1 of (sig_l + sig_l+1) / 2 * cell_l * eedf_(l - shift)
__device__ double conv_sum(const PostGrid& g, const double* sig, const double* eedf, int lmin, int shift,
                           double* red) {
  double s = 0.0;
  for (int l = lmin + (int)threadIdx.x; l < g.nc; l += blockDim.x)
    s += (sig[l] + sig[l + 1]) / 2.0 * g.cell(l) * eedf[l - shift];
  return block_sum(s, red);
}

// One block per EEDF (row blockIdx.x of eedf_in or eeh); the two-term swarm
// parameters from row 0 unless rates_only.
__global__ void __launch_bounds__(kPostThreads) k_eedf_post(EedfPostArgs a) {
  __shared__ double red[kPostThreads / 32];
  const int nc = a.nc, nn = nc + 1;
  const int row = blockIdx.x;
  if (a.eedf_in) a.eedf_in += (size_t)row * nc;
  a.eeh += (size_t)row * nc;
  a.scratch += (size_t)row * 5 * nn;
  a.rates += (size_t)row * a.P;
  PostGrid g;
  g.nc = nc;
  g.max = a.max_energy;
  g.step = a.max_energy / nc;
  g.lo = g.step / 2.0;
  g.hi = a.max_energy - g.step / 2.0;
  g.cstep = nc > 1 ? (g.hi - g.lo) / (nc - 1) : 0.0;
  double* eedf = a.scratch;
  double* mt = eedf + nn;
  double* er = mt + nn;
  double* erc = er + nn;
  double* sig = erc + nn;  // the last forward collision's integral cross section on the nodes
  // the EEDF: given, or normalised from the context's histogram sums
  // (BoltzmannMC.C:1580: f = h / (sqrt(cell) sum(h) step))
  if (a.eedf_in) {
    for (int l = threadIdx.x; l < nc; l += blockDim.x) eedf[l] = a.eedf_in[l];
  } else {
    double s = 0.0;
    for (int l = threadIdx.x; l < nc; l += blockDim.x) s += a.eeh[l];
    const double norm = block_sum(s, red);
    for (int l = threadIdx.x; l < nc; l += blockDim.x) eedf[l] = a.eeh[l] / (sqrt(g.cell(l)) * norm * g.step);
  }
  for (int i = threadIdx.x; i < nn; i += blockDim.x) mt[i] = er[i] = erc[i] = 0.0;
  __syncthreads();
  const double factor2 = sqrt(2.0 * kQeP / kMeP);
  const double factor = factor2 / 3.0;
  double k_ion = 0.0, k_att = 0.0;
  for (int p = 0; p < a.P; ++p) {
    const double thr = a.thr[p], dens = a.dens[p];
    const double* ie = a.raw_ie + a.int_off[p];
    const double* iv = a.raw_iv + a.int_off[p];
    const double* me = a.raw_me + a.mom_off[p];
    const double* mv = a.raw_mv + a.mom_off[p];
    const int ni = a.int_len[p], nm = a.mom_len[p];
    const int lmin = (int)floor(thr / g.step);
    if (a.kind[p] == 2) {
      // superelastic copy: Klein-Rosseland at the nodes (Collision.C:290-353),
      // zero at the zero-energy node (BoltzmannMC.C:2205-2217)
      for (int i = 1 + (int)threadIdx.x; i < nn; i += blockDim.x) {
        const double u = g.node(i), x = u + thr, kr = 1.0 + thr / u;
        const double s_int = kr * (raw_at(ie, iv, ni, x) * a.stat[p]);
        const double s_mom = kr * (raw_at(me, mv, nm, x) * a.stat[p]);
        const double w = s_int * dens;
        mt[i] = mt[i] + s_mom * dens;
        er[i] = er[i] + w * thr / u;
        erc[i] = erc[i] + w;
      }
      double r = 0.0;
      const int part = nc - lmin;
      if (part > 0) {
        // the forward collision's cross section, shifted EEDF (Collision.C:390)
        double s = 0.0;
        for (int k = threadIdx.x; k < part; k += blockDim.x) {
          const int l = lmin + k;
          s += (sig[l] + sig[l + 1]) / 2.0 * g.cell(l) * eedf[k];
        }
        r = factor2 * a.stat[p] * block_sum(s, red) * g.step;
      }
      if (threadIdx.x == 0) a.rates[p] = r;
      __syncthreads();
      continue;
    }
    // forward collision: cross sections on the nodes (Collision.C:221-228:
    // every node for elastic collisions, from the first node above the
    // threshold otherwise)
    const bool elastic = a.kind[p] == 0;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const double x = g.node(i);
      const bool on = elastic || x > thr;
      const double s_int = on ? raw_at(ie, iv, ni, x) : 0.0;
      const double s_mom = on ? raw_at(me, mv, nm, x) : 0.0;
      sig[i] = s_int;
      mt[i] = mt[i] + s_mom * dens;
      if (elastic) {
        er[i] = er[i] + 2.0 * a.mass_ratio[p] * s_int * dens;
      } else {
        const double w = s_int * dens;
        if (i > 0) er[i] = er[i] + w * thr / x;
        erc[i] = erc[i] + w;
      }
    }
    __syncthreads();
    double r = 0.0;
    if (nc - lmin > 0) r = factor2 * conv_sum(g, sig, eedf, lmin, 0, red) * g.step;
    if (threadIdx.x == 0) a.rates[p] = r;
    if (a.ion[p] == 1) k_ion += dens * r;
    if (a.ion[p] == 2) k_att += dens * r;
    __syncthreads();
  }
  if (a.rates_only) return;
  // two-term swarm parameters (BoltzmannMC.C:2220-2266)
  const double N = a.gas_density, w = a.omega, wc = a.omega_c;
  const double growth = k_ion - k_att;
  auto mta = [&](int i) {  // momentum transfer plus the growth term (BoltzmannMC.C:2233-2234)
    return i == 0 ? mt[0] : mt[i] + 1.0 / (3.0 * factor * sqrt(g.node(i))) * growth;
  };
  double s_mt = 0, s_er = 0, s_erc = 0, s_de = 0, s_d = 0, s_me = 0, s_m = 0;
  double s_xr = 0, s_xi = 0, s_yr = 0, s_yi = 0, s_zr = 0, s_zi = 0;
  for (int l = threadIdx.x; l < nc; l += blockDim.x) {
    const double c = g.cell(l), f = eedf[l];
    s_mt += f * c * ((mt[l + 1] + mt[l]) * 0.5);
    s_er += f * c * ((er[l + 1] + er[l]) * 0.5);
    s_erc += f * c * ((erc[l + 1] + erc[l]) * 0.5);
    const double den = mta(l) + mta(l + 1);
    s_de += c * c * f / den;
    s_d += c * f / den;
    if (l >= 1) {
      const double x = g.node(l), m = mta(l), df = f - eedf[l - 1];
      s_me += x * x * df / m;
      s_m += x * df / m;
      const double aux1 = -2.0 / 3.0 * kQeP / kMeP * pow(x, 1.5) * df;
      const double fr = N * m * 3.0 * factor * sqrt(x);
      const double f2 = fr * fr;
      const double aux2 = (f2 + (w - wc) * (w - wc)) * (f2 + (w + wc) * (w + wc));
      const double aux3 = f2 + w * w;
      s_xr += fr * (f2 + w * w + wc * wc) / aux2 * aux1;
      s_xi += w * (f2 + w * w - wc * wc) / aux2 * aux1;
      s_yr += (f2 - w * w + wc * wc) / aux2 * aux1;
      s_yi += fr / aux2 * aux1;
      s_zr += fr / aux3 * aux1;
      s_zi += w / aux3 * aux1;
    }
  }
  const double pre = N * 3.0 * factor * g.step;
  const double v_mt = pre * block_sum(s_mt, red);
  const double v_er = pre * block_sum(s_er, red);
  const double v_erc = pre * block_sum(s_erc, red);
  const double v_de = 2.0 * factor * g.step * block_sum(s_de, red);
  const double v_me = -factor * block_sum(s_me, red);
  const double v_d = 2.0 * factor * g.step * block_sum(s_d, red);
  const double v_m = -factor * block_sum(s_m, red);
  const double v_xr = N * block_sum(s_xr, red);
  const double v_xi = -N * block_sum(s_xi, red);
  const double v_yr = -N * wc * block_sum(s_yr, red);
  const double v_yi = N * 2.0 * w * wc * block_sum(s_yi, red);
  const double v_zr = N * block_sum(s_zr, red);
  const double v_zi = -N * block_sum(s_zi, red);
  if (threadIdx.x == 0) {
    double* o = a.params;
    o[0] = k_ion;
    o[1] = k_att;
    o[2] = v_mt;
    o[3] = v_er;
    o[4] = v_erc;
    o[5] = v_de;
    o[6] = v_me;
    o[7] = v_d;
    o[8] = v_m;
    o[9] = v_d / v_m;
    o[10] = v_xr;
    o[11] = v_xi;
    o[12] = v_yr;
    o[13] = v_yi;
    o[14] = v_zr;
    o[15] = v_zi;
  }
}

}  // namespace

void launch_eedf_post(const EedfPostArgs& a, cudaStream_t s) {
  k_eedf_post<<<a.n_eedf, kPostThreads, 0, s>>>(a);
}

}  // namespace lgpu
