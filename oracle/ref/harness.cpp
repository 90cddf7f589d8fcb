// Test infrastructure for the oracle build of the reference (never shipped).
//
// A C-callable wrapper around the reference engine built from its own
// sources (Code/LoKI-MC/Sources/*.C). It constructs Setup<BoltzmannMC> the
// way lokimc.C:14-41 does, exposes the flattened process arrays that
// BoltzmannMC::allocateEvaluateVariablesFirstTime builds
// (BoltzmannMC.C:29-271), and lets a driver script call the per-electron
// routines accelerateElectron (BoltzmannMC.C:804-905) and performCollision
// (BoltzmannMC.C:907-1113) on chosen electron states with a replayed stream
// of uniforms, or run a full solve() (BoltzmannMC.C:273-297) with a seeded
// generator. Its outputs become the golden vectors under tests/golden/.
#include "LoKI-MC/Headers/BoltzmannMC.h"
#include "LoKI-MC/Headers/Constant.h"
#include "LoKI-MC/Headers/FieldInfo.h"
#include "LoKI-MC/Headers/Parse.h"
#include "LoKI-MC/Headers/Setup.h"

#include <cmath>
#include <cstring>
#include <string>

namespace {
Setup<BoltzmannMC>* g_setup = nullptr;
BoltzmannMC* g_mc = nullptr;

int sampler_code(Collision* c) {
  const std::string& t = c->angularScatteringType;
  if (t == "isotropic") return 0;
  if (t == "forward") return 1;
  if (t == "bornDipole") return 2;
  if (t == "surendra") return 3;
  if (t == "coulombScreen") return 4;
  if (t == "momentumConservationIonization") return 5;
  return -1;
}
}  // namespace

extern "C" {

int ref_open(const char* setup_file) {
  std::string name(setup_file);
  Parse::setupFile(name);
  g_setup = new Setup<BoltzmannMC>(name);
  g_setup->initializeSimulation();
  g_mc = g_setup->electronKinetics;
  return g_mc ? g_mc->nProcesses : -1;
}

int ref_n_processes() { return g_mc->nProcesses; }
int ref_n_gases() { return g_mc->nGases; }
int ref_n_electrons() { return (int)g_mc->nElectrons; }
int ref_table_size() { return g_mc->interpolCrossSectionSize; }

// per-process scalars (length nProcesses each)
void ref_get_processes(int* type, int* is_super, int* is_elastic, int* sampler, double* sampler_p0,
                       double* sampler_p1, int* is_momcons, double* superw, double* emin, double* emax,
                       double* rel_dens, double* mass, double* red_mass, double* eloss, double* wparam,
                       int* raw_len) {
  BoltzmannMC* m = g_mc;
  for (int i = 0; i < m->nProcesses; ++i) {
    type[i] = m->processTypes[i];
    is_super[i] = m->isSuperElastic[i] ? 1 : 0;
    is_elastic[i] = (m->realCollisionPointers[i]->type == "Elastic" && !m->isSuperElastic[i]) ? 1 : 0;
    sampler[i] = sampler_code(m->realCollisionPointers[i]);
    const std::vector<double>& pr = m->angularScatteringParams[i];
    sampler_p0[i] = pr.size() > 0 ? pr[0] : 0.0;
    sampler_p1[i] = pr.size() > 1 ? pr[1] : 0.0;
    is_momcons[i] = m->isMomentumConservationIonizationScattering[i] ? 1 : 0;
    superw[i] = m->superElasticStatWeightFactors[i];
    emin[i] = m->energyMinLimits[i];
    emax[i] = m->energyMaxLimits[i];
    rel_dens[i] = m->relDensities[i];
    mass[i] = m->targetMasses[i];
    red_mass[i] = m->reducedMasses[i];
    eloss[i] = m->energyLosses[i];
    wparam[i] = m->wParameters[i];
    raw_len[i] = (int)m->crossSectionEnergies[i].size();
  }
}

void ref_get_raw(int p, double* e, double* v) {
  const Eigen::ArrayXd& E = g_mc->crossSectionEnergies[p];
  const Eigen::ArrayXd& V = g_mc->crossSectionValues[p];
  for (int k = 0; k < E.size(); ++k) {
    e[k] = E[k];
    v[k] = V[k];
  }
}

void ref_get_gases(double* first, double* last, double* frac) {
  for (int g = 0; g < g_mc->nGases; ++g) {
    first[g] = g_mc->firstProcessIndexPerGas[g];
    last[g] = g_mc->lastProcessIndexPerGas[g];
    frac[g] = g_mc->gasFractions[g];
  }
}

// scalars: [0] totalGasDensity [1] gasTemperature [2] energyMaxElastic
// [3] E/N (Td) [4] elecFieldAngle [5] excitationFrequency (Hz) [6] B/N (Hx)
// [7] cyclotronFrequency [8] electric field x [9] y [10] z
// [11] energySharingIonizType [12] energySharingFactor [13] gasTemperatureEffect
// [14] trialCollisionFrequency [15] maxInterpolatedEnergy [16] crossSectionEnergyStep
// [17] gasEnergy [18] initialElecTempOverGasTemp [19] synchronizationTimeXMaxCollisionFrequency
void ref_get_scalars(double* s) {
  BoltzmannMC* m = g_mc;
  s[0] = m->totalGasDensity;
  s[1] = m->gasTemperature;
  s[2] = m->energyMaxElastic;
  s[3] = m->reducedElecField;
  s[4] = m->elecFieldAngle;
  s[5] = m->excitationFrequency;
  s[6] = m->reducedMagField;
  s[7] = m->cyclotronFrequency;
  s[8] = m->electricField[0];
  s[9] = m->electricField[1];
  s[10] = m->electricField[2];
  s[11] = m->energySharingIonizType;
  s[12] = m->energySharingFactor;
  s[13] = m->gasTemperatureEffect;
  s[14] = m->trialCollisionFrequency;
  s[15] = m->maxInterpolatedEnergy;
  s[16] = m->crossSectionEnergyStep;
  s[17] = m->gasEnergy;
  s[18] = m->initialElecTempOverGasTemp;
  s[19] = m->synchronizationTimeXMaxCollisionFrequency;
}

// BoltzmannMC.C:428-559 (per-job variables, initial ensemble, first tables)
void ref_eval_nonconstant() {
  g_mc->maxInterpolatedEnergy = -1.0;
  g_mc->evaluateNonConstantVariables();
}

// BoltzmannMC.C:561-615
void ref_interpolate(double max_energy) { g_mc->interpolateCrossSections(max_energy); }

void ref_get_tables(double* grid, double* sig, double* cum, double* nu_tot, double* nu_max) {
  BoltzmannMC* m = g_mc;
  const int M = m->interpolCrossSectionSize, P = m->nProcesses;
  for (int i = 0; i < M; ++i) {
    grid[i] = m->crossSectionEnergyGrid[i];
    nu_tot[i] = m->totalCollisionFrequencies[i];
    nu_max[i] = m->maxCollisionFrequencies[i];
    for (int p = 0; p < P; ++p) {
      sig[(size_t)i * P + p] = m->interpolCrossSectionsXrelDens[i][p];
      cum[(size_t)i * P + p] = m->cumulSumInterpolCrossSectionsXrelDens[i][p];
    }
  }
}

// Overrides the field state that accelerateElectron reads
// (BoltzmannMC.C:461-489): E vector (V/m, already including the AC sqrt(2)),
// excitation frequency (Hz), B/N (Hx, only tested against zero) and the
// cyclotron frequency (rad/s).
void ref_set_fields(double ex, double ey, double ez, double exc_hz, double red_mag, double cyclotron) {
  BoltzmannMC* m = g_mc;
  m->electricField[0] = ex;
  m->electricField[1] = ey;
  m->electricField[2] = ez;
  m->excitationFrequency = exc_hz;
  m->excitationFrequencyRadians = exc_hz * 2.0 * M_PI;
  m->reducedMagField = red_mag;
  m->cyclotronFrequency = cyclotron;
  m->accelerationElecField = -Constant::electronCharge / Constant::electronMass * m->electricField;
}

void ref_set_collision_options(int gas_temp_effect, int sharing_type, double sharing_factor) {
  g_mc->gasTemperatureEffect = gas_temp_effect;
  g_mc->energySharingIonizType = sharing_type;
  g_mc->energySharingFactor = sharing_factor;
}

// BoltzmannMC.C:804-905. io: pos[3], vel[3], energy in; out the same plus the
// field energy gain.
void ref_accelerate(double t, double dt, double* pos, double* vel, double* energy, double* gain) {
  Eigen::Array3d p(pos[0], pos[1], pos[2]), v(vel[0], vel[1], vel[2]);
  double e = *energy;
  g_mc->accelerateElectron(0, t, dt, p, v, e);
  for (int k = 0; k < 3; ++k) {
    pos[k] = p[k];
    vel[k] = v[k];
  }
  *energy = e;
  *gain = g_mc->energyGainsField[0];
}

// BoltzmannMC.C:907-1113 for electron slot 0 with the given trial frequency.
// out[0] chosen process id, out[1..3] velocity, out[4] energy,
// out[5] energy change, out[6] change / incident energy,
// out[7..9] ejected velocity, out[10] ejected energy.
void ref_collide(double nu_trial, double* pos, double* vel, double energy, double* out) {
  BoltzmannMC* m = g_mc;
  m->trialCollisionFrequenciesEachElectron[0] = nu_trial;
  m->electronEnergyChanges[0] = 0;
  m->electronEnergyChangesOverIncidEnergies[0] = 0;
  m->ejectedElectronVelocities.row(0) = Eigen::Array3d::Zero();
  m->ejectedElectronEnergies[0] = 0;
  Eigen::Array3d p(pos[0], pos[1], pos[2]), v(vel[0], vel[1], vel[2]);
  double e = energy;
  m->performCollision(0, p, v, e);
  out[0] = m->chosenProcessIDs[0];
  out[1] = v[0];
  out[2] = v[1];
  out[3] = v[2];
  out[4] = e;
  out[5] = m->electronEnergyChanges[0];
  out[6] = m->electronEnergyChangesOverIncidEnergies[0];
  out[7] = m->ejectedElectronVelocities(0, 0);
  out[8] = m->ejectedElectronVelocities(0, 1);
  out[9] = m->ejectedElectronVelocities(0, 2);
  out[10] = m->ejectedElectronEnergies[0];
}

// Full solve (BoltzmannMC.C:273-297) with the current RNG mode. Results:
// r[0] mean energy, r[1] its error, r[2..4] flux v, r[5..7] errors,
// r[8..10] flux D diag, r[11..13] errors, r[14..16] bulk v, r[17..19] errors,
// r[20..22] bulk D diag, r[23..25] errors, r[26] real collisions,
// r[27] null collisions, r[28] elapsed s, r[29] power balance rel. error,
// r[30] steady-state time, r[31] final time, r[32] integration points,
// r[33] collisions at SS, r[34] null at SS, r[35] trial freq,
// r[36] power field, r[37] power growth, r[38] max EEDF energy.
// rate[nProcesses] MC rate coefficients.
void ref_solve(double* r, double* rate) {
  BoltzmannMC* m = g_mc;
  m->maxInterpolatedEnergy = -1.0;
  m->solve();
  r[0] = m->averagedMeanEnergy;
  r[1] = m->averagedMeanEnergyError;
  for (int k = 0; k < 3; ++k) {
    r[2 + k] = m->averagedFluxDriftVelocity[k];
    r[5 + k] = m->averagedFluxDriftVelocityError[k];
    r[8 + k] = m->averagedFluxDiffusionCoeffs(k, k);
    r[11 + k] = m->averagedFluxDiffusionCoeffsError(k, k);
    r[14 + k] = m->averagedBulkDriftVelocity[k];
    r[17 + k] = m->averagedBulkDriftVelocityError[k];
    r[20 + k] = m->averagedBulkDiffusionCoeffs(k, k);
    r[23 + k] = m->averagedBulkDiffusionCoeffsError(k, k);
  }
  r[26] = (double)m->totalCollisionCounter;
  r[27] = (double)m->nullCollisionCounter;
  r[28] = m->elapsedTime;
  r[29] = m->powerBalanceRelError;
  r[30] = m->steadyStateTime;
  r[31] = m->time;
  r[32] = m->nIntegrationPoints;
  r[33] = (double)m->collisionCounterAtSS;
  r[34] = (double)m->nullCollisionCounterAtSS;
  r[35] = m->trialCollisionFrequency;
  r[36] = m->averagedPowerGainField;
  r[37] = m->averagedPowerGrowth;
  r[38] = m->maxEedfEnergy;
  for (int i = 0; i < m->nProcesses; ++i) rate[i] = m->averagedRateCoeffs[i];
}

int ref_n_eedf_cells() { return (int)g_mc->nEnergyCells; }
void ref_get_eedf(double* cells, double* eedf) {
  for (int i = 0; i < (int)g_mc->nEnergyCells; ++i) {
    cells[i] = g_mc->eedfEnergyCells[i];
    eedf[i] = g_mc->eedf[i];
  }
}

// Distributions and periodic averages after a solve (BoltzmannMC.C:1574-1605,
// 1728-1741). sizes: energy cells, cos cells, radial cells, axial cells,
// phases, cylindrical symmetry (EADF/EVDF exist), AC field (periodic outputs).
void ref_dist_sizes(int* s) {
  BoltzmannMC* m = g_mc;
  s[0] = (int)m->nEnergyCells;
  s[1] = (int)m->nCosAngleCells;
  s[2] = (int)m->nRadialVelocityCells;
  s[3] = (int)m->nAxialVelocityCells;
  s[4] = (int)m->nIntegrationPhases;
  s[5] = m->isCylindricallySymmetric ? 1 : 0;
  s[6] = m->excitationFrequencyRadians != 0 ? 1 : 0;
}

// efadf, esadf [nE]; eadf [nE x nCos] and evdf [nR x nA] row-major; radial and
// axial cell centres (cylindrical conditions only)
void ref_get_anisotropic(double* f1, double* f2, double* eadf, double* evdf, double* rc, double* ac) {
  BoltzmannMC* m = g_mc;
  const int nE = (int)m->nEnergyCells, nC = (int)m->nCosAngleCells, nR = (int)m->nRadialVelocityCells,
            nA = (int)m->nAxialVelocityCells;
  for (int i = 0; i < nE; ++i) {
    f1[i] = m->efadf[i];
    f2[i] = m->esadf[i];
    for (int k = 0; k < nC; ++k) eadf[(size_t)i * nC + k] = m->eadf(i, k);
  }
  for (int i = 0; i < nR; ++i) {
    rc[i] = m->radialVelocityCells[i];
    for (int k = 0; k < nA; ++k) evdf[(size_t)i * nA + k] = m->evdf(i, k);
  }
  for (int k = 0; k < nA; ++k) ac[k] = m->axialVelocityCells[k];
}

// per phase: samples, mean energy, flux and bulk velocity (x3), flux and bulk
// diffusion (x9), EEDF [nPh x nE] (AC conditions only)
void ref_get_periodic(double* n, double* me, double* fv, double* bv, double* fd, double* bd, double* eedf_per) {
  BoltzmannMC* m = g_mc;
  const int nPh = (int)m->nIntegrationPhases, nE = (int)m->nEnergyCells;
  for (int q = 0; q < nPh; ++q) {
    n[q] = m->nIntegrationPointsPerPhase[q];
    me[q] = m->meanEnergies_periodic[q];
    for (int k = 0; k < 3; ++k) {
      fv[3 * q + k] = m->fluxVelocities_periodic(q, k);
      bv[3 * q + k] = m->bulkVelocities_periodic(q, k);
    }
    for (int k = 0; k < 9; ++k) {
      fd[9 * q + k] = m->fluxDiffusionCoeffs_periodic(q, k);
      bd[9 * q + k] = m->bulkDiffusionCoeffs_periodic(q, k);
    }
    for (int c = 0; c < nE; ++c) eedf_per[(size_t)q * nE + c] = m->eedf_periodic(q, c);
  }
}

// time-averaged power per process, gain and loss (BoltzmannMC.C:1640-1649)
void ref_get_power(double* gain, double* loss) {
  for (int i = 0; i < g_mc->nProcesses; ++i) {
    gain[i] = g_mc->averagedPowerGainProcesses[i];
    loss[i] = g_mc->averagedPowerLossProcesses[i];
  }
}

// the mean-energy time series (samplingTimes, meanEnergies), its length first
int ref_n_samples() { return g_mc->nSamplingPoints; }
void ref_get_energy_series(double* t, double* e) {
  for (int i = 0; i < g_mc->nSamplingPoints; ++i) {
    t[i] = g_mc->samplingTimes[i];
    e[i] = g_mc->meanEnergies[i];
  }
}

// ---- EEDF post-processing pins (after ref_solve): the collision behind each
// MC process, as the reference's end-of-job routines read it
// (BoltzmannMC.C:2186-2266, 2268-2384; Collision.C:355-397)
int ref_twoterm_sizes(int i, int* n_int, int* n_mom) {
  Collision* c = g_mc->realCollisionPointers[i];
  *n_int = (int)c->rawIntegralCrossSection[0].size();
  *n_mom = (int)c->rawMomTransfCrossSection[0].size();
  return g_mc->isSuperElastic[i] ? 1 : 0;
}
// s: kind (0 elastic, 1 inelastic, 2 superelastic copy), density (target's, the
// product's for the copy), threshold (eV), m_e / M of the target gas,
// g_target / g_product (reversible collisions, else 0), 1 ionization / 2 attachment
void ref_get_twoterm(int i, double* s, double* int_e, double* int_v, double* mom_e, double* mom_v) {
  Collision* c = g_mc->realCollisionPointers[i];
  const bool sup = g_mc->isSuperElastic[i];
  s[0] = sup ? 2.0 : (c->type == "Elastic" ? 0.0 : 1.0);
  s[1] = sup ? c->productArray[0]->density : c->target->density;
  s[2] = c->threshold;
  s[3] = Constant::electronMass / c->target->gas->mass;
  s[4] = c->isReverse ? c->target->statisticalWeight / c->productArray[0]->statisticalWeight : 0.0;
  s[5] = c->type == "Ionization" ? 1.0 : (c->type == "Attachment" ? 2.0 : 0.0);
  for (size_t k = 0; k < c->rawIntegralCrossSection[0].size(); ++k) {
    int_e[k] = c->rawIntegralCrossSection[0][k];
    int_v[k] = c->rawIntegralCrossSection[1][k];
  }
  for (size_t k = 0; k < c->rawMomTransfCrossSection[0].size(); ++k) {
    mom_e[k] = c->rawMomTransfCrossSection[0][k];
    mom_v[k] = c->rawMomTransfCrossSection[1][k];
  }
}
// the EEDF-convolved rate coefficient of each MC process: ineRateCoeff of its
// collision, supRateCoeff for a superelastic copy
void ref_get_eedf_rates(double* rate) {
  for (int i = 0; i < g_mc->nProcesses; ++i) {
    Collision* c = g_mc->realCollisionPointers[i];
    rate[i] = g_mc->isSuperElastic[i] ? c->supRateCoeff : c->ineRateCoeff;
  }
}
// the per-phase ones of an AC run (rateCoeffAll_periodic, BoltzmannMC.C:2276-2330),
// [phase][process], superelastic copies their collision's supRate
void ref_get_eedf_rates_periodic(double* rate) {
  BoltzmannMC* m = g_mc;
  const int P = m->nProcesses;
  for (size_t ph = 0; ph < m->rateCoeffAll_periodic.size(); ++ph) {
    const auto& row = m->rateCoeffAll_periodic[ph];
    size_t k = 0;
    for (int i = 0; i < P; ++i) {
      if (m->isSuperElastic[i]) continue;
      const auto& rc = row[k++];
      rate[ph * P + i] = rc.ineRate;
      if (i + 1 < P && m->isSuperElastic[i + 1]) rate[ph * P + i + 1] = rc.supRate;
    }
  }
}
int ref_n_phases_periodic() { return (int)g_mc->rateCoeffAll_periodic.size(); }
double ref_swarm_param(const char* key) {
  auto it = g_mc->swarmParam.find(key);
  return it == g_mc->swarmParam.end() ? NAN : it->second;
}
// omega, omega_c, gas density, energy-grid step and cell number
void ref_get_twoterm_grid(double* s) {
  s[0] = g_mc->excitationFrequencyRadians;
  s[1] = g_mc->cyclotronFrequency;
  s[2] = g_mc->totalGasDensity;
  s[3] = g_mc->energyGrid->step;
  s[4] = (double)g_mc->energyGrid->cellNumber;
}
// the total momentum-transfer cross section on the grid nodes
void ref_get_total_mt(double* mt) {
  for (int k = 0; k < (int)g_mc->totalMomTransfCrossSection.size(); ++k) mt[k] = g_mc->totalMomTransfCrossSection[k];
}

// Statistical helpers used by the engine's host side.
double ref_statistical_error(const double* a, int n, double nbins) {
  Eigen::ArrayXd arr(n);
  for (int i = 0; i < n; ++i) arr[i] = a[i];
  return MathFunctions::statisticalError(arr, nbins);
}
void ref_histogram(const double* x, int n, const double* nodes, int nn, double* counts) {
  Eigen::ArrayXd a(n), g(nn);
  for (int i = 0; i < n; ++i) a[i] = x[i];
  for (int i = 0; i < nn; ++i) g[i] = nodes[i];
  Eigen::ArrayXd c = MathFunctions::histogramCount(a, g);
  for (int i = 0; i < nn - 1; ++i) counts[i] = c[i];
}
}
