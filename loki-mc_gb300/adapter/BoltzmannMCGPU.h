// BoltzmannMCGPU.h - drop-in GPU electron-kinetics engine for LoKI-MC.
//
// The reference's host code takes the engine as a template parameter
// (Setup<T>, Output<T>, GUI<T>; Code/LoKI-MC/Sources/lokimc.C:14-41). This
// class derives from the reference's BoltzmannMC
// (Code/LoKI-MC/Headers/BoltzmannMC.h:23-431), so it has every public member
// those templates read, and replaces evaluateEEDF (BoltzmannMC.C:299-426) -
// the Monte Carlo itself - with one call into libloki_gpu.so through the C
// ABI of include/loki_gpu.h. The end-of-job routines evaluatePower,
// evaluateRateCoeff and evaluateSwarmParameters (BoltzmannMC.C:1950-2384) run
// unchanged on the members it fills.
//
// Build: compile with the reference's sources (and its Boost/GSL), add
// -I<repo>/include and link libloki_gpu.so. Select it in lokimc.C by the
// setup key electronKinetics.numericsMC.backend: gpu, as lokimc_gpu_main.cpp
// does. Optional setup keys (ignored by the reference):
//   electronKinetics.numericsMC.gpuDevice: <int>   (default 0)
//   electronKinetics.numericsMC.gpuSeed: <int>     (default 12345)
#ifndef LOKI_GPU_BOLTZMANN_MC_GPU_H
#define LOKI_GPU_BOLTZMANN_MC_GPU_H

#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "LoKI-MC/Headers/BoltzmannMC.h"
#include "LoKI-MC/Headers/FieldInfo.h"
#include "LoKI-MC/Headers/Message.h"
#include "loki_gpu.h"

class BoltzmannMCGPU : public BoltzmannMC {
 public:
  template <class SetupType>
  explicit BoltzmannMCGPU(SetupType* setup) : BoltzmannMC(setup) {
    lgpu_config cfg;
    lgpu_config_default(&cfg);
    if (FieldInfo::getField("electronKinetics.numericsMC.gpuDevice"))
      cfg.device = (int)FieldInfo::getFieldNumericValue("electronKinetics.numericsMC.gpuDevice");
    if (FieldInfo::getField("electronKinetics.numericsMC.gpuSeed"))
      cfg.seed = (uint64_t)FieldInfo::getFieldNumericValue("electronKinetics.numericsMC.gpuSeed");
    // the numericsMC keys as the reference constructor parsed them (BoltzmannMC.h:262-376)
    cfg.n_electrons = nElectrons;
    cfg.n_interp = interpolCrossSectionSize;
    cfg.gas_temperature_effect = gasTemperatureEffect;
    cfg.sharing = energySharingIonizType;
    cfg.init_temp_ratio = initialElecTempOverGasTemp;
    cfg.min_coll_before_ss = minCollisionsBeforeSteadyState / nElectrons;
    cfg.max_coll_before_ss = maxCollisionsBeforeSteadyState / nElectrons;
    cfg.max_coll_after_ss = maxCollisionsAfterSteadyState / nElectrons;
    cfg.req_integration_points = requiredIntegrationPoints;
    cfg.req_ss_times = requiredIntegratedSSTimes;
    cfg.req_abs_time = requiredIntegratedAbsoluteTime;
    cfg.errors_checked = errorsToBeChecked ? 1 : 0;
    cfg.req_err_mean_energy = requiredMeanEnergyRelError;
    cfg.req_err_flux_v = requiredFluxDriftVelocityRelError;
    cfg.req_err_flux_d = requiredFluxDiffusionCoeffsRelError;
    cfg.req_err_bulk_v = requiredBulkDriftVelocityRelError;
    cfg.req_err_bulk_d = requiredBulkDiffusionCoeffsRelError;
    cfg.req_err_power = requiredPowerBalanceRelError;
    cfg.n_energy_cells = (int)nEnergyCells;
    cfg.n_cos_cells = (int)nCosAngleCells;
    cfg.n_radial_cells = (int)nRadialVelocityCells;
    cfg.n_axial_cells = (int)nAxialVelocityCells;
    cfg.n_phases = (int)nIntegrationPhases;
    cfg.sync_x = synchronizationTimeXMaxCollisionFrequency;
    cfg.sync_oversampling = synchronizationOverSampling;
    check(lgpu_create(&cfg, &ctx_), "lgpu_create");
  }

  ~BoltzmannMCGPU() { lgpu_destroy(ctx_); }

  // BoltzmannMC::solve (BoltzmannMC.C:273-297) with the GPU evaluateEEDF
  void solve() {
    const auto start = std::chrono::high_resolution_clock::now();
    evaluateEEDFOnGPU();
    evaluatePower();
    evaluateRateCoeff();
    evaluateSwarmParameters();
    const auto end = std::chrono::high_resolution_clock::now();
    elapsedTime = std::chrono::duration_cast<std::chrono::milliseconds>(end - start).count() * 1E-3;
    obtainedNewEedfSignal();
  }

 private:
  lgpu_ctx* ctx_ = nullptr;

  void check(int rc, const char* what) {
    if (rc == LGPU_OK) return;
    char buf[512] = {0};
    lgpu_last_error(ctx_, buf, sizeof(buf));
    Message::error(std::string(what) + ": " + buf);  // logs and exits, as the reference does (Message.C:6-16)
  }

  static int samplerCode(const std::string& t) {
    if (t == "forward") return 1;
    if (t == "bornDipole") return 2;
    if (t == "surendra") return 3;
    if (t == "coulombScreen") return 4;
    if (t == "momentumConservationIonization") return 5;
    return 0;
  }

  // The per-job host state of evaluateNonConstantVariables (BoltzmannMC.C:428-559)
  // without its start ensemble and its FP64 tables: the device samples the
  // ensemble and builds the tables itself, so the host does neither.
  void prepareJob() {
    gasTemperature = workCond->gasTemperature;
    gasEnergy = 1.5 * Constant::boltzmann * gasTemperature / Constant::electronCharge;
    totalGasDensity = workCond->gasDensity;
    int k = 0;
    for (auto& gas : gasArray) {
      for (auto& collision : gas->collisionArray) {
        if (collision->type == "Effective") continue;
        relDensities[k] = collision->target->density;
        thermalStdDeviations[k] = std::sqrt(Constant::boltzmann * gasTemperature / targetMasses[k]);
        ++k;
        if (collision->isReverse) {
          relDensities[k] = collision->productArray[0]->density;
          thermalStdDeviations[k] = std::sqrt(Constant::boltzmann * gasTemperature / targetMasses[k]);
          ++k;
        }
      }
    }
    time = 0;
    steadyStateTime = Constant::NON_DEF;
    reducedElecField = workCond->reducedElecField;
    electricFieldValue = workCond->reducedElecFieldSI * totalGasDensity;
    elecFieldAngle = workCond->elecFieldAngle;
    if (elecFieldAngle == 180) {
      electricField[0] = 0;
      electricField[1] = 0;
      electricField[2] = -electricFieldValue;
    } else {
      electricField[0] = electricFieldValue * std::sin(elecFieldAngle / 180.0 * M_PI);
      electricField[1] = 0;
      electricField[2] = electricFieldValue * std::cos(elecFieldAngle / 180.0 * M_PI);
    }
    excitationFrequency = workCond->excitationFrequency;
    excitationFrequencyRadians = excitationFrequency * 2.0 * M_PI;
    if (excitationFrequency != 0) electricField *= std::sqrt(2);
    reducedMagField = workCond->reducedMagField;
    cyclotronFrequency = Constant::electronCharge * workCond->reducedMagFieldSI * totalGasDensity / Constant::electronMass;
    isCylindricallySymmetric = workCond->isCylindricallySymmetric;
    accelerationElecField = -Constant::electronCharge / Constant::electronMass * electricField;
    if (excitationFrequencyRadians != 0) {
      integrationPhaseStep = 2.0 * M_PI / nIntegrationPhases;
      integrationPhases = Eigen::ArrayXd::LinSpaced(nIntegrationPhases, 0.5 * integrationPhaseStep,
                                                    2.0 * M_PI - 0.5 * integrationPhaseStep);
    }
    averagedMeanEnergy = Constant::NON_DEF;
    averagedFluxDiffusionCoeffs = Eigen::Matrix3d::Constant(Constant::NON_DEF);
    averagedFluxDiffusionCoeffsError = Eigen::Matrix3d::Constant(Constant::NON_DEF);
    averagedBulkDiffusionCoeffs = Eigen::Matrix3d::Constant(Constant::NON_DEF);
    averagedBulkDiffusionCoeffsError = Eigen::Matrix3d::Constant(Constant::NON_DEF);
    energyGainField = 0;
    energyGrowth = 0;
    totalCollisionCounter = 0;
    nullCollisionCounter = 0;
    for (int i = 0; i < nProcesses; ++i) {
      energyGainProcesses[i] = 0;
      energyLossProcesses[i] = 0;
      collisionCounters[i] = 0;
    }
    goodStatisticalErrors = false;
    failedCollisionDueToGrid = 0;
  }

  void evaluateEEDFOnGPU() {
    // per-job variables, relative densities and fields (BoltzmannMC.C:428-559)
    prepareJob();

    // the flattened processes of BoltzmannMC.C:29-271
    std::vector<lgpu_process> procs(nProcesses);
    for (int i = 0; i < nProcesses; ++i) {
      lgpu_process& q = procs[i];
      Collision* c = realCollisionPointers[i];
      q.type = processTypes[i];
      q.is_super = isSuperElastic[i] ? 1 : 0;
      q.is_elastic = (c->type == "Elastic" && !isSuperElastic[i]) ? 1 : 0;
      q.sampler = samplerCode(c->angularScatteringType);
      q.sampler_p0 = angularScatteringParams[i].size() > 0 ? angularScatteringParams[i][0] : 0.0;
      q.sampler_p1 = angularScatteringParams[i].size() > 1 ? angularScatteringParams[i][1] : 0.0;
      q.superw = superElasticStatWeightFactors[i];
      q.emin = energyMinLimits[i];
      q.emax = energyMaxLimits[i];
      q.rel_dens = relDensities[i];
      q.mass = targetMasses[i];
      q.eloss = energyLosses[i];
      q.wparam = wParameters[i];
      q.raw_len = isSuperElastic[i] ? 0 : (int)crossSectionEnergies[i].size();
      q.raw_e = crossSectionEnergies[i].data();
      q.raw_v = crossSectionValues[i].data();
    }
    std::vector<lgpu_gas> gases(nGases);
    for (int g = 0; g < nGases; ++g) {
      gases[g].first = (int)firstProcessIndexPerGas[g];
      gases[g].last = (int)lastProcessIndexPerGas[g];
      gases[g].fraction = gasFractions[g];
    }
    check(lgpu_set_processes(ctx_, procs.data(), nProcesses, gases.data(), nGases, energyMaxElastic),
          "lgpu_set_processes");
    lgpu_conditions cond;
    cond.gas_density = totalGasDensity;
    cond.gas_temperature = gasTemperature;
    cond.reduced_field_td = reducedElecField;
    cond.field_angle_deg = elecFieldAngle;
    cond.excitation_freq_hz = excitationFrequency;
    cond.reduced_mag_field_hx = reducedMagField;
    check(lgpu_set_conditions(ctx_, &cond), "lgpu_set_conditions");

    lgpu_result r;
    check(lgpu_solve(ctx_, &r), "lgpu_solve");

    // results into the members Output<T> and the end-of-job routines read
    time = r.final_time;
    steadyStateTime = r.ss_time;
    trialCollisionFrequency = r.trial_freq;
    nIntegrationPoints = (int)r.integration_points;
    nSamplingPoints = (int)r.sampling_points;
    firstIntegrationIndex = (int)r.first_integration_index;
    totalIntegratedTime = time - steadyStateTime;
    totalCollisionCounter = (unsigned long long)r.real_collisions;
    nullCollisionCounter = (unsigned long long)r.null_collisions;
    collisionCounterAtSS = (unsigned long long)r.coll_at_ss;
    nullCollisionCounterAtSS = (unsigned long long)r.null_at_ss;
    collisionCounterAfterSS = totalCollisionCounter - collisionCounterAtSS;
    averagedMeanEnergy = r.mean_energy;
    averagedMeanEnergyError = r.mean_energy_err;
    for (int k = 0; k < 3; ++k) {
      averagedFluxDriftVelocity[k] = r.flux_v[k];
      averagedFluxDriftVelocityError[k] = r.flux_v_err[k];
      averagedBulkDriftVelocity[k] = r.bulk_v[k];
      averagedBulkDriftVelocityError[k] = r.bulk_v_err[k];
      for (int l = 0; l < 3; ++l) {
        averagedFluxDiffusionCoeffs(k, l) = r.flux_d[3 * k + l];
        averagedFluxDiffusionCoeffsError(k, l) = r.flux_d_err[3 * k + l];
        averagedBulkDiffusionCoeffs(k, l) = r.bulk_d[3 * k + l];
        averagedBulkDiffusionCoeffsError(k, l) = r.bulk_d_err[3 * k + l];
      }
    }
    averagedPowerGainField = r.power_field;
    averagedPowerGrowth = r.power_growth;
    powerBalanceRelError = r.power_balance_rel_err;
    maxEedfEnergy = r.max_eedf_energy;

    std::vector<unsigned long long> counts(nProcesses);
    check(lgpu_get_process_results(ctx_, counts.data(), averagedRateCoeffs, averagedPowerGainProcesses,
                                   averagedPowerLossProcesses, nProcesses),
          "lgpu_get_process_results");
    for (int i = 0; i < nProcesses; ++i) collisionCounters[i] = counts[i];

    // time series (BoltzmannMC.h:124-167)
    const long long rows = lgpu_get_series(ctx_, 0, nullptr, 1LL << 40);
    samplingTimes.resize(rows);
    meanEnergies.resize(rows);
    meanPositions.resize(rows, 3);
    meanVelocities.resize(rows, 3);
    fluxDiffusionCoeffs.resize(rows, 9);
    positionCovariances.resize(rows, 9);
    bulkVelocities.resize(rows, 3);
    bulkDiffusionCoeffs.resize(rows, 9);
    std::vector<double> buf((size_t)rows * 9);
    auto fetch = [&](int which, int width, Eigen::ArrayXXd* dst2, Eigen::ArrayXd* dst1) {
      lgpu_get_series(ctx_, which, buf.data(), rows);
      for (long long i = 0; i < rows; ++i)
        for (int k = 0; k < width; ++k) {
          if (dst2) (*dst2)(i, k) = buf[(size_t)i * width + k];
          else (*dst1)[i] = buf[(size_t)i];
        }
    };
    fetch(0, 1, nullptr, &samplingTimes);
    fetch(1, 1, nullptr, &meanEnergies);
    fetch(2, 3, &meanPositions, nullptr);
    fetch(3, 3, &meanVelocities, nullptr);
    fetch(4, 9, &fluxDiffusionCoeffs, nullptr);
    fetch(5, 9, &positionCovariances, nullptr);
    fetch(6, 3, &bulkVelocities, nullptr);
    fetch(7, 9, &bulkDiffusionCoeffs, nullptr);

    // distributions (BoltzmannMC.C:1574-1605, 1728-1741)
    const int nEC = (int)nEnergyCells, nCos = (int)nCosAngleCells, nR = (int)nRadialVelocityCells,
              nA = (int)nAxialVelocityCells, nPh = (int)nIntegrationPhases;
    std::vector<double> cells(nEC), ee(nEC), f1(nEC), f2(nEC), ead((size_t)nEC * nCos), evd((size_t)nR * nA),
        rc(nR), ac(nA), per((size_t)nPh * nEC);
    check(lgpu_get_distributions(ctx_, cells.data(), ee.data(), f1.data(), f2.data(), ead.data(), evd.data(),
                                 rc.data(), ac.data(), per.data()),
          "lgpu_get_distributions");
    eedfEnergyStep = maxEedfEnergy / nEnergyCells;
    eedfEnergyCells = Eigen::Map<Eigen::ArrayXd>(cells.data(), nEC);
    eedfEnergyNodes = Eigen::ArrayXd::LinSpaced(nEC + 1, 0.0, maxEedfEnergy);
    eedf = Eigen::Map<Eigen::ArrayXd>(ee.data(), nEC);
    efadf = Eigen::Map<Eigen::ArrayXd>(f1.data(), nEC);
    esadf = Eigen::Map<Eigen::ArrayXd>(f2.data(), nEC);
    eadf.resize(nEC, nCos);
    for (int i = 0; i < nEC; ++i)
      for (int k = 0; k < nCos; ++k) eadf(i, k) = ead[(size_t)i * nCos + k];
    evdf.resize(nR, nA);
    for (int i = 0; i < nR; ++i)
      for (int k = 0; k < nA; ++k) evdf(i, k) = evd[(size_t)i * nA + k];
    radialVelocityCells = Eigen::Map<Eigen::ArrayXd>(rc.data(), nR);
    axialVelocityCells = Eigen::Map<Eigen::ArrayXd>(ac.data(), nA);
    if (excitationFrequencyRadians != 0) {
      eedf_periodic.resize(nPh, nEC);
      for (int q = 0; q < nPh; ++q)
        for (int c = 0; c < nEC; ++c) eedf_periodic(q, c) = per[(size_t)q * nEC + c];
      std::vector<double> n(nPh), me(nPh), fv((size_t)nPh * 3), bv((size_t)nPh * 3), fd((size_t)nPh * 9),
          bd((size_t)nPh * 9);
      check(lgpu_get_periodic(ctx_, n.data(), me.data(), fv.data(), bv.data(), fd.data(), bd.data()),
            "lgpu_get_periodic");
      nIntegrationPointsPerPhase = Eigen::Map<Eigen::ArrayXd>(n.data(), nPh);
      meanEnergies_periodic = Eigen::Map<Eigen::ArrayXd>(me.data(), nPh);
      fluxVelocities_periodic.resize(nPh, 3);
      bulkVelocities_periodic.resize(nPh, 3);
      fluxDiffusionCoeffs_periodic.resize(nPh, 9);
      bulkDiffusionCoeffs_periodic.resize(nPh, 9);
      for (int q = 0; q < nPh; ++q) {
        for (int k = 0; k < 3; ++k) {
          fluxVelocities_periodic(q, k) = fv[3 * q + k];
          bulkVelocities_periodic(q, k) = bv[3 * q + k];
        }
        for (int k = 0; k < 9; ++k) {
          fluxDiffusionCoeffs_periodic(q, k) = fd[9 * q + k];
          bulkDiffusionCoeffs_periodic(q, k) = bd[9 * q + k];
        }
      }
    }
    // the energy grid follows the EEDF range (BoltzmannMC.C:425)
    energyGrid->updateMaxValue(maxEedfEnergy);
  }
};

#endif
