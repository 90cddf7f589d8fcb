// lokimc_gpu_main.cpp - an entry point for LoKI-MC that can run the electron
// kinetics on the GPU backend.
//
// It behaves like the reference's main (Code/LoKI-MC/Sources/lokimc.C:44-91):
// `lokimc_gpu setupFile [nThreads]`, setup read from Input/, outputs written by
// the reference's own Output class. When the setup sets
// electronKinetics.numericsMC.backend to "gpu", the boltzmannMC engine is
// BoltzmannMCGPU; otherwise the reference's engines run unchanged. Build it
// with the reference's sources except lokimc.C (oracle/ref/Makefile, target
// dropin).
#include <omp.h>

#include <cstdio>
#include <iostream>
#include <string>

#include "BoltzmannMCGPU.h"
#include "LoKI-MC/Headers/BoltzmannMC.h"
#include "LoKI-MC/Headers/FieldInfo.h"
#include "LoKI-MC/Headers/Message.h"
#include "LoKI-MC/Headers/Parse.h"
#include "LoKI-MC/Headers/PrescribedEedf.h"
#include "LoKI-MC/Headers/Setup.h"

template <class Engine>
static void runJobs(const std::string& setupFileName) {
  Setup<Engine> setup(setupFileName);
  setup.initializeSimulation();
  for (; setup.currentJobID < setup.numberOfJobs; setup.nextJob()) {
    if (setup.enableElectronKinetics) setup.electronKinetics->solve();
  }
  setup.finishSimulation();
}

int main(int argc, char* argv[]) {
  std::remove("errorLog.txt");
  if (argc < 2) {
    std::cout << "usage: lokimc_gpu SETUP_FILE [NUM_THREADS]\n";
    return 1;
  }
  const std::string setupFileName(argv[1]);
  const int threads = argc > 2 ? std::atoi(argv[2]) : 1;
  omp_set_num_threads(threads);
  Eigen::setNbThreads(threads);

  Parse::setupFile(setupFileName);
  const std::string eedfType = FieldInfo::getFieldValue("electronKinetics.eedfType");
  const bool gpu = FieldInfo::getField("electronKinetics.numericsMC.backend") &&
                   FieldInfo::getFieldValue("electronKinetics.numericsMC.backend") == "gpu";
  if (eedfType == "boltzmannMC") {
    if (gpu) runJobs<BoltzmannMCGPU>(setupFileName);
    else runJobs<BoltzmannMC>(setupFileName);
  } else if (eedfType == "prescribedEedf") {
    runJobs<PrescribedEedf>(setupFileName);
  } else {
    Message::error("Please choose a valid 'electronKinetics->eedfType' in the setup file: 'boltzmannMC' or 'prescribedEedf'.");
  }
  return 0;
}
