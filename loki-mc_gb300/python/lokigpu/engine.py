"""BoltzmannMC: the reference engine's interface over the GB300 backend.

Mirrors the public surface of the reference class (Code/LoKI-MC/Headers/BoltzmannMC.h:23-431)
that its host code reads after ``solve()`` (BoltzmannMC.C:273-297): the
time-averaged swarm parameters with their errors, rate coefficients, power
terms, distributions and the collision counters. Construction takes the gas
mixture (lokigpu.synth.Gas objects, flattened as BoltzmannMC.C:29-271 does),
the working conditions and the ``numericsMC`` keys by their setup-file names.
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence

import numpy as np

from . import capi
from . import constants as C
from .synth import Gas, ProcessSet, flatten

_GAS_TEMP = {"false": C.GAS_TEMP_FALSE, "true": C.GAS_TEMP_TRUE, "smartActivation": C.GAS_TEMP_SMART}
_SHARING = {"equalSharing": C.EQUAL_SHARING, "oneTakesAll": C.ONE_TAKES_ALL, "usingSDCS": C.USING_SDCS,
            "randomUniform": C.RANDOM_UNIFORM}

# numericsMC key -> (config field, scale by nElectrons)
_NUMERICS = {
    "initialElecTempOverGasTemp": ("init_temp_ratio", False),
    "minCollisionsBeforeSteadyState": ("min_coll_before_ss", False),
    "maxCollisionsBeforeSteadyState": ("max_coll_before_ss", False),
    "maxCollisionsAfterSteadyState": ("max_coll_after_ss", False),
    "nEnergyCells": ("n_energy_cells", False),
    "nCosAngleCells": ("n_cos_cells", False),
    "nRadialVelocityCells": ("n_radial_cells", False),
    "nAxialVelocityCells": ("n_axial_cells", False),
    "nIntegrationPoints": ("req_integration_points", False),
    "nIntegratedSSTimes": ("req_ss_times", False),
    "integratedAbsoluteTime": ("req_abs_time", False),
    "nIntegrationPhases": ("n_phases", False),
    "nInterpPoints": ("n_interp", False),
    "synchronizationTimeXMaxCollisionFrequency": ("sync_x", False),
    "synchronizationOverSampling": ("sync_oversampling", False),
}
_REL_ERR = {"meanEnergy": "req_err_mean_energy", "fluxDriftVelocity": "req_err_flux_v",
            "fluxDiffusionCoeffs": "req_err_flux_d", "bulkDriftVelocity": "req_err_bulk_v",
            "bulkDiffusionCoeffs": "req_err_bulk_d", "powerBalance": "req_err_power"}
_INT_FIELDS = {"n_energy_cells", "n_cos_cells", "n_radial_cells", "n_axial_cells", "n_phases", "n_interp",
               "sync_oversampling"}


def make_config(n_electrons: float, gas_temperature_effect: str = "false", ionization_operator: str = "equalSharing",
                numerics: Optional[Dict[str, float]] = None, rel_error: Optional[Dict[str, float]] = None,
                seed: int = 12345, device: int = 0, max_seconds: float = 0.0, max_sync_steps: int = 0) -> capi.Config:
    cfg = capi.default_config(device=device, seed=seed, n_electrons=float(n_electrons),
                              gas_temperature_effect=_GAS_TEMP[gas_temperature_effect],
                              sharing=_SHARING[ionization_operator], max_seconds=max_seconds,
                              max_sync_steps=max_sync_steps)
    for k, v in (numerics or {}).items():
        field, _ = _NUMERICS[k]
        setattr(cfg, field, int(v) if field in _INT_FIELDS else float(v))
    if rel_error is not None:
        cfg.errors_checked = 1
        for k, v in rel_error.items():
            setattr(cfg, _REL_ERR[k], float(v))
    return cfg


class BoltzmannMC:
    """One electron-kinetics engine on the GPU for a fixed mixture."""

    def __init__(self, gases: Sequence[Gas] = None, *, processes: Optional[ProcessSet] = None,
                 gas_density: float, gas_temperature: float = 300.0, n_electrons: float = 1e4,
                 gas_temperature_effect: str = "false", ionization_operator: str = "equalSharing",
                 numerics: Optional[Dict[str, float]] = None, rel_error: Optional[Dict[str, float]] = None,
                 seed: int = 12345, device: int = 0, max_seconds: float = 0.0, max_sync_steps: int = 0):
        self.processes = processes if processes is not None else flatten(gases)
        self.cfg = make_config(n_electrons, gas_temperature_effect, ionization_operator, numerics, rel_error, seed,
                               device, max_seconds, max_sync_steps)
        self.ctx = capi.Context(self.cfg)
        ps = self.processes
        self.ctx.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        self.totalGasDensity = float(gas_density)
        self.gasTemperature = float(gas_temperature)
        self.nElectrons = float(n_electrons)
        self.nProcesses = ps.n

    # WorkingConditions.h:55-132
    def set_conditions(self, reduced_field: float, angle: float = 180.0, excitation_frequency: float = 0.0,
                       reduced_mag_field: float = 0.0):
        self.reducedElecField = reduced_field
        self.elecFieldAngle = angle
        self.excitationFrequency = excitation_frequency
        self.reducedMagField = reduced_mag_field
        self.ctx.set_conditions(self.totalGasDensity, self.gasTemperature, reduced_field, angle,
                                excitation_frequency, reduced_mag_field)

    def solve(self):
        """The evaluateEEDF loop plus the end-of-job averages (BoltzmannMC.C:273-426)."""
        r = self.ctx.solve()
        self.result = r
        self.averagedMeanEnergy = r.mean_energy
        self.averagedMeanEnergyError = r.mean_energy_err
        self.averagedFluxDriftVelocity = np.array(r.flux_v[:])
        self.averagedFluxDriftVelocityError = np.array(r.flux_v_err[:])
        self.averagedFluxDiffusionCoeffs = np.array(r.flux_d[:]).reshape(3, 3)
        self.averagedFluxDiffusionCoeffsError = np.array(r.flux_d_err[:]).reshape(3, 3)
        self.averagedBulkDriftVelocity = np.array(r.bulk_v[:])
        self.averagedBulkDriftVelocityError = np.array(r.bulk_v_err[:])
        self.averagedBulkDiffusionCoeffs = np.array(r.bulk_d[:]).reshape(3, 3)
        self.averagedBulkDiffusionCoeffsError = np.array(r.bulk_d_err[:]).reshape(3, 3)
        self.totalCollisionCounter = r.real_collisions
        self.nullCollisionCounter = r.null_collisions
        self.collisionCounterAtSS = r.coll_at_ss
        self.nullCollisionCounterAtSS = r.null_at_ss
        self.steadyStateTime = r.ss_time
        self.time = r.final_time
        self.nIntegrationPoints = r.integration_points
        self.trialCollisionFrequency = r.trial_freq
        self.powerBalanceRelError = r.power_balance_rel_err
        self.averagedPowerGainField = r.power_field
        self.averagedPowerGrowth = r.power_growth
        self.elapsedTime = r.elapsed
        counts, rate, gain, loss = self.ctx.process_results()
        self.collisionCounters = counts
        self.averagedRateCoeffs = rate
        self.averagedPowerGainProcesses = gain
        self.averagedPowerLossProcesses = loss
        d = self.ctx.distributions()
        self.eedfEnergyCells = d["eedf_cells"]
        self.eedf = d["eedf"]
        self.efadf = d["efadf"]
        self.esadf = d["esadf"]
        self.eadf = d["eadf"]
        self.evdf = d["evdf"]
        self.radialVelocityCells = d["radial_cells"]
        self.axialVelocityCells = d["axial_cells"]
        self.eedf_periodic = d["eedf_periodic"]
        return r

    def series(self):
        """Sampled time series (BoltzmannMC.h:124-167)."""
        c = self.ctx
        return dict(samplingTimes=c.series(0, 1), meanEnergies=c.series(1, 1), meanPositions=c.series(2, 3),
                    meanVelocities=c.series(3, 3), fluxDiffusionCoeffs=c.series(4, 9),
                    positionCovariances=c.series(5, 9), bulkVelocities=c.series(6, 3),
                    bulkDiffusionCoeffs=c.series(7, 9))

    def close(self):
        self.ctx.close()
