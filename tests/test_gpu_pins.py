"""GPU solves against results that need no reference run.

* Maxwell model (constant momentum-transfer frequency nu = 1e9 s^-1, elastic
  and isotropic, cold gas, m/M = 1.37e-4 as the atomic gas of the plain
  configuration, N = 3.22e22 m^-3). For a constant collision frequency the
  moment equations close exactly:
    momentum  e E = m nu (1 - <s c>) v_d   (flux drift velocity),
    energy    e E v_d = nu a <eps>         (mean energy),
  where a = 2 m M / (m + M)^2 is the mean fractional energy loss of a cold
  elastic collision (BoltzmannMC.C:1160-1187: the speed after is
  v sqrt(1 - a (1 - cos chi))), s = sqrt(1 - a (1 - c)) and <s c> the average
  over isotropic c = cos chi (a/6 to first order). At 100 Td the mean energy
  would be ~6.7 keV, beyond any table (BoltzmannMC.C:1426-1430 stops such a
  run), so the check runs at E/N = 2 Td (v_d ~ 1.13e4 m/s, <eps> ~ 2.66 eV).
  The cross section nu / (N sqrt(2 e eps / m)) is tabulated on 400 log points
  over 1e-4..1e3 eV; its linear interpolation moves nu by ~1e-3 at most.
  Flux and bulk drift (no ionization or attachment: equal) and mean energy
  must agree within two standard errors or 0.5 %.
* Reid's ramp model at 1, 12 and 24 Td (the reference's benchmark case 1,
  ReidRamp_setup_DC.in: 133.32 Pa, 300 K, 1e5 electrons, 1e4 integration
  points, two integrated steady-state times) against the reference's
  published results (benchmarkCalculations_LoKI-MC_v1.0.0.pdf, Table 1: mean
  energy, bulk drift velocity, N D_T and N D_L with their relative standard
  deviations): within two combined standard errors or 0.5 %.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
QE, ME = 1.6021766208e-19, 9.10938356e-31
KB = 1.38064852e-23


def _solve(gases, N, red_field, **cfg_kw):
    from lokigpu import capi, synth

    ps = synth.flatten(gases)
    cfg = capi.default_config(**cfg_kw)
    ctx = capi.Context(cfg)
    ctx.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
    ctx.set_conditions(N, 300.0, red_field)
    r = ctx.solve()
    ctx.close()
    assert r.capped == 0
    return r


def _maxwell_expected(E, nu, mass_ratio):
    m = ME
    M = m / mass_ratio
    a = 2.0 * m * M / (m + M) ** 2
    c = np.linspace(-1.0, 1.0, 200001)
    trapezoid = getattr(np, "trapezoid", None) or np.trapz
    sc = trapezoid(c * np.sqrt(1.0 - a * (1.0 - c)), c) / 2.0
    v_d = QE * E / (m * nu * (1.0 - sc))
    mean_energy = E * v_d / (nu * a)  # eV: e E v_d / (nu a) in J, divided by e
    return v_d, mean_energy


def test_maxwell_model_drift_and_mean_energy():
    from lokigpu import synth

    N, nu, td, ratio = 3.22e22, 1e9, 2.0, 1.37e-4
    E = td * 1e-21 * N
    v_d, mean_energy = _maxwell_expected(E, nu, ratio)
    # energy relaxation takes ~1 / (nu a) = 3.6 us, i.e. some 3600 intervals of
    # ~1 ns: a long steady-state search and integration
    r = _solve([synth.maxwell_gas(nu, N, mass_ratio=ratio)], N, td, n_electrons=1e5, init_temp_ratio=1.0 / (
        KB / QE * 300.0), req_integration_points=40000, max_coll_before_ss=5e4, seed=99)
    # E along -z (angle 180): the electrons drift along +z
    checks = [("flux v_z", r.flux_v[2], r.flux_v_err[2], v_d), ("bulk v_z", r.bulk_v[2], r.bulk_v_err[2], v_d),
              ("mean energy", r.mean_energy, r.mean_energy_err, mean_energy)]
    bad = [f"{k}: gpu {g:.6g} +- {e:.2g}, analytic {x:.6g}" for k, g, e, x in checks
           if abs(g - x) > max(2.0 * e, 5e-3 * abs(x))]
    print("Maxwell model:", [f"{k} {g:.6g} +- {e:.2g} (analytic {x:.6g})" for k, g, e, x in checks])
    assert not bad, "\n".join(bad)


# Table 1 of the reference's benchmark document: E/N (Td) -> mean energy (eV),
# bulk drift velocity (m/s), N D_T and N D_L (1/(m s)), each with its relative
# standard deviation (%)
REID_TABLE1 = {
    1.0: ((0.1014, 0.06), (1.264e4, 0.43), (0.9637e24, 0.70), (0.7542e24, 0.68)),
    12.0: ((0.2691, 0.10), (6.838e4, 0.09), (1.137e24, 0.44), (0.5679e24, 0.35)),
    24.0: ((0.4081, 0.10), (8.881e4, 0.07), (1.138e24, 0.53), (0.4595e24, 0.56)),
}


@pytest.mark.parametrize("td", sorted(REID_TABLE1))
def test_reid_ramp_against_published_results(td):
    from lokigpu import synth

    N = 133.32 / (KB * 300.0)
    r = _solve([synth.reid_ramp_gas()], N, td, n_electrons=1e5, req_integration_points=1e4, req_ss_times=2,
               seed=2024 + int(td))
    dt = N * 0.5 * (r.bulk_d[0] + r.bulk_d[4])
    dt_err = N * 0.5 * math.hypot(r.bulk_d_err[0], r.bulk_d_err[4])
    got = [(r.mean_energy, r.mean_energy_err), (r.bulk_v[2], r.bulk_v_err[2]), (dt, dt_err),
           (N * r.bulk_d[8], N * r.bulk_d_err[8])]
    names = ("mean energy", "bulk drift velocity", "N D_T", "N D_L")
    bad = []
    for name, (g, ge), (p, pe_pct) in zip(names, got, REID_TABLE1[td]):
        sig = math.hypot(ge, abs(p) * pe_pct / 100.0)
        ok = abs(g - p) <= max(2.0 * sig, 5e-3 * abs(p))
        print(f"Reid {td:g} Td {name}: gpu {g:.5g} +- {ge:.2g}, published {p:.5g} ({pe_pct}%)")
        if not ok:
            bad.append(f"{td} Td {name}: gpu {g:.6g} +- {ge:.2g}, published {p:.6g} ({pe_pct} %)")
    assert not bad, "\n".join(bad)
