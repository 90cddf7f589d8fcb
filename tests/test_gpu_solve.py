"""GPU statistical parity: full solves against seeded FP64 solves of the
reference built from its own sources (tests/golden/stats_*.json, made by
tests/golden/make_golden.py --stats with 1e4 electrons).

The GPU solve uses the reference's own parsed inputs (the per-process arrays
of the matching kin_*.npz), the same numerics keys and 1e5 electrons. Every
swarm parameter the reference pins (mean energy, flux and bulk drift velocity,
flux and bulk diffusion along the axes) must agree within 0.5% or within
three combined standard errors (50-block batch means of both runs,
BoltzmannMC.C:1484-1726); components the reference cannot resolve (below five
of its standard errors) are skipped. The batch-means errors of a 1e4-electron
run understate its scatter (seeded reference runs of the atomic case differ by
about 2 of their own errors), hence 0.5% as the floor. Rate coefficients
of processes with at least 2000 reference counts agree within three combined
Poisson errors doubled for autocorrelation, plus 1%. The time-averaged EEDF
agrees in 20 coarse energy bins (bins holding more than 1 % within 5 % +
0.003) and in the mean energy it implies (1 %).
"""
import glob
import json
import os

import numpy as np
import pytest

import golden_util as gu

pytestmark = pytest.mark.gpu
KB_EV = 1.38064852e-23 / 1.6021766208e-19
CASES = sorted(os.path.basename(p)[6:-5] for p in glob.glob(os.path.join(gu.GOLDEN, "stats_*.json")))
META = {"atomic": dict(N=3.22e22, red_field=100.0), "n2": dict(N=3.22e22, red_field=200.0),
        "mix": dict(N=3.22e22, red_field=100.0)}
GAS_TEMP = {"false": 0, "true": 1, "smartActivation": 2}


def run_gpu(rec, n_electrons=100_000):
    from lokigpu import capi

    g = gu.load(rec["case"])
    arrays = gu.proc_arrays(g)
    ps = gu.processes(arrays)
    meta = dict(META[rec["case"]], **rec["overrides"])
    num = rec["numerics"]
    cfg = capi.default_config(n_electrons=float(n_electrons), n_interp=int(num.get("nInterpPoints", 2000)),
                              seed=int(os.environ.get("LGPU_TEST_SEED", "4242")), init_temp_ratio=1.0 / (KB_EV * 300.0),
                              gas_temperature_effect=GAS_TEMP[meta.get("gas_temp", "false")],
                              req_integration_points=float(num["nIntegrationPoints"]),
                              max_coll_before_ss=float(num["maxCollisionsBeforeSteadyState"]),
                              n_phases=int(num.get("nIntegrationPhases", 100)), max_seconds=600.0)
    ctx = capi.Context(cfg)
    ctx.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
    ctx.set_conditions(meta["N"], 300.0, meta["red_field"], meta.get("angle", 180.0), meta.get("freq", 0.0),
                       meta.get("red_mag", 0.0))
    r = ctx.solve()
    counts, rate, _, _ = ctx.process_results()
    dist = ctx.distributions()
    ctx.close()
    return r, counts, rate, ps, dist


def coarse_probabilities(cells, eedf, edges):
    """Probability of each coarse energy bin from a normalised EEDF on uniform
    cells: sum of f(e) sqrt(e) de over the cells whose centre lies in the bin
    (BoltzmannMC.C:1574-1605 normalises f so that the full sum is 1)."""
    cells = np.asarray(cells)
    de = cells[1] - cells[0]
    w = np.asarray(eedf) * np.sqrt(cells) * de
    idx = np.digitize(cells, edges) - 1
    return np.array([w[idx == k].sum() for k in range(len(edges) - 1)])


@pytest.mark.parametrize("name", CASES)
def test_swarm_parameters_match_reference(name):
    with open(os.path.join(gu.GOLDEN, f"stats_{name}.json")) as f:
        rec = json.load(f)
    ref = np.array(rec["result"])
    r, counts, rate, ps, dist = run_gpu(rec)
    assert r.capped == 0 and r.integration_points >= float(rec["numerics"]["nIntegrationPoints"]) - 1
    pairs = [("mean energy", r.mean_energy, r.mean_energy_err, ref[0], ref[1])]
    for k in range(3):
        pairs += [(f"flux v[{k}]", r.flux_v[k], r.flux_v_err[k], ref[2 + k], ref[5 + k]),
                  (f"flux D[{k}{k}]", r.flux_d[4 * k], r.flux_d_err[4 * k], ref[8 + k], ref[11 + k]),
                  (f"bulk v[{k}]", r.bulk_v[k], r.bulk_v_err[k], ref[14 + k], ref[17 + k]),
                  (f"bulk D[{k}{k}]", r.bulk_d[4 * k], r.bulk_d_err[4 * k], ref[20 + k], ref[23 + k])]
    failures, checked = [], 0
    for label, gv, ge, rv, re in pairs:
        if abs(rv) < 5.0 * re:
            continue
        checked += 1
        tol = max(3.0 * np.hypot(ge, re), 5e-3 * abs(rv))
        if abs(gv - rv) > tol:
            failures.append(f"{label}: gpu {gv:.6g} +- {ge:.3g}, reference {rv:.6g} +- {re:.3g}")
    assert checked >= 4, name
    # rate coefficients (BoltzmannMC.C:1627-1638)
    ref_rate = np.array(rec["rate"])
    t_int = ref[31] - ref[30]
    n_ref = float(rec["n_electrons"])
    for p in range(ps.n):
        if ref_rate[p] <= 0 or ps.rel_dens[p] <= 0:
            continue
        c_ref = ref_rate[p] * t_int * n_ref * ps.rel_dens[p] * META[rec["case"]]["N"]
        if c_ref < 2000 or counts[p] < 2000:
            continue
        rel = 2.0 * 3.0 * np.sqrt(1.0 / c_ref + 1.0 / counts[p]) + 0.01
        if abs(rate[p] / ref_rate[p] - 1.0) > rel:
            failures.append(f"rate[{p}]: gpu {rate[p]:.6g}, reference {ref_rate[p]:.6g} (counts {counts[p]}, {c_ref:.0f})")
    # time-averaged EEDF (BoltzmannMC.C:1492-1580): 20 coarse bins over the
    # common energy range, bins holding > 1 % within 5 % + 0.003; the mean
    # energy of the distribution within 1 %
    cg, fg = dist["eedf_cells"], dist["eedf"]
    cr, fr = np.array(rec["eedf_cells"]), np.array(rec["eedf"])
    edges = np.linspace(0.0, min(cg[-1], cr[-1]), 21)
    pg, pr = coarse_probabilities(cg, fg, edges), coarse_probabilities(cr, fr, edges)
    for k in range(20):
        if pr[k] > 0.01 and abs(pg[k] - pr[k]) > 0.05 * pr[k] + 0.003:
            failures.append(f"EEDF bin {edges[k]:.3g}-{edges[k + 1]:.3g} eV: gpu {pg[k]:.4f}, reference {pr[k]:.4f}")
    mg = np.sum(fg * cg ** 1.5) * (cg[1] - cg[0])
    mr = np.sum(fr * cr ** 1.5) * (cr[1] - cr[0])
    if abs(mg / mr - 1.0) > 0.01:
        failures.append(f"EEDF mean energy: gpu {mg:.5g}, reference {mr:.5g}")
    assert not failures, "\n".join(failures)
