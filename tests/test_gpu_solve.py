"""GPU statistical parity: full solves against seeded FP64 solves of the
reference built from its own sources (tests/golden/stats_*.json and
stats_*_dist.npz, made by tests/golden/make_golden.py --stats: 1e5
electrons, 1e4 integration intervals, 1e4 table points): the atomic gas, the
N2-like gas (cold and thermal targets), the N2/O2-like mixture under DC, AC
and crossed B, and the field-complex batch's branches (crossed B at 500 and
2000 Hx, AC at omega/N = 1e-14 m^3/s) on the sweep's mixture.

The GPU solve uses the reference's own parsed inputs (the per-process arrays
of the matching kin_*.npz; the product's flattening for the sweep's
mixture), the same numerics keys and 1e6 electrons, so
that the combined error is close to the reference's own. Criteria, for every
swarm parameter the reference resolves (mean energy, flux and bulk drift
velocity, flux and bulk diffusion along the axes; components below five of
its standard errors are not resolved) and every rate coefficient
(BoltzmannMC.C:1627-1638) of a process with at least 1e4 counts in both runs:

* the deviation is printed in combined standard errors (50-block batch means
  of both runs, BoltzmannMC.C:1484-1726, MathFunctions.C:211-231; Poisson
  errors of the collision counts for the rates) and in percent;
* within two combined standard errors or 0.5 % for at least 90 % of the
  quantities of a case: with tens of quantities per case, a few beyond two
  standard errors are expected of two statistically equal runs (4.6 % each),
  so "every quantity within 2 sigma" would fail by chance;
* every quantity within four combined standard errors or 0.5 % (a
  deviation that statistics alone would produce once in 16000);
* per-process power gains and losses (BoltzmannMC.C:1640-1649) above 1 % of
  the field's power within 1 % or four Poisson errors of the process's counts.

Distributions (BoltzmannMC.C:1492-1605), compared through cumulative
probabilities at common edges (the two runs' grids follow their own largest
energies; tests/golden_util.py): the EEDF's and each of ten cos(angle)
groups of the EADF's cumulative probability within 0.005 at 20 energy
edges, the cumulative first and second anisotropies (probability times P1,
P2 of cos) within 0.002 + 1 % of their totals (not the first under AC:
it cancels over a period), the EVDF's 2-D cumulative
probability within 0.005 on a 10 x 10 grid, the EEDF's mean energy within
0.5 %. AC (BoltzmannMC.C:1468-1481, 1728-1741): the phases with samples,
and per phase the mean energy within 1 %, the flux drift velocity within 2 %
of its largest magnitude over the period and the EEDF's cumulative
probability within 0.01.
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
        "mix": dict(N=3.22e22, red_field=100.0), "sweep": dict(N=3.22e22, red_field=100.0)}


def _inputs(case):
    """Per-process arrays of a case: the reference's own (kin_*.npz), or for
    the sweep's mixture the product's flattening of the same synthetic gases
    (pinned to the reference's flattening by test_flatten.py)."""
    if case == "sweep":
        from lokigpu import synth
        ps = synth.flatten([synth.n2_like_gas(fraction=0.8, e_max=1e4), synth.o2_like_gas(fraction=0.2, e_max=1e4)])
        return ps, dict(gas_first=ps.gas_first, gas_last=ps.gas_last, gas_frac=ps.gas_fraction)
    arrays = gu.proc_arrays(gu.load(case))
    return gu.processes(arrays), arrays


GAS_TEMP = {"false": 0, "true": 1, "smartActivation": 2}
N_GPU = 1_000_000


def run_gpu(rec, n_electrons=N_GPU):
    from lokigpu import capi

    ps, arrays = _inputs(rec["case"])
    meta = dict(META[rec["case"]], **rec["overrides"])
    num = rec["numerics"]
    cfg = capi.default_config(n_electrons=float(n_electrons), n_interp=int(num.get("nInterpPoints", 10000)),
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
    counts, rate, gain, loss = ctx.process_results()
    dist = ctx.distributions()
    per = ctx.periodic() if meta.get("freq", 0.0) else None
    ctx.close()
    return r, counts, rate, gain, loss, ps, dist, per


@pytest.fixture(scope="module", params=CASES)
def solved(request):
    name = request.param
    with open(os.path.join(gu.GOLDEN, f"stats_{name}.json")) as f:
        rec = json.load(f)
    dist_path = os.path.join(gu.GOLDEN, f"stats_{name}_dist.npz")
    ref_dist = dict(np.load(dist_path)) if os.path.exists(dist_path) else None
    return name, rec, ref_dist, run_gpu(rec)


def compare_quantities(name, pairs, rate_rows):
    """pairs: (label, gpu, gpu err, ref, ref err); rate_rows: (label, gpu,
    ref, gpu counts, ref counts). Returns (lines, failures)."""
    lines, devs = [], []
    for label, gv, ge, rv, re in pairs:
        sig = float(np.hypot(ge, re))
        devs.append((label, (gv - rv) / sig, gv / rv - 1.0))
        lines.append(f"{name} {label}: gpu {gv:.6g} +- {ge:.2g}, reference {rv:.6g} +- {re:.2g} "
                     f"({devs[-1][1]:+.2f} sigma, {100 * devs[-1][2]:+.3f} %)")
    for label, gv, rv, cg, cr in rate_rows:
        rel_sig = float(np.sqrt(1.0 / cr + 1.0 / cg))
        dev = gv / rv - 1.0
        devs.append((label, dev / rel_sig, dev))
        lines.append(f"{name} {label}: gpu {gv:.6g} ({cg:.0f} counts), reference {rv:.6g} ({cr:.0f}): "
                     f"{dev / rel_sig:+.2f} sigma, {100 * dev:+.3f} %")
    within2 = sum(1 for _, z, d in devs if abs(z) <= 2.0 or abs(d) <= 5e-3)
    failures = [f"{label}: {z:+.2f} sigma, {100 * d:+.3f} %" for label, z, d in devs
                if abs(z) > 4.0 and abs(d) > 5e-3]
    lines.append(f"{name}: {within2} of {len(devs)} quantities within 2 sigma or 0.5 %")
    if devs and within2 < 0.9 * len(devs):
        failures.append(f"only {within2} of {len(devs)} within 2 sigma or 0.5 %")
    return lines, failures


def test_swarm_parameters_and_rates(solved):
    name, rec, _, (r, counts, rate, gain, loss, ps, dist, per) = solved
    ref = np.array(rec["result"])
    assert r.capped == 0 and r.integration_points >= float(rec["numerics"]["nIntegrationPoints"]) - 1
    pairs = [("mean energy", r.mean_energy, r.mean_energy_err, ref[0], ref[1])]
    for k in range(3):
        pairs += [(f"flux v[{k}]", r.flux_v[k], r.flux_v_err[k], ref[2 + k], ref[5 + k]),
                  (f"flux D[{k}{k}]", r.flux_d[4 * k], r.flux_d_err[4 * k], ref[8 + k], ref[11 + k]),
                  (f"bulk v[{k}]", r.bulk_v[k], r.bulk_v_err[k], ref[14 + k], ref[17 + k]),
                  (f"bulk D[{k}{k}]", r.bulk_d[4 * k], r.bulk_d_err[4 * k], ref[20 + k], ref[23 + k])]
    pairs = [p for p in pairs if abs(p[3]) >= 5.0 * p[4]]
    assert len(pairs) >= 4, name
    ref_rate = np.array(rec["rate"])
    t_int = ref[31] - ref[30]
    n_ref = float(rec["n_electrons"])
    rows = []
    for p in range(ps.n):
        if ref_rate[p] <= 0 or ps.rel_dens[p] <= 0:
            continue
        c_ref = ref_rate[p] * t_int * n_ref * ps.rel_dens[p] * META[rec["case"]]["N"]
        if c_ref >= 1e4 and counts[p] >= 1e4:
            rows.append((f"rate[{p}]", rate[p], ref_rate[p], float(counts[p]), c_ref))
    lines, failures = compare_quantities(name, pairs, rows)
    if "power_gain" in rec:
        # a process's power follows its collision count: within 1 % or four
        # Poisson errors of the two runs' counts
        rg, rl = np.array(rec["power_gain"]), np.array(rec["power_loss"])
        field = abs(ref[36])
        for p in range(ps.n):
            c_ref = ref_rate[p] * t_int * n_ref * ps.rel_dens[p] * META[rec["case"]]["N"]
            tol = max(0.01, 4.0 * np.sqrt(1.0 / max(c_ref, 1.0) + 1.0 / max(float(counts[p]), 1.0)))
            for lab, gv, rv in (("gain", gain[p], rg[p]), ("loss", loss[p], rl[p])):
                if abs(rv) > 0.01 * field and abs(gv / rv - 1.0) > tol:
                    failures.append(f"power {lab}[{p}]: gpu {gv:.6g}, reference {rv:.6g} (bound {100 * tol:.2f} %)")
    print("\n".join(lines))
    assert not failures, f"{name}:\n" + "\n".join(failures)


def _edges(ref_dist, cells, n=20):
    top = min(ref_dist["e_edges"][-1], gu.energy_nodes(cells)[-1])
    return np.linspace(0.0, top, n + 1)


def test_distributions(solved):
    name, rec, ref_dist, (r, counts, rate, gain, loss, ps, dist, per) = solved
    if ref_dist is None:
        pytest.skip("no reference distributions for this case")
    failures = []
    cells = dist["eedf_cells"]
    nodes = gu.energy_nodes(cells)
    e = _edges(ref_dist, cells)
    ge = gu.cdf_at(nodes, gu.eedf_mass(cells, dist["eedf"]), e)
    re_ = gu.cdf_at(ref_dist["e_edges"], np.diff(ref_dist["eedf_cdf"]), e)
    d = np.max(np.abs(ge - re_))
    print(f"{name} EEDF: largest cumulative difference {d:.4f}")
    if d > 0.005:
        failures.append(f"EEDF cumulative probability differs by {d:.4f}")
    mg = np.sum(gu.eedf_mass(cells, dist["eedf"]) * cells)
    rc = np.array(rec["eedf_cells"])
    mr = np.sum(gu.eedf_mass(rc, rec["eedf"]) * rc)
    if abs(mg / mr - 1.0) > 5e-3:
        failures.append(f"EEDF mean energy: gpu {mg:.5g}, reference {mr:.5g}")
    if "eadf_cdf" in ref_dist:
        ga = gu.cdf_at(nodes, gu.eadf_mass(cells, dist["eadf"], 10), e)
        ra = gu.cdf_at(ref_dist["e_edges"], np.diff(ref_dist["eadf_cdf"], axis=0), e)
        d = np.max(np.abs(ga - ra))
        print(f"{name} EADF (10 cos groups): largest cumulative difference {d:.4f}")
        if d > 0.005:
            failures.append(f"EADF cumulative probability differs by {d:.4f}")
        # under an AC field the first anisotropy changes sign with the field,
        # so its time average nearly cancels and rests on where each run's
        # window ends within a period: it is compared phase by phase through
        # the flux drift below instead
        ac = per is not None
        for deg, key, fk in ((1, "f1_cdf", "efadf"), (2, "f2_cdf", "esadf")):
            if ac and deg == 1:
                continue
            gl = gu.cdf_at(nodes, gu.legendre_mass(cells, dist[fk], deg), e)
            rl = gu.cdf_at(ref_dist["e_edges"], np.diff(ref_dist[key]), e)
            tol = 0.002 + 0.01 * abs(rl[-1])
            d = np.max(np.abs(gl - rl))
            print(f"{name} anisotropy {deg}: totals gpu {gl[-1]:.5f}, reference {rl[-1]:.5f}; "
                  f"largest cumulative difference {d:.5f} (bound {tol:.5f})")
            if d > tol:
                failures.append(f"{fk} cumulative differs by {d:.5f} (totals {gl[-1]:.5f}, {rl[-1]:.5f})")
        rr, rz = ref_dist["r_edges"], ref_dist["z_edges"]
        gr = np.linspace(0.0, min(rr[-1], dist["radial_cells"][-1]), 11)
        gz = np.linspace(max(rz[0], dist["axial_cells"][0]), min(rz[-1], dist["axial_cells"][-1]), 11)
        gv = gu.evdf_cdf(dist["radial_cells"], dist["axial_cells"], dist["evdf"], gr, gz)
        # the reference's 2-D cumulative on its sub-grid, bilinear at the common grid
        rv = np.stack([np.interp(gz, rz, row) for row in ref_dist["evdf_cdf"]], axis=0)
        rv = np.stack([np.interp(gr, rr, rv[:, j]) for j in range(rv.shape[1])], axis=1)
        d = np.max(np.abs(gv - rv))
        print(f"{name} EVDF: largest 2-D cumulative difference {d:.4f}")
        if d > 0.005:
            failures.append(f"EVDF cumulative probability differs by {d:.4f}")
    if per is not None and "per_n" in ref_dist:
        if not np.array_equal(per["n"] > 0, ref_dist["per_n"] > 0):
            failures.append("phases with samples differ")
        dme = np.max(np.abs(per["mean_energy"] / ref_dist["per_mean_energy"] - 1.0))
        amp = np.max(np.abs(ref_dist["per_flux_v"][:, 2]))
        dv = np.max(np.abs(per["flux_v"][:, 2] - ref_dist["per_flux_v"][:, 2])) / amp
        print(f"{name} periodic: mean energy within {100 * dme:.3f} %, flux v_z within {100 * dv:.3f} % of "
              f"its amplitude {amp:.4g} m/s")
        if dme > 0.01:
            failures.append(f"periodic mean energy differs by {100 * dme:.3f} %")
        if dv > 0.02:
            failures.append(f"periodic flux drift differs by {100 * dv:.3f} % of its amplitude")
        pe = ref_dist["per_e_edges"]
        ee = np.linspace(0.0, min(pe[-1], nodes[-1]), 11)
        dmax = 0.0
        for q in range(len(ref_dist["per_n"])):
            gq = gu.cdf_at(nodes, gu.eedf_mass(cells, dist["eedf_periodic"][q]), ee)
            rq = gu.cdf_at(pe, np.diff(ref_dist["per_eedf_cdf"][q]), ee)
            dmax = max(dmax, float(np.max(np.abs(gq - rq))))
        print(f"{name} periodic EEDFs: largest cumulative difference {dmax:.4f}")
        if dmax > 0.01:
            failures.append(f"periodic EEDF cumulative probability differs by {dmax:.4f}")
    assert not failures, f"{name}:\n" + "\n".join(failures)
