"""CPU restatement of the reference's end-of-job post-processing of an EEDF.

TEST INFRASTRUCTURE, NOT PRODUCT: the checker of the device's
lgpu_eedf_postprocess, pinned to the reference's own outputs in
tests/golden/eedf_post_*.npz (made by tests/golden/make_eedf_post.py).

It follows, in numpy double precision and in the reference's order of
elementwise operations (so the per-node totals come out bit for bit):

* the energy grid of Grid::updateMaxValue (Grid.C:44-53) with Eigen's
  LinSpaced (node i = i * step, the last node the maximum itself; cell i =
  step/2 + i * cell step, the last cell max - step/2);
* Collision::interpolatedCrossSection (Collision.C:229-288): linear
  interpolation of a raw table, zero below the first node above the threshold
  (every node for elastic collisions) and outside the table;
* Collision::superElasticCrossSection (Collision.C:290-353): Klein-Rosseland,
  sigma_f,i(u) = (g_i/g_f) (1 + threshold/u) sigma_i,f(u + threshold), zero at u = 0;
* Collision::evaluateRateCoeff (Collision.C:355-397): the EEDF-convolved
  inelastic (and superelastic) rate coefficient;
* BoltzmannMC::evaluateSwarmParameters (BoltzmannMC.C:2186-2266): the total
  momentum-transfer and energy-relaxation cross sections and the two-term
  swarm parameters from the EEDF.

The sums over cells use numpy's summation order, not Eigen's, so they agree
with the reference to rounding (~1e-15 relative), not bit for bit.
"""
from __future__ import annotations

import numpy as np

E_CHARGE = 1.6021766208e-19  # C (Constant.h:7)
E_MASS = 9.10938356e-31      # kg (Constant.h:8)

# the two-term swarm parameters, in the order of the device's lgpu_eedf_params
KEYS = ("totalIonRateCoeff", "totalAttRateCoeff", "momTransfFreq", "energyRelaxFreq", "energyRelaxFreqClassic",
        "redDiffCoeffEnergy_eedf", "redMobCoeffEnergy_eedf", "redDiffCoeff_eedf", "redMobCoeff_DC_eedf",
        "characEnergy_eedf", "redMobCoeff_xx_real_eedf", "redMobCoeff_xx_imag_eedf", "redMobCoeff_xy_real_eedf",
        "redMobCoeff_xy_imag_eedf", "redMobCoeff_zz_real_eedf", "redMobCoeff_zz_imag_eedf")


def grid(max_energy: float, n_cells: int):
    """(step, nodes, cells) of Grid::updateMaxValue with Eigen's LinSpaced."""
    step = max_energy / n_cells
    node = np.arange(n_cells + 1, dtype=np.float64) * step
    node[-1] = max_energy
    lo, hi = step / 2.0, max_energy - step / 2.0
    cstep = (hi - lo) / (n_cells - 1)
    cell = lo + np.arange(n_cells, dtype=np.float64) * cstep
    cell[-1] = hi
    return step, node, cell


def interp(e, v, x, threshold, elastic):
    """Collision::interpolatedCrossSection at the energies x."""
    out = np.zeros(len(x))
    if elastic:
        first = 0
    else:
        above = np.nonzero(x > threshold)[0]
        if len(above) == 0:
            return out
        first = above[0]
    n = len(e)
    for i in range(first, len(x)):
        xi = x[i]
        if xi < e[0] or xi > e[-1]:
            continue
        lo, hi = 0, n - 1
        while hi > lo + 1:
            mid = (hi + lo) // 2
            if e[mid] > xi:
                hi = mid
            else:
                lo = mid
        out[i] = v[lo] + (xi - e[lo]) / (e[lo + 1] - e[lo]) * (v[lo + 1] - v[lo])
    return out


def postprocess(eedf, max_energy, omega, omega_c, gas_density, procs):
    """The EEDF-convolved rate coefficient of every MC process and the two-term
    swarm parameters (KEYS order).

    procs: per MC process, in the reference's flattening order (a reversible
    collision followed by its superelastic copy), a dict with kind (0 elastic,
    1 inelastic, 2 superelastic copy), density (the target's; the product's for
    a copy), threshold (eV), mass_ratio (m_e / M), stat_ratio (g_target /
    g_product), ion (1 ionization, 2 attachment, else 0) and the collision's
    raw integral and momentum-transfer tables int_e, int_v, mom_e, mom_v (a copy
    carries its collision's)."""
    eedf = np.asarray(eedf, dtype=np.float64)
    nc = len(eedf)
    step, node, cell = grid(max_energy, nc)
    factor2 = np.sqrt(2.0 * E_CHARGE / E_MASS)
    factor = factor2 / 3.0
    mt = np.zeros(nc + 1)
    er = np.zeros(nc + 1)
    erc = np.zeros(nc + 1)
    rates = np.zeros(len(procs))
    sig = None  # the forward collision's integral cross section on the nodes
    k_ion = k_att = 0.0
    for p, q in enumerate(procs):
        thr = q["threshold"]
        if q["kind"] == 2:
            # Klein-Rosseland at the nodes (BoltzmannMC.C:2211-2218)
            s_int = np.zeros(nc + 1)
            s_mom = np.zeros(nc + 1)
            kr = 1.0 + thr / node[1:]
            s_int[1:] = kr * (interp(q["int_e"], q["int_v"], node + thr, thr, False)[1:] * q["stat_ratio"])
            s_mom[1:] = kr * (interp(q["mom_e"], q["mom_v"], node + thr, thr, False)[1:] * q["stat_ratio"])
            w = s_int * q["density"]
            aux = np.zeros(nc + 1)
            aux[1:] = w[1:] * thr / node[1:]
            mt = mt + s_mom * q["density"]
            er = er + aux
            erc = erc + w
            lmin = int(np.floor(thr / step))
            part = nc - lmin
            if part > 0:
                a = (sig[lmin:lmin + part] + sig[lmin + 1:lmin + 1 + part]) / 2.0 * cell[lmin:lmin + part]
                rates[p] = factor2 * q["stat_ratio"] * np.sum(a * eedf[0:part]) * step
            continue
        elastic = q["kind"] == 0
        sig = interp(q["int_e"], q["int_v"], node, thr, elastic)
        s_mom = interp(q["mom_e"], q["mom_v"], node, thr, elastic)
        mt = mt + s_mom * q["density"]
        if elastic:
            er = er + 2.0 * q["mass_ratio"] * sig * q["density"]
        else:
            w = sig * q["density"]
            aux = np.zeros(nc + 1)
            aux[1:] = w[1:] * thr / node[1:]
            er = er + aux
            erc = erc + w
        lmin = int(np.floor(thr / step))
        part = nc - lmin
        if part > 0:
            a = (sig[lmin:lmin + part] + sig[lmin + 1:lmin + 1 + part]) / 2.0 * cell[lmin:lmin + part]
            rates[p] = factor2 * np.sum(a * eedf[lmin:lmin + part]) * step
        if q["ion"] == 1:
            k_ion += q["density"] * rates[p]
        elif q["ion"] == 2:
            k_att += q["density"] * rates[p]
    N = gas_density
    out = dict(totalIonRateCoeff=k_ion, totalAttRateCoeff=k_att)
    pre = N * 3.0 * factor * step
    out["momTransfFreq"] = pre * np.sum(eedf * cell * ((mt[1:] + mt[:-1]) * 0.5))
    out["energyRelaxFreq"] = pre * np.sum(eedf * cell * ((er[1:] + er[:-1]) * 0.5))
    out["energyRelaxFreqClassic"] = pre * np.sum(eedf * cell * ((erc[1:] + erc[:-1]) * 0.5))
    mta = mt.copy()
    mta[1:] = mta[1:] + 1.0 / (3.0 * factor * np.sqrt(node[1:])) * (k_ion - k_att)
    mtf = N * mta * 3.0 * factor * np.sqrt(node)
    d_eedf = eedf[1:nc] - eedf[0:nc - 1]
    out["redDiffCoeffEnergy_eedf"] = 2.0 * factor * step * np.sum(cell ** 2 * eedf / (mta[:-1] + mta[1:]))
    out["redMobCoeffEnergy_eedf"] = -factor * np.sum(node[1:nc] ** 2 * d_eedf / mta[1:nc])
    out["redDiffCoeff_eedf"] = 2.0 * factor * step * np.sum(cell * eedf / (mta[:-1] + mta[1:]))
    out["redMobCoeff_DC_eedf"] = -factor * np.sum(node[1:nc] * d_eedf / mta[1:nc])
    out["characEnergy_eedf"] = out["redDiffCoeff_eedf"] / out["redMobCoeff_DC_eedf"]
    aux1 = -2.0 / 3.0 * E_CHARGE / E_MASS * node[1:nc] ** 1.5 * d_eedf
    f = mtf[1:nc]
    w, wc = omega, omega_c
    aux2 = (f * f + (w - wc) ** 2) * (f * f + (w + wc) ** 2)
    aux3 = f * f + w * w
    out["redMobCoeff_xx_real_eedf"] = N * np.sum(f * (f * f + w * w + wc * wc) / aux2 * aux1)
    out["redMobCoeff_xx_imag_eedf"] = -N * np.sum(w * (f * f + w * w - wc * wc) / aux2 * aux1)
    out["redMobCoeff_xy_real_eedf"] = -N * wc * np.sum((f * f - w * w + wc * wc) / aux2 * aux1)
    out["redMobCoeff_xy_imag_eedf"] = N * 2.0 * w * wc * np.sum(f / aux2 * aux1)
    out["redMobCoeff_zz_real_eedf"] = N * np.sum(f / aux3 * aux1)
    out["redMobCoeff_zz_imag_eedf"] = -N * np.sum(w / aux3 * aux1)
    return rates, np.array([out[k] for k in KEYS]), mt


def procs_from_fixture(d):
    """The per-process inputs of a tests/golden/eedf_post_*.npz fixture."""
    s = d["twoterm_scalars"]
    ni, nm = d["int_len"], d["mom_len"]
    oi = np.concatenate([[0], np.cumsum(ni)])
    om = np.concatenate([[0], np.cumsum(nm)])
    out = []
    for p in range(len(s)):
        out.append(dict(kind=int(s[p, 0]), density=float(s[p, 1]), threshold=float(s[p, 2]),
                        mass_ratio=float(s[p, 3]), stat_ratio=float(s[p, 4]), ion=int(s[p, 5]),
                        int_e=d["int_e"][oi[p]:oi[p + 1]], int_v=d["int_v"][oi[p]:oi[p + 1]],
                        mom_e=d["mom_e"][om[p]:om[p + 1]], mom_v=d["mom_v"][om[p]:om[p + 1]]))
    return out
