"""Loading helpers for the golden vectors in tests/golden/ (made by
tests/golden/make_golden.py from the reference built from source)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("atomic", "n2", "mix", "screen")
BRANCHES = ("dc", "ac", "b", "ecr", "acb")


def load(case):
    return dict(np.load(os.path.join(GOLDEN, f"kin_{case}.npz")))


def proc_arrays(g):
    keys = ("ptype", "is_super", "is_elastic", "sampler", "sampler_p0", "sampler_p1", "superw", "emin", "emax",
            "rel_dens", "mass", "red_mass", "eloss", "wparam", "raw_off", "raw_len", "raw_e", "raw_v", "gas_first",
            "gas_last", "gas_frac", "energy_max_elastic")
    return {k: g[k] for k in keys}


def n_modes(g):
    return len([k for k in g if k.endswith("_opts")])


def processes(arrays):
    """ProcessSet view of the golden per-process arrays."""
    from lokigpu.synth import ProcessSet

    off, ln = arrays["raw_off"], arrays["raw_len"]
    raw_e = [arrays["raw_e"][off[p]:off[p] + ln[p]] for p in range(len(off))]
    raw_v = [arrays["raw_v"][off[p]:off[p] + ln[p]] for p in range(len(off))]
    return ProcessSet(ptype=arrays["ptype"], is_super=arrays["is_super"], is_elastic=arrays["is_elastic"],
                      sampler=arrays["sampler"], sampler_p0=arrays["sampler_p0"], sampler_p1=arrays["sampler_p1"],
                      superw=arrays["superw"], emin=arrays["emin"], emax=arrays["emax"], rel_dens=arrays["rel_dens"],
                      mass=arrays["mass"], red_mass=arrays["red_mass"], eloss=arrays["eloss"],
                      wparam=arrays["wparam"], raw_e=raw_e, raw_v=raw_v, gas_first=arrays["gas_first"],
                      gas_last=arrays["gas_last"], gas_fraction=arrays["gas_frac"],
                      energy_max_elastic=float(arrays["energy_max_elastic"]),
                      gas_index=np.zeros(len(off), np.int32))


# ---- distributions on common coarse grids ----------------------------------
# The reference's and the device's distributions live on grids that follow
# each run's own largest energy (BoltzmannMC.C:1497-1548, 1862-1889), so they
# are compared through cumulative probabilities evaluated at common edges:
# the probability mass of every fine cell is summed into a cumulative curve
# over the cell nodes and interpolated linearly (exact at the nodes).

def energy_nodes(cells):
    cells = np.asarray(cells, np.float64)
    de = cells[1] - cells[0]
    return np.arange(len(cells) + 1) * de


def eedf_mass(cells, eedf):
    """Probability of each energy cell: f sqrt(e) de (BoltzmannMC.C:1574-1580
    normalises f so that these sum to 1)."""
    cells = np.asarray(cells, np.float64)
    return np.asarray(eedf, np.float64) * np.sqrt(cells) * (cells[1] - cells[0])


def cdf_at(nodes, mass, edges):
    """Cumulative mass at arbitrary edges; mass may carry trailing axes."""
    mass = np.asarray(mass, np.float64)
    c = np.concatenate([np.zeros((1,) + mass.shape[1:]), np.cumsum(mass, axis=0)], axis=0)
    flat = c.reshape(c.shape[0], -1)
    out = np.stack([np.interp(edges, nodes, flat[:, j]) for j in range(flat.shape[1])], axis=-1)
    return out.reshape((len(edges),) + mass.shape[1:])


def eadf_mass(cells, eadf, cos_groups):
    """Probability per (energy cell, group of cos cells): eadf is 2 h /
    (sqrt(e) norm de dcos) (BoltzmannMC.C:1583-1586)."""
    cells = np.asarray(cells, np.float64)
    eadf = np.asarray(eadf, np.float64)
    n_cos = eadf.shape[1]
    m = eadf * (np.sqrt(cells) * (cells[1] - cells[0]))[:, None] * (1.0 / n_cos)
    return m.reshape(len(cells), cos_groups, n_cos // cos_groups).sum(axis=2)


def legendre_mass(cells, f, degree):
    """Sum over cos of the cell probability times P_degree(cos): the first and
    second anisotropies are (l + 1/2) sum_k eadf P_l(cos_k) dcos
    (BoltzmannMC.C:1588-1600)."""
    cells = np.asarray(cells, np.float64)
    return np.asarray(f, np.float64) * np.sqrt(cells) * (cells[1] - cells[0]) / (2.0 * degree + 1.0)


def evdf_cdf(radial_cells, axial_cells, evdf, r_edges, z_edges):
    """2-D cumulative probability of the EVDF at (radial, axial) edges: the
    cell probability is evdf 2 pi v_r dv_r dv_z (BoltzmannMC.C:1603)."""
    rc, ac = np.asarray(radial_cells, np.float64), np.asarray(axial_cells, np.float64)
    dr, dz = rc[1] - rc[0], ac[1] - ac[0]
    m = np.asarray(evdf, np.float64) * (2.0 * np.pi * rc * dr)[:, None] * dz
    rn = np.arange(len(rc) + 1) * dr
    zn = ac[0] - 0.5 * dz + np.arange(len(ac) + 1) * dz
    c = np.zeros((len(rc) + 1, len(ac) + 1))
    c[1:, 1:] = np.cumsum(np.cumsum(m, axis=0), axis=1)
    cr = np.stack([np.interp(r_edges, rn, c[:, j]) for j in range(c.shape[1])], axis=1)
    return np.stack([np.interp(z_edges, zn, cr[i, :]) for i in range(cr.shape[0])], axis=0)
