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
