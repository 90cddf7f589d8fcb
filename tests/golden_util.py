"""Loading helpers for the golden vectors in tests/golden/ (made by
tests/golden/make_golden.py from the reference built from source)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("atomic", "n2", "mix")
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
