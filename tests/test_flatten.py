"""Host logic: the product's flattening of a gas mixture into per-process
arrays (lokigpu.synth.flatten) equals the reference's own flattening
(BoltzmannMC.C:29-271), recorded in the golden vectors from the reference
built from source, including relative densities and superelastic weights.

The raw cross-section values agree to 1e-15 relative rather than bit for bit:
the reference reads every LXCat number through its expression parser, whose
text round trip (Parse.C:727-745) can move the last bit."""
import os
import sys

import numpy as np
import pytest

import golden_util as gu
from lokigpu import synth

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402  (case definitions only; the reference is not loaded)


@pytest.mark.parametrize("case", gu.CASES)
def test_flatten_matches_reference(case):
    g = gu.load(case)
    gases, _ = make_golden.case_gases(case)
    ps = synth.flatten(gases)
    for k in ("ptype", "is_super", "sampler", "gas_first", "gas_last"):
        assert np.array_equal(getattr(ps, k), g[k]), k
    for k in ("sampler_p0", "sampler_p1", "superw", "emin", "emax", "mass", "red_mass", "eloss", "wparam"):
        assert np.array_equal(getattr(ps, k), g[k]), k
    np.testing.assert_allclose(ps.rel_dens, g["rel_dens"], rtol=1e-14, atol=0)
    np.testing.assert_array_equal(ps.gas_fraction, g["gas_frac"])
    assert ps.energy_max_elastic == float(g["energy_max_elastic"])
    for p in range(ps.n):
        o, n = g["raw_off"][p], g["raw_len"][p]
        assert len(ps.raw_e[p]) == n, p
        np.testing.assert_allclose(ps.raw_e[p], g["raw_e"][o:o + n], rtol=1e-15, atol=0)
        np.testing.assert_allclose(ps.raw_v[p], g["raw_v"][o:o + n], rtol=1e-15, atol=0)
