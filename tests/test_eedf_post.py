"""The CPU restatement of the reference's end-of-job EEDF post-processing
(oracle/eedf_post.py) against the reference's own outputs on the same EEDFs
(tests/golden/eedf_post_*.npz, made by tests/golden/make_eedf_post.py from
short seeded solves of the reference built from its sources): the total
momentum-transfer cross section on the grid nodes bit for bit
(BoltzmannMC.C:2186-2218), the EEDF-convolved rate coefficient of every
process (Collision.C:355-397) and the two-term swarm parameters
(BoltzmannMC.C:2220-2266) to 1e-12 relative (the sums over cells run in a
different order). The cases cover elastic, inelastic, superelastic,
ionization and attachment processes, every angular law (the momentum-transfer
cross sections of the reference's angular integration), DC, crossed B and AC
fields."""
import glob
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import eedf_post as E  # noqa: E402

FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "eedf_post_*.npz")))


def test_fixtures_cover_the_cases():
    names = {os.path.basename(f)[10:-4] for f in FIXTURES}
    assert {"atomic_dc100", "n2_dc200", "mix_dc300", "mix_b100", "mix_ac150", "screen_dc100"} <= names
    kinds = set()
    for f in FIXTURES:
        d = np.load(f)
        kinds |= {int(k) for k in d["twoterm_scalars"][:, 0]}
        kinds |= {10 + int(k) for k in d["twoterm_scalars"][:, 5]}
        # the MC flattening's relative densities are the collisions' target
        # (product, for a superelastic copy) densities
        assert np.array_equal(d["proc_rel_dens"], d["twoterm_scalars"][:, 1])
    assert kinds >= {0, 1, 2, 11, 12}  # elastic, inelastic, superelastic, ionization, attachment


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[10:-4] for f in FIXTURES])
def test_oracle_repeats_the_reference_postprocessing(path):
    d = np.load(path)
    g = d["grid"]
    rates, swarm, mt = E.postprocess(d["eedf"], float(d["max_eedf_energy"]), g[0], g[1], g[2],
                                     E.procs_from_fixture(d))
    step, node, cell = E.grid(float(d["max_eedf_energy"]), len(d["eedf"]))
    assert step == g[3] and np.array_equal(cell, d["cells"])
    assert np.array_equal(mt, d["total_mt"])
    ref = d["rates"]
    assert np.all(np.abs(rates - ref) <= 1e-12 * np.abs(ref)), np.max(np.abs(rates - ref) / np.abs(ref))
    assert list(d["swarm_keys"]) == list(E.KEYS)
    bad = [(k, a, b) for k, a, b in zip(E.KEYS, swarm, d["swarm"]) if abs(a - b) > 1e-12 * abs(b)]
    assert not bad, bad


def test_oracle_repeats_the_reference_periodic_rates():
    """Under AC the reference also convolves every phase's EEDF
    (BoltzmannMC.C:2276-2330)."""
    d = np.load(os.path.join(HERE, "golden", "eedf_post_mix_ac150.npz"))
    g = d["grid"]
    assert g[0] > 0 and d["eedf_periodic"].shape[0] == 16
    procs = E.procs_from_fixture(d)
    for ph, row in enumerate(d["eedf_periodic"]):
        rates, _, _ = E.postprocess(row, float(d["max_eedf_energy"]), g[0], g[1], g[2], procs)
        ref = d["rates_periodic"][ph]
        assert np.all(np.abs(rates - ref) <= 1e-12 * np.abs(ref)), ph
