"""The CPU oracle (oracle/loki_oracle.c) against the reference's own outputs.

The golden vectors were produced by the reference engine built from its own
sources (tests/golden/make_golden.py, oracle/ref/). Everything here is FP64
and must agree bit for bit: the interpolated tables (BoltzmannMC.C:561-615),
free flights in every field branch (BoltzmannMC.C:804-905) and collision
events driven by recorded uniforms (BoltzmannMC.C:907-1280), including the
number of uniforms each event consumes.
"""
import numpy as np
import pytest

import golden_util as gu
import oracle as O


@pytest.fixture(scope="module", params=gu.CASES)
def case(request):
    g = gu.load(request.param)
    sc = g["scalars_tab"]
    pr = O.OracleProcs(gu.proc_arrays(g), len(g["tab_grid"]))
    pr.build_tables(O.make_fields(sc[0], sc[1]), sc[15])
    return request.param, g, pr


def test_tables_bit_exact(case):
    _, g, pr = case
    assert pr.s.step == g["scalars_tab"][16]
    for k in ("grid", "sig", "cum", "nu_tot", "nu_max"):
        assert np.array_equal(getattr(pr, k), g["tab_" + k]), k


@pytest.mark.parametrize("branch", gu.BRANCHES)
def test_free_flight_bit_exact(case, branch):
    _, g, _ = case
    sc = g["scalars_tab"]
    fp = g[f"acc_{branch}_field"]
    f = O.make_fields(sc[0], sc[1], E=fp[:3], freq_hz=fp[3], red_mag=fp[4], omega_c=fp[5])
    for k in range(len(g[f"acc_{branch}_t"])):
        p, v, e, gain = O.accelerate(f, g[f"acc_{branch}_t"][k], g[f"acc_{branch}_dt"][k], g[f"acc_{branch}_pos"][k],
                                     g[f"acc_{branch}_vel"][k], g[f"acc_{branch}_energy"][k])
        assert np.array_equal(p, g[f"acc_{branch}_pos_out"][k])
        assert np.array_equal(v, g[f"acc_{branch}_vel_out"][k])
        assert e == g[f"acc_{branch}_energy_out"][k]
        assert gain == g[f"acc_{branch}_gain"][k]


def test_collisions_bit_exact(case):
    name, g, pr = case
    sc = g["scalars_tab"]
    for m in range(gu.n_modes(g)):
        gte, shr, fac = g[f"col{m}_opts"]
        f = O.make_fields(sc[0], sc[1], gas_temp_effect=int(gte), sharing=int(shr), sharing_factor=fac)
        chosen = set()
        for k in range(len(g[f"col{m}_nu"])):
            out, used, overrun = O.collide(pr, f, g[f"col{m}_nu"][k], g[f"col{m}_vel"][k], g[f"col{m}_energy"][k],
                                           g[f"col{m}_u"][k])
            ref = g[f"col{m}_out"][k]
            assert overrun == 0
            assert used == g[f"col{m}_used"][k], (name, m, k)
            assert np.array_equal(out, ref), (name, m, k, out - ref)
            chosen.add(int(ref[0]))
        assert -1 in chosen and len(chosen) > 2  # null and several real processes exercised


def test_statistical_error_and_histogram():
    g = gu.load("atomic")
    # Eigen's mean() sums with SIMD packets, a different order than a plain
    # loop: the batch-means error agrees to rounding, not bit for bit.
    assert O.statistical_error(g["staterr_in"]) == pytest.approx(float(g["staterr_out"]), rel=1e-12)
    counts = np.zeros(100)
    step = g["hist_nodes"][1] - g["hist_nodes"][0]
    for x in g["hist_x"]:
        c = int((x - g["hist_nodes"][0]) / step)
        if c < 100:
            counts[c] += 1
    assert np.array_equal(counts, g["hist_counts"])
