"""The advance's per-process energy tallies, modelled on the host.

A block adds every real collision's energy change dE (FP32) to its
condition's per-process tallies in shared memory. A plain FP32 running sum of
thousands of nearly equal inelastic losses rounds by up to ~1e-4 relative;
the kernel (lane_real / block_flush in loki-mc_gb300/csrc/lgpu_advance.cuh)
instead keeps, per process and sign, the count and the FP32 sum of
dE - nominal (minus the process's threshold; zero for attachment), and adds
count x nominal back in FP64 at the flush. This replays both in numpy with
FP32 sequential accumulation (np.add.accumulate adds in order, in the array's
type) and checks the split sum against an FP64 sum of the same FP32 values.
"""
import numpy as np
import pytest


def sequential_fp32(v):
    return float(np.add.accumulate(np.asarray(v, dtype=np.float32))[-1])


@pytest.mark.parametrize("n,eloss,spread", [(30000, 2.3, 2e-4), (10000, 0.289, 2e-4), (5000, 11.7, 1e-3),
                                            (20000, -0.0012, 1e-2)])
def test_split_tally_keeps_the_power_terms_exact(n, eloss, spread):
    rng = np.random.default_rng(7)
    # an inelastic loss (a superelastic gain for eloss < 0) plus a small recoil
    d_e = (-eloss - np.sign(eloss) * rng.exponential(spread * abs(eloss), n)).astype(np.float32)
    exact = float(np.sum(d_e.astype(np.float64)))
    nominal = np.float32(-eloss)
    rest = (d_e - nominal).astype(np.float32)           # exact (Sterbenz) for these magnitudes
    assert np.all(rest.astype(np.float64) == d_e.astype(np.float64) - np.float64(nominal))
    split = n * float(nominal) + sequential_fp32(rest)
    assert abs(split - exact) <= 1e-7 * abs(exact)
    # the plain FP32 running sum it replaces
    plain = sequential_fp32(d_e)
    if n >= 10000 and abs(eloss) > 0.1:
        assert abs(plain - exact) > 1e-6 * abs(exact)


def test_ionization_and_elastic_remainders():
    """Ionization changes the energy by exactly minus its threshold (nothing
    left to sum); an elastic collision has no nominal change (its recoils are
    summed as they are: an FP32 sum of 10,000 of them within a few 1e-6)."""
    thr = np.float32(15.6)
    assert float(np.float32(-thr) - np.float32(-thr)) == 0.0
    rng = np.random.default_rng(3)
    recoil = (-rng.exponential(1e-4, 10000)).astype(np.float32)
    exact = float(np.sum(recoil.astype(np.float64)))
    assert abs(sequential_fp32(recoil) - exact) <= 1e-5 * abs(exact)
