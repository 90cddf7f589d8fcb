"""The device's EEDF post-processing (lgpu_set_twoterm + lgpu_eedf_postprocess)
against the reference's own end-of-job routines on the same EEDFs.

tests/golden/eedf_post_*.npz (tests/golden/make_eedf_post.py) hold, for six
cases, the EEDF a short seeded reference solve ended with, the collision
behind every MC process as the reference's Collision holds it, and what the
reference computed from them: the EEDF-convolved rate coefficient of every
process (Collision.C:355-397) and the two-term swarm parameters
(BoltzmannMC.C:2186-2266). The device reads the same EEDF and the same
collisions under the same field frequencies and gas density; every value
agrees to 1e-12 relative (the device's elementwise steps round as the
reference's, its sums over cells run in another order). Then the context's
own EEDF after a solve, against the oracle's post-processing of the EEDF the
context reports, and the entry points' refusals.
"""
import glob
import os
import sys

import numpy as np
import pytest

import golden_util as gu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import eedf_post as E  # noqa: E402

pytestmark = pytest.mark.gpu
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "eedf_post_*.npz")))


def _context(d, n_electrons=1000, seed=1):
    from lokigpu import capi
    arrays = {k[5:]: v for k, v in d.items() if k.startswith("proc_")}
    el = arrays["is_elastic"] == 1
    arrays["energy_max_elastic"] = float(np.min(arrays["emax"][el])) if el.any() else 1e3
    ps = gu.processes(arrays)
    # start at kT = 1 eV, as the fixtures' reference runs did
    ctx = capi.Context(capi.default_config(n_electrons=float(n_electrons), n_interp=2000, seed=seed,
                                           init_temp_ratio=1.0 / (8.617333262e-5 * 300.0),
                                           req_integration_points=500.0, max_coll_before_ss=100.0))
    ctx.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
    w, wc, N = (float(x) for x in d["grid"][:3])
    ctx.set_conditions(N, 300.0, 100.0)
    if w or wc:
        ctx.set_field_raw([0.0, 0.0, -1e3], w / (2.0 * np.pi), 0.0, wc)
    return ctx


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[10:-4] for f in FIXTURES])
def test_device_repeats_the_reference_postprocessing(path):
    d = dict(np.load(path))
    ctx = _context(d)
    ctx.set_twoterm(E.procs_from_fixture(d))
    out, rates = ctx.eedf_postprocess(d["eedf"], float(d["max_eedf_energy"]))
    ref = d["rates"]
    bad = [(p, rates[p], ref[p]) for p in range(len(ref)) if abs(rates[p] - ref[p]) > 1e-12 * abs(ref[p])]
    assert not bad, bad
    vals = out.values()
    bad = [(k, a, b) for k, a, b in zip(E.KEYS, vals, d["swarm"]) if abs(a - b) > 1e-12 * abs(b)]
    assert not bad, bad
    ctx.close()


def test_own_eedf_after_a_solve():
    """After a solve the context post-processes its own time-averaged EEDF;
    the oracle, given the EEDF and grid the context reports, agrees."""
    d = dict(np.load(os.path.join(HERE, "golden", "eedf_post_n2_dc200.npz")))
    from lokigpu import capi
    ctx = _context(d, n_electrons=20000, seed=5)
    with pytest.raises(capi.LokiGpuError):
        ctx.eedf_postprocess()  # no two-term inputs yet
    ctx.set_twoterm(E.procs_from_fixture(d))
    with pytest.raises(capi.LokiGpuError):
        ctx.eedf_postprocess()  # no EEDF before the steady state
    ctx.set_conditions(float(d["grid"][2]), 300.0, 200.0)
    r = ctx.solve()
    assert r.integration_points > 0
    out, rates = ctx.eedf_postprocess()
    eedf = ctx.distributions()["eedf"]
    o_rates, o_vals, _ = E.postprocess(eedf, r.max_eedf_energy, 0.0, 0.0, float(d["grid"][2]),
                                       E.procs_from_fixture(d))
    assert np.all(np.abs(rates - o_rates) <= 1e-10 * np.abs(o_rates) + 1e-300)
    vals = out.values()
    bad = [(k, a, b) for k, a, b in zip(E.KEYS, vals, o_vals) if abs(a - b) > 1e-10 * abs(b)]
    assert not bad, bad
    # the characteristic energy of a DC swarm is of the order of its mean energy
    assert 0.1 * r.mean_energy < out.charac_energy < 10.0 * r.mean_energy
    ctx.close()


def test_refusals():
    from lokigpu import capi
    d = dict(np.load(os.path.join(HERE, "golden", "eedf_post_atomic_dc100.npz")))
    ctx = _context(d)
    procs = E.procs_from_fixture(d)
    with pytest.raises(capi.LokiGpuError):
        ctx.set_twoterm(procs[:1])  # one entry per process
    bad = [dict(q) for q in procs]
    bad[1]["int_e"] = bad[1]["int_e"][::-1].copy()
    with pytest.raises(capi.LokiGpuError):
        ctx.set_twoterm(bad)  # energies must increase
    ctx.set_twoterm(procs)
    with pytest.raises(capi.LokiGpuError):
        ctx.eedf_postprocess(d["eedf"][:1], 10.0)  # at least two cells
    ctx.close()


def test_device_repeats_the_reference_periodic_rates():
    """The rate coefficients of every phase's EEDF of an AC run
    (lgpu_eedf_rates, BoltzmannMC.C:2276-2330), given the reference's
    per-phase EEDFs; then a context's own per-phase EEDFs after an AC solve
    against the oracle on the per-phase EEDFs it reports."""
    from lokigpu import capi
    d = dict(np.load(os.path.join(HERE, "golden", "eedf_post_mix_ac150.npz")))
    ctx = _context(d)
    procs = E.procs_from_fixture(d)
    ctx.set_twoterm(procs)
    rates = ctx.eedf_rates(d["eedf_periodic"], float(d["max_eedf_energy"]))
    ref = d["rates_periodic"]
    assert rates.shape == ref.shape
    assert np.all(np.abs(rates - ref) <= 1e-12 * np.abs(ref))
    with pytest.raises(capi.LokiGpuError):
        ctx.eedf_rates()  # no EEDF yet
    ctx.close()
    # a context's own per-phase EEDFs (16 phases, omega/N = 1e-14 m^3/s)
    w = float(d["grid"][0])
    cfg = capi.default_config(n_electrons=20000.0, n_interp=2000, seed=9, n_phases=16,
                              init_temp_ratio=1.0 / (8.617333262e-5 * 300.0), req_integration_points=500.0,
                              max_coll_before_ss=100.0)
    arrays = {k[5:]: v for k, v in d.items() if k.startswith("proc_")}
    arrays["energy_max_elastic"] = float(np.min(arrays["emax"][arrays["is_elastic"] == 1]))
    ctx = capi.Context(cfg)
    ctx.set_processes(gu.processes(arrays), arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
    ctx.set_conditions(float(d["grid"][2]), 300.0, 150.0, 180.0, w / (2.0 * np.pi))
    ctx.set_twoterm(procs)
    r = ctx.solve()
    own = ctx.eedf_rates()
    per = ctx.distributions()["eedf_periodic"]
    for ph in range(per.shape[0]):
        if not np.isfinite(per[ph]).all() or per[ph].sum() == 0:
            continue
        o, _, _ = E.postprocess(per[ph], r.max_eedf_energy, w, 0.0, float(d["grid"][2]), procs)
        assert np.all(np.abs(own[ph] - o) <= 1e-10 * np.abs(o) + 1e-300), ph
    ctx.close()
