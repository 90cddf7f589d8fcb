"""Requests from the reference's own input files (lgpu_request_*): the
library parses a setup file and its LXCat files (texts, no file access) and
flattens them as the reference does (BoltzmannMC.C:29-271). Against the
reference's own flattening of the same files (the golden vectors from the
reference built from source): the same processes, types, samplers,
thresholds, masses, superelastic weights, relative densities and raw cross
sections (1e-15: the reference reads numbers through its expression parser,
whose text round trip can move the last bit, Parse.C:727-745), and the
collision tables its end-of-job routines read (momentum transfer from the
angular laws). Also the
working-condition vector that makes one job per entry, expressions,
boltzmannPopulation@T families, the errors for inputs this front end does
not read, and the parse rate a server needs."""
import os
import sys
import time

import numpy as np
import pytest

import golden_util as gu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402  (case definitions only; the reference is not loaded)

KB = 1.38064852e-23


def _texts(tmp):
    inp = os.path.join(tmp, "Input")
    setup = open(os.path.join(inp, "case.in")).read()
    files = {f: open(os.path.join(inp, f)).read() for f in os.listdir(inp) if f.endswith("_LXCat.txt")}
    return setup, files


@pytest.mark.parametrize("case", gu.CASES)
def test_request_flattening_matches_the_reference(case, tmp_path):
    from lokigpu import capi

    _, meta, _ = make_golden.write_inputs(case, str(tmp_path))
    req = capi.Request(*_texts(str(tmp_path)))
    assert len(req) == 1
    got = req.processes()
    g = gu.load(case)
    assert np.array_equal(got["type"], g["ptype"])
    for k in ("is_super", "sampler", "gas_first", "gas_last"):
        assert np.array_equal(got[k], g[k]), k
    for k in ("sampler_p0", "sampler_p1", "superw", "emin", "emax", "mass", "eloss", "wparam"):
        assert np.array_equal(got[k], g[k]), k
    np.testing.assert_allclose(got["rel_dens"], g["rel_dens"], rtol=1e-14, atol=0)
    np.testing.assert_array_equal(got["gas_frac"], g["gas_frac"])
    assert got["energy_max_elastic"] == float(g["energy_max_elastic"])
    for p in range(len(got["type"])):
        if got["is_super"][p]:
            continue
        o, n = g["raw_off"][p], g["raw_len"][p]
        np.testing.assert_allclose(got["raw_e"][p], g["raw_e"][o:o + n], rtol=1e-15, atol=0)
        np.testing.assert_allclose(got["raw_v"][p], g["raw_v"][o:o + n], rtol=1e-15, atol=0)
    j = req.job(0)
    assert abs(j.conditions.gas_density / meta["N"] - 1.0) < 1e-12
    assert j.conditions.reduced_field_td == meta["red_field"]
    assert j.config.n_electrons == 1e4 and j.config.n_interp == 2000
    req.close()


def test_request_jobs_from_a_vector_and_expressions(tmp_path):
    from lokigpu import capi, synth

    synth.write_case(str(tmp_path), [synth.reid_ramp_gas()], pressure_pa=133.32, red_field=[1.0, 12.0, 24.0],
                     n_electrons=1e5, extra_numerics={"nIntegrationPoints": "1E4", "nIntegratedSSTimes": "2"})
    setup, files = _texts(str(tmp_path))
    setup = setup.replace("gasPressure: 133.32", "gasPressure: 1.3332E2*(1+0)   % in Pa")
    req = capi.Request(setup, files)
    assert len(req) == 3
    for k, td in enumerate((1.0, 12.0, 24.0)):
        j = req.job(k)
        assert j.conditions.reduced_field_td == td
        assert abs(j.conditions.gas_density / (133.32 / (KB * 300.0)) - 1.0) < 1e-14
        assert j.config.req_ss_times == 2.0 and j.config.req_integration_points == 1e4
    p = req.processes()
    assert list(p["type"]) == [0, 0] and p["eloss"][1] == 0.2 and abs(p["mass"][0] - 4.0 * 1.660539040e-27) < 1e-40
    # a logspace vector of E/N
    req2 = capi.Request(setup.replace("reducedElecField: [1.0,12.0,24.0]", "reducedElecField: logspace(0,3,64)"),
                        files)
    assert len(req2) == 64 and abs(req2.job(63).conditions.reduced_field_td - 1000.0) < 1e-9


def test_request_boltzmann_populations(tmp_path):
    """Vibrational populations given as boltzmannPopulation@gasTemperature over
    the family X2(X,v=*) equal the explicit Boltzmann values the synthetic
    setup writes (StatePropertyFunctions.h:172-197)."""
    from lokigpu import capi

    import re

    make_golden.write_inputs("n2", str(tmp_path))
    setup, files = _texts(str(tmp_path))
    ref = capi.Request(setup, files).processes()
    out, in_pop = [], False
    for l in setup.splitlines():
        if l.strip() == "population:":
            in_pop = True
            out += [l, "      - X2(X,v=*) = boltzmannPopulation@gasTemperature"]
            continue
        if in_pop and re.match(r"\s*- X2\(X,v=\d+\) =", l):
            continue  # the family's explicit values
        if in_pop and not l.startswith("      -"):
            in_pop = False
        out.append(l)
    got = capi.Request("\n".join(out) + "\n", files).processes()
    np.testing.assert_allclose(got["rel_dens"], ref["rel_dens"], rtol=1e-12, atol=1e-300)


def test_request_errors_name_what_is_not_read(tmp_path):
    from lokigpu import capi

    make_golden.write_inputs("screen", str(tmp_path))
    setup, files = _texts(str(tmp_path))
    # a momentum-transfer cross section of a process with an anisotropic law
    bad = {k: v.replace(", Integral]", "]") for k, v in files.items()}
    with pytest.raises(capi.LokiGpuError) as e:
        capi.Request(setup, bad)
    assert "momentum-transfer" in str(e.value)
    with pytest.raises(capi.LokiGpuError) as e:
        capi.Request(setup.replace("eedfType: boltzmannMC", "eedfType: prescribedEedf"), files)
    assert "boltzmannMC" in str(e.value)
    with pytest.raises(capi.LokiGpuError) as e:
        capi.Request(setup, {})
    assert "was not given" in str(e.value)


def test_request_parse_rate(tmp_path):
    """A server parses a request of the two-gas mixture (65 processes, 200-point
    grids, ~40 KB of text; the momentum-transfer integration of its angular
    laws over 1000 angles included) in some 10 milliseconds, beside solves of
    seconds."""
    from lokigpu import capi

    make_golden.write_inputs("mix", str(tmp_path))
    setup, files = _texts(str(tmp_path))
    capi.Request(setup, files).close()
    n = 50
    t0 = time.perf_counter()
    for _ in range(n):
        capi.Request(setup, files).close()
    per = (time.perf_counter() - t0) / n
    print(f"request parse: {1e3 * per:.3f} ms per request ({1.0 / per:.0f} requests/s)")
    assert per < 0.05


@pytest.mark.parametrize("name", ["atomic_dc100", "n2_dc200", "mix_dc300", "screen_dc100"])
def test_request_twoterm_inputs_match_the_reference(name, tmp_path):
    """The collision behind each process as the reference's end-of-job
    routines read it (tests/golden/eedf_post_*.npz, from the reference built
    from source): the raw integral cross section (the LXCat table, an elastic
    one starting at zero energy, Collision.C:40-43), the momentum-transfer one
    the angular law gives (the trapezoidal integration of Collision.C:127-199
    over angleNumber angles, for the Born-dipole, Surendra, screened-Coulomb
    and forward laws of these mixtures), target and product densities,
    thresholds, mass and statistical-weight ratios."""
    import make_eedf_post
    from lokigpu import capi

    case, over, numerics = make_eedf_post.CASES[name]
    make_golden.write_inputs(case, str(tmp_path), n_electrons=2e4, extra=numerics, **over)
    req = capi.Request(*_texts(str(tmp_path)))
    got = req.twoterm(0)
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"eedf_post_{name}.npz"))
    s = d["twoterm_scalars"]
    oi = np.concatenate([[0], np.cumsum(d["int_len"])])
    om = np.concatenate([[0], np.cumsum(d["mom_len"])])
    assert len(got) == len(s)
    for p, t in enumerate(got):
        assert (t["kind"], t["ion"]) == (int(s[p, 0]), int(s[p, 5])), p
        np.testing.assert_allclose([t["density"], t["threshold"], t["mass_ratio"]], s[p, 1:4], rtol=1e-14, atol=0)
        if s[p, 4] != 0:
            assert abs(t["stat_ratio"] / s[p, 4] - 1.0) < 1e-15, p
        np.testing.assert_allclose(t["int_e"], d["int_e"][oi[p]:oi[p + 1]], rtol=1e-15, atol=0)
        np.testing.assert_allclose(t["int_v"], d["int_v"][oi[p]:oi[p + 1]], rtol=1e-15, atol=0)
        np.testing.assert_allclose(t["mom_e"], d["mom_e"][om[p]:om[p + 1]], rtol=1e-15, atol=0)
        # 1 - (angular integral): for strongly forward laws at high energy the
        # integral nears 1, so the last-bit differences of the cos x sin weights
        # (the reference's come from its vector library) grow to ~1e-11
        np.testing.assert_allclose(t["mom_v"], d["mom_v"][om[p]:om[p + 1]], rtol=1e-10, atol=1e-300)
