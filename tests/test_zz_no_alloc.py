"""lgpu_replay_flights_noalloc: free flights for callers that cannot
allocate device memory (a serving process that reserved the device up front,
an application whose own allocator owns the device, a pipeline stage that
must not allocate). It runs the same free-flight kernel as
lgpu_replay_flights, staged through a static device array instead of a
context's buffers, so its outputs must equal that entry point's - here on two
calls in a row with different fields and inputs, since every call shares the
static array and the second must not see the first's contents. Collected last
(file name) so that a run stopping at the first failure has run every other
test first."""
import numpy as np
import pytest

import golden_util as gu

pytestmark = pytest.mark.gpu


def _existing(branch, g):
    from lokigpu import capi

    sc = g["scalars_tab"]
    fp = g[f"acc_{branch}_field"]
    arrays = gu.proc_arrays(g)
    ps = gu.processes(arrays)
    ctx = capi.Context(capi.default_config(n_electrons=1024, n_interp=len(g["tab_grid"])))
    ctx.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
    ctx.set_conditions(sc[0], sc[1], 100.0)
    ctx.set_field_raw(fp[:3], fp[3], fp[4], fp[5])
    out = ctx.replay_flights(g[f"acc_{branch}_t"], g[f"acc_{branch}_dt"], g[f"acc_{branch}_pos"],
                             g[f"acc_{branch}_vel"])
    ctx.close()
    return out


def test_noalloc_flights_match_existing_entry_point():
    from lokigpu import capi

    g = gu.load("n2")
    for branch in ("acb", "dc"):  # two calls in a row on the shared static array
        fp = g[f"acc_{branch}_field"]
        got = capi.replay_flights_noalloc(0, fp[:3], fp[3], fp[4], fp[5], g[f"acc_{branch}_t"],
                                          g[f"acc_{branch}_dt"], g[f"acc_{branch}_pos"], g[f"acc_{branch}_vel"])
        ref = _existing(branch, g)
        for a, b in zip(got, ref):
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)
        # and the oracle tolerance of the parity tests, against the reference's outputs
        vref = g[f"acc_{branch}_vel_out"]
        assert np.all(np.linalg.norm(got[1] - vref, axis=1) <= 1e-5 * np.linalg.norm(vref, axis=1))


def test_noalloc_short_call_after_a_long_one():
    """A call with fewer flights than the previous one must not pick up the
    values the longer call left in the shared static array."""
    from lokigpu import capi

    g = gu.load("n2")
    branch = "ac"
    fp = g[f"acc_{branch}_field"]
    args = [g[f"acc_{branch}_{k}"] for k in ("t", "dt", "pos", "vel")]
    n = len(args[0])
    assert n > 7
    capi.replay_flights_noalloc(0, fp[:3], fp[3], fp[4], fp[5], *args)
    short = [a[n - 7:] for a in args]
    got = capi.replay_flights_noalloc(0, fp[:3], fp[3], fp[4], fp[5], *short)
    sc = g["scalars_tab"]
    arrays = gu.proc_arrays(g)
    ctx = capi.Context(capi.default_config(n_electrons=1024, n_interp=len(g["tab_grid"])))
    ctx.set_processes(gu.processes(arrays), arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
    ctx.set_conditions(sc[0], sc[1], 100.0)
    ctx.set_field_raw(fp[:3], fp[3], fp[4], fp[5])
    ref = ctx.replay_flights(*short)
    ctx.close()
    for a, b in zip(got, ref):
        assert len(a) == 7
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)


def test_noalloc_rejects_a_negative_device():
    from lokigpu import capi

    z = np.zeros(4)
    with pytest.raises(capi.LokiGpuError) as e:
        capi.replay_flights_noalloc(-1, [0.0, 0.0, -1e3], 0.0, 0.0, 0.0, z, z + 1e-12, np.zeros((4, 3)),
                                    np.ones((4, 3)))
    assert e.value.code == 1


def test_noalloc_rejects_sizes_beyond_the_static_array():
    from lokigpu import capi

    n = 4097
    z = np.zeros(n)
    with pytest.raises(capi.LokiGpuError) as e:
        capi.replay_flights_noalloc(0, [0.0, 0.0, -1e3], 0.0, 0.0, 0.0, z, z + 1e-12, np.zeros((n, 3)),
                                    np.ones((n, 3)))
    assert e.value.code == 1
