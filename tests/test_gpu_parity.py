"""GPU parity: the production device functions against the oracle.

The oracle (oracle/loki_oracle.c) reproduces the reference bit for bit on
these vectors (tests/test_oracle_golden.py). The GPU computes in FP32, so:

* tables: the FP32 values the kernels use equal the FP64 oracle tables
  rounded to FP32 (the device builds them in FP64 with round-to-nearest
  operations);
* free flights (every field branch): velocity within 1e-5 of |v| and
  position within 1e-5 of (|x| + |v dt|), energy and field gain within
  2e-5 of the energy (the FP32 tolerance of the per-electron kinematics);
* collision events: the chosen process agrees except where the event sits
  within FP32 rounding of a boundary between processes (a relative
  perturbation of the inputs of 1e-5 moves the oracle to the device's choice;
  at most 0.5 % of events), and the post-collision velocity, energy,
  secondary and uniform count match the oracle to 1e-5 relative (1e-4
  against the perturbed oracle event on a boundary);
* the production null test with its block bounds decides every event as the
  plain one does.
"""
import numpy as np
import pytest

import golden_util as gu
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=gu.CASES)
def gpu_case(request):
    from lokigpu import capi

    g = gu.load(request.param)
    sc = g["scalars_tab"]
    M = len(g["tab_grid"])
    arrays = gu.proc_arrays(g)
    ps = gu.processes(arrays)
    ctx = capi.Context(capi.default_config(n_electrons=1024, n_interp=M))
    ctx.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
    ctx.set_conditions(sc[0], sc[1], 100.0)
    yield request.param, g, ctx, ps
    ctx.close()


def test_tables(gpu_case):
    _, g, ctx, ps = gpu_case
    sc = g["scalars_tab"]
    M = len(g["tab_grid"])
    nu_tot, nu_max, sig, cum = ctx.build_tables(sc[15], M, ps.n)
    np.testing.assert_allclose(nu_tot, g["tab_nu_tot"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(nu_max, g["tab_nu_max"], rtol=1e-15, atol=0)
    assert np.array_equal(sig, g["tab_sig"].astype(np.float32))
    assert np.array_equal(cum, g["tab_cum"].astype(np.float32))


@pytest.mark.parametrize("branch", gu.BRANCHES)
def test_free_flights(gpu_case, branch):
    _, g, ctx, _ = gpu_case
    fp = g[f"acc_{branch}_field"]
    ctx.set_field_raw(fp[:3], fp[3], fp[4], fp[5])
    t, dt = g[f"acc_{branch}_t"], g[f"acc_{branch}_dt"]
    pos, vel = g[f"acc_{branch}_pos"], g[f"acc_{branch}_vel"]
    po, vo, eo, go = ctx.replay_flights(t, dt, pos, vel)
    ref_p, ref_v = g[f"acc_{branch}_pos_out"], g[f"acc_{branch}_vel_out"]
    ref_e, ref_g = g[f"acc_{branch}_energy_out"], g[f"acc_{branch}_gain"]
    for k in range(len(t)):
        vs = np.linalg.norm(ref_v[k])
        assert np.linalg.norm(vo[k] - ref_v[k]) <= 1e-5 * vs, (branch, k)
        ps_ = np.linalg.norm(pos[k]) + np.linalg.norm(vel[k]) * dt[k]
        assert np.linalg.norm(po[k] - ref_p[k]) <= 1e-5 * ps_, (branch, k)
        assert abs(eo[k] - ref_e[k]) <= 2e-5 * ref_e[k], (branch, k)
        assert abs(go[k] - ref_g[k]) <= 2e-5 * max(ref_e[k], g[f"acc_{branch}_energy"][k]), (branch, k)


def _f32(a):
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


# Relative size of the input perturbations that stand for the FP32 rounding of
# the device's intermediate values (a few units in the last place of FP32,
# i.e. ~1e-7, amplified by the few operations before a comparison).
PERTURB = 1e-5


def _perturbed_choices(pr, f, nu, vel, en, u, rng):
    """Oracle outcomes of one event under small relative perturbations of its
    inputs (trial frequency, velocity, energy, uniforms), each outcome with the
    perturbed inputs' result: the processes the event can pick within the
    FP32 rounding of the device arithmetic."""
    out = []
    for k in range(24):
        if k < 8:  # one input at a time, both signs
            which, sign = k // 2, 1.0 if k % 2 == 0 else -1.0
            d = np.zeros(4)
            d[which] = sign
            dn, dv, de, du = d * PERTURB
            dvv = np.full(3, dv)
            duu = np.full(len(u), du)
        else:  # all inputs at once, random signs
            dn, de = rng.choice([-1.0, 1.0], 2) * PERTURB
            dvv = rng.choice([-1.0, 1.0], 3) * PERTURB
            duu = rng.choice([-1.0, 1.0], len(u)) * PERTURB
        uu = np.clip(u * (1.0 + duu), 1e-300, 1.0)
        res, used, _ = O.collide(pr, f, nu * (1.0 + dn), vel * (1.0 + dvv), en * (1.0 + de), uu)
        out.append((res, used))
    return out


def _kinematics_agree(got, ref, en, tol):
    vs = np.linalg.norm(ref[1:4])
    es = np.linalg.norm(ref[7:10])
    return (np.linalg.norm(got[1:4] - ref[1:4]) <= tol * max(vs, 1.0) and abs(got[4] - ref[4]) <= tol * max(en, 1e-3)
            and abs(got[5] - ref[5]) <= tol * max(en, 1e-3) and
            np.linalg.norm(got[7:10] - ref[7:10]) <= tol * max(es, 1.0))


def test_collisions(gpu_case):
    """The kernel reads its inputs (trial frequency, velocity, energy and the
    recorded uniforms) as FP32; the oracle gets the same FP32-rounded values,
    so the comparison measures the FP32 arithmetic of the device alone.

    Every event, cold and thermal: where the device picks the oracle's
    process, the post-collision velocity, energy, energy change, secondary and
    uniform count agree to 1e-5 relative. Where it picks another one, that
    process must be one the oracle picks under a relative perturbation of the
    inputs of 1e-5 (the event sits on a boundary within FP32 rounding), and
    the kinematics must agree with that perturbed oracle event to 1e-4. The
    production null test (block bounds first, lgpu_replay_collisions_coarse)
    takes the same decisions. The mismatch count per mode is printed."""
    name, g, ctx, ps = gpu_case
    sc = g["scalars_tab"]
    M = len(g["tab_grid"])
    pr = O.OracleProcs(gu.proc_arrays(g), M)
    pr.build_tables(O.make_fields(sc[0], sc[1]), sc[15])
    from lokigpu import capi

    rng = np.random.default_rng(7)
    for m in range(gu.n_modes(g)):
        gte, shr, fac = g[f"col{m}_opts"]
        cfg = capi.default_config(n_electrons=1024, n_interp=M, gas_temperature_effect=int(gte), sharing=int(shr))
        c2 = capi.Context(cfg)
        arrays = gu.proc_arrays(g)
        c2.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
        c2.set_conditions(sc[0], sc[1], 100.0)
        c2.build_tables(sc[15], M, ps.n)
        nu, vel, en, U = (_f32(g[f"col{m}_{k}"]) for k in ("nu", "vel", "energy", "u"))
        out, used = c2.replay_collisions(nu, vel, en, U)
        out_c, used_c = c2.replay_collisions(nu, vel, en, U, coarse=True)
        c2.close()
        # same decisions, uniform counts and kinematics bit for bit: the device
        # code is built without multiply-add contraction, so both replay paths
        # round every step alike
        assert np.array_equal(out[:, 0], out_c[:, 0]) and np.array_equal(used, used_c), (name, m)
        assert np.array_equal(out, out_c), (name, m)
        f = O.make_fields(sc[0], sc[1], gas_temp_effect=int(gte), sharing=int(shr), sharing_factor=fac)
        mismatch, compared, real = 0, 0, 0
        for k in range(len(nu)):
            ref, ref_used, _ = O.collide(pr, f, nu[k], vel[k], en[k], U[k])
            if out[k][0] == ref[0]:
                if ref[0] < 0:
                    continue
                real += 1
                compared += 1
                assert used[k] == ref_used, (name, m, k)
                assert _kinematics_agree(out[k], ref, en[k], 1e-5), (name, m, k, out[k], ref)
                continue
            mismatch += 1
            alts = [(r, u_) for r, u_ in _perturbed_choices(pr, f, nu[k], vel[k], en[k], U[k], rng)
                    if r[0] == out[k][0]]
            assert alts, (f"{name} mode {m} event {k}: device picks {out[k][0]:.0f}, the oracle {ref[0]:.0f} "
                          f"and no perturbation of 1e-5 moves it there")
            if out[k][0] >= 0:
                assert any(_kinematics_agree(out[k], r, en[k], 1e-4) for r, _ in alts), (name, m, k, out[k], alts[0][0])
                compared += 1
        print(f"{name} mode {m} (gas temperature {int(gte)}, sharing {int(shr)}): {len(nu)} events, "
              f"{real} real collisions compared, {mismatch} process choices on a boundary")
        assert compared > 100, (name, m, compared)
        assert mismatch <= 0.005 * len(nu), (name, m, mismatch)


def test_coarse_null_test_never_changes_a_decision(gpu_case):
    """The advance kernels' null test compares the random frequency with an
    upper bound of the total frequency over a block of table rows before it
    reads the row. Over random energies across the whole table and random
    uniforms, the coarse and the plain null test decide alike, event by event."""
    name, g, ctx, ps = gpu_case
    sc = g["scalars_tab"]
    M = len(g["tab_grid"])
    ctx.build_tables(sc[15], M, ps.n)
    rng = np.random.default_rng(11)
    n = 200_000
    en = _f32(rng.uniform(0.0, sc[15] * (M - 1) / M, n))
    speed = np.sqrt(2.0 * en * 1.6021766208e-19 / 9.10938356e-31)
    d = rng.normal(size=(n, 3))
    vel = _f32(d / np.linalg.norm(d, axis=1)[:, None] * speed[:, None])
    nu_max = float(np.max(g["tab_nu_max"]))
    nu = _f32(np.full(n, nu_max))
    U = _f32(rng.uniform(1e-7, 1.0, (n, 12)))
    out, used = ctx.replay_collisions(nu, vel, en, U)
    out_c, used_c = ctx.replay_collisions(nu, vel, en, U, coarse=True)
    assert np.array_equal(out[:, 0], out_c[:, 0]), (name, np.flatnonzero(out[:, 0] != out_c[:, 0])[:10])
    assert np.array_equal(used, used_c), name
    assert np.count_nonzero(out[:, 0] >= 0) > 100, name
