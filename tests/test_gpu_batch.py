"""Batched and served solves against the same solves run alone.

A batch (lgpu_batch_*) advances many contexts with one launch sequence per
synchronisation interval; a server (lgpu_server_*) does the same for jobs that
arrive while others run. Neither may change a result:

* without ionization and attachment nothing couples the electrons and every
  electron's random stream is fixed by (seed, electron, interval), so a
  batched solve repeats the solve alone: the device code is built without
  multiply-add contraction, so the single-condition kernel and the batched
  one in every launch shape compute the same bits. The tests allow 1e-4
  relative under DC and crossed B and 1e-3 under AC (time-dependent fields
  through the sines and cosines of the phase);
* with ionization and attachment the secondaries draw from streams named by
  the warp that pushes them and population control claims slots with
  atomics, so the runs are statistically equivalent: mean energy and drift
  agree within four combined standard errors or 1%, and the rates of processes
  with at least 2000 counts within five combined Poisson errors doubled for
  autocorrelation, plus 2%.

The cases use the reference's parsed inputs of tests/golden/kin_{atomic,mix}.npz
(the mixture is 80/20 two-gas with ionization and attachment) under DC, AC and
crossed-B fields with uneven electron counts.
"""
import time

import numpy as np
import pytest

import golden_util as gu

pytestmark = pytest.mark.gpu
KB_EV = 1.38064852e-23 / 1.6021766208e-19
N_GAS = 3.22e22
F_AC = N_GAS * 1e-16 / (2 * np.pi)  # omega/N = 1e-16 m^3/s

# (case, electrons, E/N (Td), angle, frequency (Hz), B/N (Hx), seed)
ATOMIC = [("atomic", 20000, 50.0, 180.0, 0.0, 0.0, 11), ("atomic", 50000, 100.0, 180.0, 0.0, 0.0, 12),
          ("atomic", 30000, 100.0, 90.0, 0.0, 500.0, 13), ("atomic", 30000, 150.0, 180.0, F_AC, 0.0, 14)]
MIX = [("mix", 50000, 100.0, 180.0, 0.0, 0.0, 21), ("mix", 20000, 300.0, 180.0, 0.0, 0.0, 22),
       ("mix", 30000, 100.0, 90.0, 0.0, 500.0, 23), ("mix", 30000, 150.0, 180.0, F_AC, 0.0, 24)]
# different mixtures (2, 40 and 65 processes) in one batch
MIXTURES = [("atomic", 20000, 100.0, 180.0, 0.0, 0.0, 31), ("n2", 40000, 200.0, 180.0, 0.0, 0.0, 32),
            ("mix", 30000, 100.0, 180.0, 0.0, 0.0, 33), ("n2", 25000, 150.0, 90.0, 0.0, 800.0, 34)]


def _inputs(case):
    g = gu.load(case)
    arrays = gu.proc_arrays(g)
    return gu.processes(arrays), arrays


def _config(n_e, seed):
    from lokigpu import capi
    return capi.default_config(n_electrons=float(n_e), n_interp=2000, seed=seed, init_temp_ratio=1.0 / (KB_EV * 300.0),
                               req_integration_points=300.0, max_coll_before_ss=100.0, n_phases=16, max_seconds=300.0)


def _context(spec):
    from lokigpu import capi
    case, n_e, red_field, angle, freq, red_mag, seed = spec
    ps, arrays = _inputs(case)
    ctx = capi.Context(_config(n_e, seed))
    ctx.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
    ctx.set_conditions(N_GAS, 300.0, red_field, angle, freq, red_mag)
    return ctx


def _alone(specs, dists=False):
    out = []
    for spec in specs:
        ctx = _context(spec)
        r = ctx.solve()
        counts, rate, _, _ = ctx.process_results()
        out.append((r, counts, rate, ctx.distributions()) if dists else (r, counts, rate))
        ctx.close()
    return out


def _batched(specs, max_slots=64, schedule=None, dists=False):
    from lokigpu import capi
    b = capi.Batch(0, max_slots)
    if schedule is not None:
        b.set_schedule(*schedule)
    ctxs = [_context(s) for s in specs]
    for c in ctxs:
        b.add(c)
    res, st, rep = b.run()
    out = []
    for c, r, s in zip(ctxs, res, st):
        assert s == 0, c.last_error()
        counts, rate, _, _ = c.process_results()
        out.append((r, counts, rate, c.distributions()) if dists else (r, counts, rate))
        c.close()
    b.close()
    return out, rep


def _drift_axis(spec):
    # the field axis: z at 180 degrees, x at 90 degrees (BoltzmannMC.C:465-474)
    return 2 if spec[3] == 180.0 else 0


def _statistically_equal(spec, a, b):
    ra, ca, qa = a
    rb, cb, qb = b
    fails = []
    k = _drift_axis(spec)
    for label, va, ea, vb, eb in [("mean energy", ra.mean_energy, ra.mean_energy_err, rb.mean_energy, rb.mean_energy_err),
                                  ("flux v", ra.flux_v[k], ra.flux_v_err[k], rb.flux_v[k], rb.flux_v_err[k])]:
        tol = max(4.0 * np.hypot(ea, eb), 0.01 * abs(va))
        if abs(va - vb) > tol:
            fails.append(f"{spec}: {label} {va:.6g} +- {ea:.3g} vs {vb:.6g} +- {eb:.3g}")
    for p in range(len(qa)):
        if ca[p] < 2000 or cb[p] < 2000:
            continue
        rel = 2.0 * 5.0 * np.sqrt(1.0 / ca[p] + 1.0 / cb[p]) + 0.02
        if abs(qb[p] / qa[p] - 1.0) > rel:
            fails.append(f"{spec}: rate[{p}] {qa[p]:.6g} vs {qb[p]:.6g} (counts {ca[p]}, {cb[p]})")
    return fails


@pytest.fixture(scope="module")
def mix_alone():
    return _alone(MIX)


def test_batch_repeats_alone_without_ionization():
    alone = _alone(ATOMIC)
    batched, rep = _batched(ATOMIC)
    assert rep.intervals > 0 and rep.kernel_launches > 0 and rep.electron_steps > 0
    for spec, (ra, ca, _), (rb, cb, _) in zip(ATOMIC, alone, batched):
        assert ra.capped == 0 and rb.capped == 0
        assert rb.sync_steps == ra.sync_steps, spec
        k = _drift_axis(spec)
        tol = 1e-4 if spec[4] == 0.0 else 1e-3  # DC and crossed B / AC
        assert abs(rb.real_collisions / ra.real_collisions - 1.0) < tol, spec
        assert abs(rb.null_collisions / ra.null_collisions - 1.0) < tol, spec
        big = ca > 10000
        assert np.all(np.abs(cb[big] / ca[big].astype(float) - 1.0) < 10 * tol), spec
        assert abs(rb.mean_energy / ra.mean_energy - 1.0) < tol, spec
        assert abs(rb.flux_v[k] / ra.flux_v[k] - 1.0) < tol, spec
        if spec[4] == 0.0:
            assert abs(rb.bulk_v[k] / ra.bulk_v[k] - 1.0) < 1e-3, spec


# pinned schedules: (launch shape, collision-turn threshold, coarse null test);
# shape 4 parks pending collisions in a per-warp stash
SCHEDULES = [(0, 20, 1), (1, 12, 0), (2, 28, 1), (3, 16, 1), (4, 20, 1), (4, 20, 0), (5, 20, 1)]


@pytest.mark.parametrize("schedule", SCHEDULES, ids=[f"shape{s}_t{t}_c{c}" for s, t, c in SCHEDULES])
def test_every_schedule_repeats_the_solve_alone(schedule):
    """The schedule (launch shape, the stash, the collision-turn threshold,
    the staging of the null test) changes no electron's draws, decisions or
    roundings: the batched solve in any schedule makes the collisions of the
    solve alone, bit for bit (DC, crossed B, AC). The distributions too: the
    batch counts each sample's EEDF, EADF (and EVDF) as the next interval's
    advance loads the electrons, the solve alone with its own passes over
    the ensemble, and the counts agree exactly."""
    specs = [ATOMIC[1], ATOMIC[2], ATOMIC[3]]
    alone = _alone(specs, dists=True)
    batched, rep = _batched(specs, schedule=schedule, dists=True)
    assert rep.advance_stash == (64.0 if schedule[0] >= 4 else 0.0)
    assert rep.real_batch == (32.0 if schedule[0] >= 4 else schedule[1])
    assert rep.coarse_null_test == schedule[2]
    for spec, (ra, ca, _, da), (rb, cb, _, db) in zip(specs, alone, batched):
        # every kernel rounds every step alike: the same collisions, bit for
        # bit; the swarm parameters to the grouping of the moment sums (the
        # single-condition and the batched sample passes add their per-thread
        # partial sums in different groups: ~1e-9)
        assert rb.sync_steps == ra.sync_steps, spec
        assert ra.integration_points > 0, spec
        for key in ("eedf", "eadf", "evdf", "eedf_periodic"):
            if key in da:
                assert np.array_equal(da[key], db[key], equal_nan=True), (spec, key)
        assert np.array_equal(ca, cb), spec
        assert rb.real_collisions == ra.real_collisions and rb.null_collisions == ra.null_collisions, spec
        assert abs(rb.mean_energy / ra.mean_energy - 1.0) < 1e-8, spec
        k = _drift_axis(spec)
        assert abs(rb.flux_v[k] / ra.flux_v[k] - 1.0) < 1e-8, spec


@pytest.mark.parametrize("gte", [1, 2], ids=["thermal", "smart"])
def test_stash_repeats_the_warp_turn_shape_with_thermal_targets(gte):
    """With thermal targets every trial event goes through the collision turn
    (BoltzmannMC.C:916-1031): in the stash shape every one is parked in the
    stash. Without ionization and attachment the stash shape and the
    warp-turn shape give the same collision counts and swarm parameters, bit
    for bit (the device code rounds every step alike in every shape)."""
    from lokigpu import capi
    spec = ("atomic", 30000, 20.0, 180.0, 0.0, 0.0, 71)
    out = []
    for shape in (0, 4, 5):
        b = capi.Batch(0, 4)
        b.set_schedule(shape, 20, 1)
        case, n_e, red_field, angle, freq, red_mag, seed = spec
        ps, arrays = _inputs(case)
        cfg = _config(n_e, seed)
        cfg.gas_temperature_effect = gte
        ctx = capi.Context(cfg)
        ctx.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
        ctx.set_conditions(N_GAS, 300.0, red_field, angle, freq, red_mag)
        b.add(ctx)
        res, st, rep = b.run()
        assert st[0] == 0 and rep.advance_stash == (64.0 if shape >= 4 else 0.0)
        counts = ctx.process_results()[0]
        out.append((res[0], counts))
        ctx.close()
        b.close()
    ra, ca = out[0]
    for rb, cb in out[1:]:
        assert np.array_equal(ca, cb)
        assert ra.real_collisions == rb.real_collisions and ra.null_collisions == rb.null_collisions
        assert ra.mean_energy == rb.mean_energy and ra.flux_v[2] == rb.flux_v[2]


def test_schedule_rejects_unknown_points():
    from lokigpu import capi
    b = capi.Batch(0, 4)
    for bad in [(6, 20, 1), (0, 13, 1), (0, 20, 2)]:
        with pytest.raises(capi.LokiGpuError):
            b.set_schedule(*bad)
    b.set_schedule(4, 0, 1)  # a stash shape ignores the threshold
    b.set_schedule(-1, 0, 0)  # back to on-line tuning
    b.close()


def test_stash_schedule_matches_alone_with_ionization_and_attachment(mix_alone):
    batched, rep = _batched(MIX, schedule=(4, 20, 1))
    assert rep.advance_stash == 64.0 and rep.secondaries > 0 and rep.attached > 0
    fails = []
    for spec, a, b in zip(MIX, mix_alone, batched):
        assert b[0].capped == 0 and b[0].integration_points >= 300
        fails += _statistically_equal(spec, a, b)
    assert not fails, "\n".join(fails)


def test_batch_matches_alone_with_ionization_and_attachment(mix_alone):
    batched, rep = _batched(MIX)
    fails = []
    for spec, a, b in zip(MIX, mix_alone, batched):
        assert b[0].capped == 0 and b[0].integration_points >= 300
        fails += _statistically_equal(spec, a, b)
    assert not fails, "\n".join(fails)


def test_batch_with_fewer_slots_than_contexts(mix_alone):
    # two slots for four contexts: the last two start as the first ones finish
    batched, rep = _batched(MIX, max_slots=2)
    fails = []
    for spec, a, b in zip(MIX, mix_alone, batched):
        fails += _statistically_equal(spec, a, b)
    assert not fails, "\n".join(fails)


def test_server_jobs_arriving_while_others_run(mix_alone):
    from lokigpu import capi
    srv = capi.Server(0, 16)
    ids = []
    for spec in MIX:
        case, n_e, red_field, angle, freq, red_mag, seed = spec
        ps, arrays = _inputs(case)
        ids.append(srv.submit(_config(n_e, seed), ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"],
                              N_GAS, 300.0, red_field, angle, freq, red_mag))
        time.sleep(0.02)  # later jobs join a batch already on the device
    fails = []
    starts, ends = [], []
    for spec, jid, a in zip(MIX, ids, mix_alone):
        st = srv.wait(jid, 600.0)
        assert st.state == capi.JOB_DONE, (spec, st.status, srv.last_error())
        assert st.submit_time <= st.start_time <= st.end_time
        starts.append(st.start_time)
        ends.append(st.end_time)
        ps, _ = _inputs(spec[0])
        counts, rate = srv.rates(jid, ps.n)
        fails += _statistically_equal(spec, a, (st.result, counts, rate))
    rep = srv.report()
    srv.stop()
    assert not fails, "\n".join(fails)
    assert rep.completed == len(MIX) and rep.failed == 0 and rep.intervals > 0
    # the work overlapped: two jobs were on the device at the same time
    assert any(starts[i] < ends[j] and starts[j] < ends[i] for i in range(len(ids)) for j in range(i))


def test_server_admits_by_memory_footprint():
    from lokigpu import capi
    spec = ("atomic", 10000, 100.0, 180.0, 0.0, 0.0, 5)
    ps, arrays = _inputs("atomic")
    cfg = _config(10000, 5)
    cfg.req_integration_points = 100.0
    probe = capi.Server(0, 4)
    jid = probe.submit(cfg, ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"], N_GAS, 300.0, 100.0)
    fp = probe.wait(jid, 300.0).footprint_bytes
    probe.stop()
    assert fp > 10000 * 64
    srv = capi.Server(0, 4, memory_budget_bytes=1.5 * fp)  # one job at a time
    ids = [srv.submit(cfg, ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"], N_GAS, 300.0, 100.0)
           for _ in range(3)]
    big = capi.default_config(**{k: getattr(cfg, k) for k, _ in capi.Config._fields_})
    big.n_electrons = 1e6  # larger than the whole budget
    big_id = srv.submit(big, ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"], N_GAS, 300.0, 100.0)
    sts = [srv.wait(j, 300.0) for j in ids]
    st_big = srv.wait(big_id, 300.0)
    srv.stop()
    assert all(s.state == capi.JOB_DONE for s in sts)
    for s0, s1 in zip(sts, sts[1:]):
        assert s1.start_time >= s0.end_time - 1e-6  # never two at once
    assert st_big.state == capi.JOB_FAILED and st_big.status == 2  # LGPU_ERR_OOM


def test_batch_and_server_with_different_mixtures():
    # each slot carries its own process set, tables and gases: a block that
    # moves between slots reloads them
    from lokigpu import capi
    alone = _alone(MIXTURES)
    batched, rep = _batched(MIXTURES)
    fails = []
    for spec, a, b in zip(MIXTURES, alone, batched):
        fails += _statistically_equal(spec, a, b)
    srv = capi.Server(0, 8)
    ids = []
    for spec in MIXTURES:
        case, n_e, red_field, angle, freq, red_mag, seed = spec
        ps, arrays = _inputs(case)
        ids.append(srv.submit(_config(n_e, seed), ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"],
                              N_GAS, 300.0, red_field, angle, freq, red_mag))
    for spec, jid, a in zip(MIXTURES, ids, alone):
        st = srv.wait(jid, 600.0)
        assert st.state == capi.JOB_DONE, (spec, st.status, st.error)
        ps, _ = _inputs(spec[0])
        counts, rate = srv.rates(jid, ps.n)
        fails += _statistically_equal(spec, a, (st.result, counts, rate))
    srv.stop()
    assert not fails, "\n".join(fails)


def test_server_forgets_finished_jobs():
    """A long-running server drops the records of finished jobs on request
    (lgpu_server_forget) and recycles the batch's bookkeeping of finished
    jobs, so many small jobs in a row run through a few slots."""
    from lokigpu import capi
    ps, arrays = _inputs("atomic")
    cfg = _config(4096, 7)
    cfg.req_integration_points = 50.0
    cfg.max_coll_before_ss = 20.0
    srv = capi.Server(0, 3)
    ids = [srv.submit(cfg, ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"], N_GAS, 300.0,
                      100.0 + k) for k in range(24)]
    with pytest.raises(capi.LokiGpuError) as e:  # not finished yet: still queued
        srv.forget(ids[-1])
    assert e.value.code == 6
    sts = [srv.wait(j, 300.0) for j in ids]
    assert all(s.state == capi.JOB_DONE for s in sts), [(s.state, s.error) for s in sts]
    counts, rate = srv.rates(ids[0], ps.n)
    assert counts.sum() > 0
    for j in ids[:12]:
        srv.forget(j)
    with pytest.raises(capi.LokiGpuError):
        srv.poll(ids[0])
    assert srv.poll(ids[12]).state == capi.JOB_DONE
    rep = srv.report()
    srv.stop()
    assert rep.completed == 24 and rep.running == 0 and rep.queued == 0


def test_autotuner_picks_a_launch_shape_and_keeps_it_per_mixture():
    """The batch tunes the advance's launch shape, then the collision-turn
    threshold and the table staging, and keeps the choice for the mixture: a
    second batch of the same mixture starts tuned."""
    from lokigpu import capi
    ps, arrays = _inputs("atomic")

    def batch_of(seed0):
        b = capi.Batch(0, 4)
        ctxs = []
        for k in range(3):
            cfg = _config(20000, seed0 + k)
            cfg.req_integration_points = 1e9  # timed intervals only
            c = capi.Context(cfg)
            c.set_processes(ps, arrays["gas_first"], arrays["gas_last"], arrays["gas_frac"])
            c.set_conditions(N_GAS, 300.0, 60.0 + 20.0 * k)
            b.add(c)
            ctxs.append(c)
        b.start()
        return b, ctxs

    b, ctxs = batch_of(100)
    _, rep = b.step(60)  # 6 shapes x 3 rounds, then 10 (stash: 2) candidates x 3 rounds
    assert rep.advance_threads in (256.0, 512.0) and rep.advance_chunk in (64.0, 128.0, 256.0)
    assert rep.advance_stash in (0.0, 64.0)
    assert rep.real_batch in ((32.0,) if rep.advance_stash else (12.0, 16.0, 20.0, 24.0, 28.0))
    assert rep.coarse_null_test in (0.0, 1.0)
    first = (rep.advance_threads, rep.advance_blocks_per_sm, rep.advance_chunk, rep.advance_stash, rep.real_batch,
             rep.coarse_null_test)
    b.close()
    for c in ctxs:
        c.close()
    b, ctxs = batch_of(200)
    _, rep = b.step(1)
    assert (rep.advance_threads, rep.advance_blocks_per_sm, rep.advance_chunk, rep.advance_stash, rep.real_batch,
            rep.coarse_null_test) == first
    b.close()
    for c in ctxs:
        c.close()


def test_server_admits_requests_from_input_files(tmp_path):
    """A request written as for the reference (a setup file with a vector of
    E/N and its LXCat file, parsed by lgpu_request_parse) runs one job per
    entry, each equal to the job submitted from the flattened arrays: the
    inputs are the same bits, so without ionization and attachment the
    collision counts agree exactly."""
    import os

    from lokigpu import capi, synth

    gas = synth.atomic_gas()
    synth.write_case(str(tmp_path), [gas], pressure_pa=N_GAS * 1.38064852e-23 * 300.0, red_field=[80.0, 120.0],
                     n_electrons=20000, kte_init_ev=1.0,
                     extra_numerics={"nIntegrationPoints": "500", "nInterpPoints": "2000",
                                     "maxCollisionsBeforeSteadyState": "100", "gpuSeed": "77"})
    inp = os.path.join(str(tmp_path), "Input")
    req = capi.Request(open(os.path.join(inp, "case.in")).read(),
                       {"A1_LXCat.txt": open(os.path.join(inp, "A1_LXCat.txt")).read()})
    assert len(req) == 2
    srv = capi.Server(0, 4)
    ids = srv.submit_request(req)
    ps = synth.flatten([gas])
    cfg = req.job(0).config
    ids2 = [srv.submit(cfg, ps, ps.gas_first, ps.gas_last, ps.gas_fraction, req.job(k).conditions.gas_density,
                       300.0, (80.0, 120.0)[k]) for k in range(2)]
    a = [srv.wait(j, 300.0) for j in ids]
    b = [srv.wait(j, 300.0) for j in ids2]
    srv.stop()
    for x, y in zip(a, b):
        assert x.state == capi.JOB_DONE and y.state == capi.JOB_DONE
        assert x.result.real_collisions == y.result.real_collisions
        assert x.result.mean_energy == y.result.mean_energy


def test_server_postprocesses_the_eedf_of_a_request(tmp_path):
    """A request's jobs carry the collisions behind their processes
    (lgpu_job.twoterm), and the server runs the end-of-job EEDF
    post-processing on the device as each job finishes
    (lgpu_server_job_eedf): the same values as the same job's context
    post-processing its own EEDF after a solve alone (without ionization and
    attachment the two runs' EEDF histograms hold the same counts). A job
    submitted without two-term inputs has none."""
    import os

    from lokigpu import capi, synth

    gas = synth.atomic_gas()
    synth.write_case(str(tmp_path), [gas], pressure_pa=N_GAS * 1.38064852e-23 * 300.0, red_field=[80.0],
                     n_electrons=20000, kte_init_ev=1.0,
                     extra_numerics={"nIntegrationPoints": "500", "nInterpPoints": "2000",
                                     "maxCollisionsBeforeSteadyState": "100", "gpuSeed": "77"})
    inp = os.path.join(str(tmp_path), "Input")
    req = capi.Request(open(os.path.join(inp, "case.in")).read(),
                       {"A1_LXCat.txt": open(os.path.join(inp, "A1_LXCat.txt")).read()})
    srv = capi.Server(0, 4)
    jid = srv.submit_request(req)[0]
    ps = synth.flatten([gas])
    j = req.job(0)
    plain = srv.submit(j.config, ps, ps.gas_first, ps.gas_last, ps.gas_fraction, j.conditions.gas_density, 300.0, 80.0)
    st = srv.wait(jid, 300.0)
    assert st.state == capi.JOB_DONE
    params, rates = srv.job_eedf(jid, ps.n)
    assert srv.wait(plain, 300.0).state == capi.JOB_DONE
    with pytest.raises(capi.LokiGpuError):
        srv.job_eedf(plain, ps.n)
    srv.stop()
    cfg = j.config
    ctx = capi.Context(cfg)
    ctx.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
    c = j.conditions
    ctx.set_conditions(c.gas_density, c.gas_temperature, c.reduced_field_td, c.field_angle_deg,
                       c.excitation_freq_hz, c.reduced_mag_field_hx)
    ctx.set_twoterm(req.twoterm(0))
    r = ctx.solve()
    assert r.real_collisions == st.result.real_collisions
    p2, r2 = ctx.eedf_postprocess()
    ctx.close()
    np.testing.assert_allclose(rates, r2, rtol=1e-13, atol=0)
    np.testing.assert_allclose(params.values(), p2.values(), rtol=1e-13, atol=1e-300)
    assert params.tot_ion_rate == 0.0 and params.mom_transf_freq > 0 and params.charac_energy > 0


def test_spilled_secondaries_in_every_shape():
    """Secondaries a warp cannot keep in its own queue go to the global spill
    buffer, which the drain launch pushes from their creation time
    (BoltzmannMC.C:1195-1272) before population control (:1282-1408). With
    the warp queue cut to one entry (lgpu_config.advance_queue) nearly every
    secondary of an ionization-dominated gas at 1000 Td takes that path; the
    warp-turn shape and the collision stash, both spilling, agree with the
    solve alone with the full queue."""
    from lokigpu import capi, synth

    # weak elastic scattering and a large ionization cross section
    gas = synth.atomic_gas()
    e = synth.log_grid(100)
    gas.collisions = [synth.Collision("Elastic", "A1(gnd)", "A1(gnd)", 0.0, e, np.full_like(e, 1e-21)),
                      synth.Collision("Ionization", "A1(gnd)", "A1(+)", 15.0, e, np.where(e < 15.0, 0.0, 1e-19))]
    gas.states = {"A1(gnd)": synth.State(1.0), "A1(+)": synth.State(0.0)}
    ps = synth.flatten([gas])

    def context(seed, queue):
        cfg = _config(200000, seed)
        cfg.req_integration_points = 500.0
        cfg.advance_queue = queue
        c = capi.Context(cfg)
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, 300.0, 1000.0)
        return c

    out = []
    for shape in (0, 4, 5):
        b = capi.Batch(0, 2)
        b.set_schedule(shape, 20, 1)
        c = context(91, 1)
        b.add(c)
        res, st, rep = b.run()
        assert st[0] == 0, c.last_error()
        assert rep.spilled > 0.5 * rep.secondaries > 0, (shape, rep.secondaries, rep.spilled)
        counts, rate, _, _ = c.process_results()
        out.append((res[0], counts, rate))
        c.close()
        b.close()
    c = context(92, 0)
    r = c.solve()
    counts, rate, _, _ = c.process_results()
    out.append((r, counts, rate))
    c.close()
    spec = ("ion", 200000, 1000.0, 180.0, 0.0, 0.0, 91)
    for rb in out[:3]:
        fails = _statistically_equal(spec, out[3], rb)
        assert not fails, fails


def test_secondary_buffers_grow_with_long_intervals():
    """With synchronisation intervals of 6 trial collisions per electron
    (synchronizationTimeXMaxCollisionFrequency = 6, BoltzmannMC.C:622) an
    ionizing gas at 1000 Td makes about as many secondaries in one interval as
    the ensemble holds electrons, where the reference's list of secondaries
    just grows (BoltzmannMC.C:1195-1272). The buffers start at twice the ensemble
    and grow ahead of need between intervals (each time an interval fills a
    quarter of them): the solve alone and the batched solve both finish, and
    agree."""
    from lokigpu import capi, synth

    gas = synth.atomic_gas()
    e = synth.log_grid(120, 1e-3, 1e5)
    gas.collisions = [synth.Collision("Elastic", "A1(gnd)", "A1(gnd)", 0.0, e, np.full_like(e, 1e-21)),
                      synth.Collision("Ionization", "A1(gnd)", "A1(+)", 15.0, e, np.where(e < 15.0, 0.0, 1e-20))]
    gas.states = {"A1(gnd)": synth.State(1.0), "A1(+)": synth.State(0.0)}
    ps = synth.flatten([gas])
    n = 20000

    def context(seed):
        cfg = _config(n, seed)
        cfg.sync_x = 6.0
        cfg.req_integration_points = 100.0
        c = capi.Context(cfg)
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, 300.0, 1000.0)
        return c

    c = context(93)
    ra = c.solve()
    counts_a, rate_a, _, _ = c.process_results()
    c.close()
    b = capi.Batch(0, 2)
    c = context(94)
    b.add(c)
    res, st, rep = b.run()
    assert st[0] == 0, c.last_error()
    # on average past a quarter of the first buffers (2 n records) per
    # interval, so they grew at least once
    assert rep.secondaries / rep.intervals > n / 2, (rep.secondaries, rep.intervals)
    counts_b, rate_b, _, _ = c.process_results()
    c.close()
    b.close()
    spec = ("ion", n, 1000.0, 180.0, 0.0, 0.0, 93)
    fails = _statistically_equal(spec, (ra, counts_a, rate_a), (res[0], counts_b, rate_b))
    assert not fails, fails
