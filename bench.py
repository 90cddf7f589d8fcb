#!/usr/bin/env python3
"""Benchmark of the electron Monte Carlo hot path on GB300.

Default workload (--workload sweep): the 64-point E/N sweep. E/N log-spaced
1..1000 Td over the synthetic N2-like gas mixed 80/20 with the synthetic
O2-like gas (65 processes: ionization in both gases, dissociative attachment
at 4.4 eV; 200-point log grids over 1e-3..1e4 eV), N = 3.22e22 m^-3, cold gas, uneven electron counts per condition
(seeded log-uniform 1e4..2e6, 1.98e7 in all), FP32 push with FP64 tallies.
Three forms of the same work are measured:

* batched: all 64 conditions in one lgpu_batch - one launch sequence (CUDA
  graph) per synchronisation interval advances every condition;
* plain: one condition per launch sequence (lgpu_solve / lgpu_advance), the
  drop-in path, one condition after the other;
* served: the 64 conditions submitted to lgpu_server with Poisson arrivals,
  admitted by device footprint as they arrive (continuous batching).

`value` is real collisions per second of the batched form over K timed
intervals of all 64 conditions (after R relaxation intervals and W warm-up
intervals; each timed interval is bracketed by CUDA events on the batch's
stream and preceded by a 256 MiB L2 flush outside the timed region). The plain
form is timed the same way per condition (plain.value). `e2e` is the whole
sweep solved to convergence (mean-energy standard error below 0.5%) through
the C ABI from host arrays: contexts created, processes uploaded, solved,
results and rate coefficients read back; the same for the plain form
(plain.e2e) and the served form with its p50/p99 request latency.

--workload n2_200td keeps the single-condition line: the synthetic N2-like gas
at DC 200 Td with 1e6 electrons, one plain interval per step.

--workload serve runs a request stream through lgpu_server: seeded requests of
1-5 random gases (10-40 processes on 100-400-point grids), E/N 1..1000 Td, DC,
crossed B or AC, 1e4..4e6 electrons, Poisson arrivals; each converged to 0.5 %
mean-energy error; p50/p99 latency and throughput, and the plain path on the
first requests.

--impl reference times the CPU implementation of the same path on the host
cores (the C restatement of the reference's algorithm, oracle/) on a bounded
sample of the same workload: the sweep's 64 conditions with their electron
counts, one single-threaded condition per core at a time (a sweep's best use
of a CPU), real collisions summed over time weighted by each condition's
electrons.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "loki-mc_gb300", "python"))

METRIC = "real collisions/s, batched+served vs plain, 1 GB300; sweep p50/p99 at <0.5% err"
UNIT = "collisions/s"
N_GAS = 3.22e22
T_GAS = 300.0
KT_INIT = 1.0 / (8.617333262e-5 * T_GAS)  # start Maxwellian at kT = 1 eV
STATE_BYTES_PER_ELECTRON_STEP = 64  # 32 B state read + 32 B written per electron per interval

# single-condition workload
E_N = 200.0
N_ELECTRONS = 1_000_000
# DRAM bytes per electron and interval of k_advance, from one ncu capture of the
# same kernel on 4e6 electrons (N2-like gas, DC 200 Td): 130.5 MB read +
# 73.8 MB written; traffic grows in proportion to the electrons advanced
DRAM_BYTES_PER_ELECTRON_STEP = (130.522112e6 + 73.842176e6) / 4.0e6

# DRAM bytes per electron and interval of the batched advance (DC launch, the
# collision-stash shape the tuner picks, 512 x 2), from one ncu capture of the
# sweep (the 41st interval, schedule 5,20,1): 888.3 MB read + 560.6 MB written
# for 1.98e7 electrons
SWEEP_DRAM_BYTES_PER_ELECTRON_STEP = (888.269312e6 + 560.615424e6) / 19795598

# sweep workload
SWEEP_POINTS = 64
SWEEP_SEED = 2024
SWEEP_NE_RANGE = (1e4, 2e6)
SWEEP_ERR = 0.005            # mean-energy relative standard error at convergence
SWEEP_SS_CAP = 50.0          # maxCollisionsBeforeSteadyState (x nElectrons)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()), default=None)
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.rows)}


# ------------------------------------------------------------------ workloads
def n2_processes():
    from lokigpu import synth

    return synth.flatten([synth.n2_like_gas()])


def sweep_processes():
    from lokigpu import synth

    # cross sections to 1e4 eV: at 1000 Td the electrons pass 1 keV, where tables
    # ending at 1e3 eV stop the solve (BoltzmannMC.C:1426-1430)
    return synth.flatten([synth.n2_like_gas(fraction=0.8, e_max=1e4), synth.o2_like_gas(fraction=0.2, e_max=1e4)])


def sweep_conditions():
    """(E/N in Td, electrons, field angle, frequency in Hz, B/N in Hx) of the
    64 sweep points: DC at 180 degrees."""
    import numpy as np

    en = np.logspace(0.0, 3.0, SWEEP_POINTS)
    rng = np.random.default_rng(SWEEP_SEED)
    lo, hi = np.log10(SWEEP_NE_RANGE[0]), np.log10(SWEEP_NE_RANGE[1])
    ne = np.round(10.0 ** rng.uniform(lo, hi, SWEEP_POINTS)).astype(int)
    return [(float(e), int(n), 180.0, 0.0, 0.0) for e, n in zip(en, ne)]


FIELD_ELECTRONS = 500_000
FIELD_PHASES = 64
PHASES = 100  # phase bins of the running workload's AC conditions (set by main)


def field_conditions():
    """The field-complex batch: the sweep's mixture at DC 100 Td with a crossed
    magnetic field (E at 90 degrees to B along z), B/N 0..2000 Hx in 16 steps,
    and an AC field of 150 Td rms at omega/N 1e-18..1e-14 m^3/s (16 log
    steps, 64 phase bins); 5e5 electrons each."""
    import numpy as np

    b = [(100.0, FIELD_ELECTRONS, 90.0, 0.0, float(x)) for x in np.linspace(0.0, 2000.0, 16)]
    ac = [(150.0, FIELD_ELECTRONS, 180.0, float(w * N_GAS / (2.0 * np.pi)), 0.0) for w in np.logspace(-18.0, -14.0, 16)]
    return b + ac


def sweep_config(capi, device, n_e, seed, converge, phases=100):
    """Numerics of a sweep condition: converged means the reference's stop
    criteria with relError meanEnergy 0.5% (BoltzmannMC.C:1743-1767), else a
    context that never stops by itself (timed intervals)."""
    kw = dict(device=device, seed=seed, n_electrons=float(n_e), n_interp=10000, init_temp_ratio=KT_INIT,
              n_phases=phases)
    if converge:
        kw.update(errors_checked=1, req_err_mean_energy=SWEEP_ERR, req_integration_points=200.0,
                  max_coll_before_ss=SWEEP_SS_CAP, max_seconds=300.0)
    else:
        kw.update(req_integration_points=1e15)
    return capi.default_config(**kw)


# --------------------------------------------------------------------- CPU arm
def _oracle_arrays(ps):
    import numpy as np

    off = np.concatenate([[0], np.cumsum([len(e) for e in ps.raw_e])]).astype(np.int32)
    return dict(ptype=ps.ptype, is_super=ps.is_super, sampler=ps.sampler, sampler_p0=ps.sampler_p0,
                sampler_p1=ps.sampler_p1, superw=ps.superw, emin=ps.emin, emax=ps.emax, rel_dens=ps.rel_dens,
                mass=ps.mass, red_mass=ps.red_mass, eloss=ps.eloss, wparam=ps.wparam, raw_off=off[:-1],
                raw_len=np.array([len(e) for e in ps.raw_e], np.int32), raw_e=np.concatenate(ps.raw_e),
                raw_v=np.concatenate(ps.raw_v), gas_first=ps.gas_first, gas_last=ps.gas_last,
                gas_frac=ps.gas_fraction, energy_max_elastic=ps.energy_max_elastic)


def cpu_condition(job):
    """One condition on one host core: the CPU restatement of the reference's
    path (oracle/) with `n` electrons started at kT = 1 eV, for `seconds` of
    wall time; the second half is measured. Returns (electrons of the
    condition in the workload, measured electron-intervals, real collisions,
    seconds)."""
    workload, (td, n_cfg, angle, freq, red_mag), n, seconds, seed = job
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "loki-mc_gb300", "python"))
    import oracle as O

    import math

    ps = n2_processes() if workload == "n2_200td" else sweep_processes()
    pr = O.OracleProcs(_oracle_arrays(ps), 10000)
    # the field of BoltzmannMC.C:463-485: E at `angle` to z, sqrt(2) x rms for AC,
    # cyclotron frequency e B / m with B = (B/N) N (1 Hx = 1e-27 T m^3)
    e_abs = td * 1e-21 * N_GAS * (math.sqrt(2.0) if freq else 1.0)
    E = (0.0, 0.0, -e_abs) if angle == 180.0 else (e_abs * math.sin(math.radians(angle)), 0.0,
                                                   e_abs * math.cos(math.radians(angle)))
    f = O.make_fields(N_GAS, T_GAS, E=E, freq_hz=freq, red_mag=red_mag,
                      omega_c=1.6021766208e-19 * red_mag * 1e-27 * N_GAS / 9.10938356e-31)
    cfg = O.default_run_config(n, n_threads=1, seed=seed, max_seconds=seconds, mark_seconds=0.5 * seconds,
                               req_integration_points=1e12, init_temp_ratio=KT_INIT)
    _, res, _ = O.run(pr, f, cfg)
    if res.mark_elapsed <= 0:
        return n_cfg, 0.0, 0.0, 0.0
    steps = res.sync_steps - res.mark_sync_steps
    return n_cfg, float(n * steps), res.real_collisions - res.mark_real_collisions, res.elapsed - res.mark_elapsed


def cpu_sweep_rate(samples, cores):
    """Real collisions per second of the whole workload on `cores` host cores
    running one condition each: every condition advances its electrons
    (n_cfg) each interval; a core spends n_cfg x (seconds per
    electron-interval) on it and finds n_cfg x (real collisions per
    electron-interval)."""
    real_sum = sum(n_cfg * real / el for n_cfg, el, real, _ in samples if el > 0)
    time_sum = sum(n_cfg * secs / el for n_cfg, el, _, secs in samples if el > 0)
    return cores * real_sum / time_sum if time_sum > 0 else 0.0


def cpu_sample(seconds: float, cores: int, workload: str, offset: int = 0, max_electrons: int = 10_000):
    """Times the CPU restatement of the reference's path on the host cores on
    a bounded sample of the workload. Sweep: the same 64 conditions (E/N and
    electron counts) one per core at a time, each single-threaded for
    `seconds` (as a sweep runs best on a CPU: one setup per condition and
    core), with up to `max_electrons` electrons; a round takes the next `cores`
    conditions from `offset`. n2_200td: the single condition on one core per
    sample. Returns (real collisions/s of the workload, description, cores,
    samples)."""
    import multiprocessing as mp

    if workload in ("sweep", "field"):
        conds = sweep_conditions() if workload == "sweep" else field_conditions()
        picks = [conds[(offset + k) % len(conds)] for k in range(cores)]
    else:
        picks = [(E_N, N_ELECTRONS, 180.0, 0.0, 0.0)] * cores
    jobs = [(workload, cond, min(cond[1], max_electrons), seconds, 3 + offset + k) for k, cond in enumerate(picks)]
    with mp.get_context("spawn").Pool(cores) as pool:
        samples = pool.map(cpu_condition, jobs)
    what = {"sweep": "the sweep's 64 conditions", "field": "the field-complex batch's 32 conditions"}.get(
        workload, "the N2-like gas at 200 Td")
    desc = (f"{what}, {len(jobs)} conditions per round on {cores} cores (one single-threaded run each, up to "
            f"{max_electrons} electrons from kT = 1 eV, {seconds:.1f} s of which the second half is measured), "
            f"weighted by the workload's electron counts; C restatement of the reference path")
    return cpu_sweep_rate(samples, cores), desc, cores, samples


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    t0 = time.time()
    per_step = max(2.0, min(8.0, 150.0 / max(1, args.steps + args.warmup)))
    samples, desc = [], ""
    for i in range(args.warmup + args.steps):
        _, desc, _, smp = cpu_sample(per_step, cores, args.workload, offset=i * cores)
        if i >= args.warmup:
            samples += smp
    v = cpu_sweep_rate(samples, cores)
    workload = {"sweep": "sweep64_n2o2_1-1000Td", "field": "field32_n2o2_crossedB_AC"}.get(
        args.workload, "n2_like_dc200Td_1e6e")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * (time.time() - t0) / (args.steps + args.warmup),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload, "conditions": {"sweep": 64, "field": 32}.get(args.workload, 1),
                       "impl_detail": "C restatement of the reference path (oracle/), one condition per core"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------- GPU arms
def aggregate_ranks(total_ms, real, null, device):
    """Replicas only: every rank advances its own ensembles; the job time is
    the slowest rank's, the collisions are summed over ranks."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    c = torch.tensor([real, null], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t[0]), float(c[0]), float(c[1])


def _init_ranks():
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    return int(os.environ.get("RANK", "0")), world, local


def _percentile(xs, q):
    import numpy as np

    return float(np.percentile(np.asarray(xs, dtype=np.float64), q)) if len(xs) else None


def _sweep_timed_batched(capi, ps, conds, local, rank, args, flush):
    """value: K timed batched intervals of all conditions, after relaxation."""
    import torch

    b = capi.Batch(local, len(conds))
    ctxs = []
    for i, (en, ne, ang, fr, bm) in enumerate(conds):
        c = capi.Context(sweep_config(capi, local, ne, 5000 + 100 * rank + i, converge=False, phases=PHASES))
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, T_GAS, en, ang, fr, bm)
        b.add(c)
        ctxs.append(c)
    if args.schedule:
        b.set_schedule(*(int(x) for x in args.schedule.split(",")))
    b.start()
    b.step(args.relax)
    for _ in range(args.warmup):
        flush.add_(1.0)
        torch.cuda.synchronize()
        b.step(1)
    stream = torch.cuda.ExternalStream(b.stream(), device=local)
    total_ms = real = null = adv_ms = steps = 0.0
    launches = intervals = 0
    h2d = d2h = host_ms = secondaries = spilled = regrids = 0.0
    real_batch = 0
    coarse = -1
    shape = (0, 0, 0)
    for _ in range(args.steps):
        flush.add_(1.0)                    # L2 flush (256 MiB written), outside the timed region
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        running, rep = b.step(1)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        real += rep.real_collisions
        null += rep.null_collisions
        adv_ms += rep.advance_ms
        steps += rep.electron_steps
        launches += rep.kernel_launches
        intervals += rep.intervals
        h2d += rep.h2d_bytes
        d2h += rep.d2h_bytes
        host_ms += rep.host_ms
        secondaries += rep.secondaries
        spilled += rep.spilled
        regrids += rep.regrids
        assert running == len(conds)
        real_batch = rep.real_batch
        coarse = rep.coarse_null_test
        shape = (rep.advance_threads, rep.advance_blocks_per_sm, rep.advance_chunk, rep.advance_stash)
    del b
    for c in ctxs:
        c.close()
    return dict(total_ms=total_ms, real=real, null=null, adv_ms=adv_ms, electron_steps=steps, launches=launches,
                intervals=intervals, h2d=h2d, d2h=d2h, host_ms=host_ms, secondaries=secondaries, spilled=spilled,
                real_batch=real_batch, coarse=coarse, regrids=regrids, shape=shape)


def _sweep_timed_plain(capi, ps, conds, local, rank, args, flush):
    """plain.value: the same number of timed intervals per condition, one
    condition per launch sequence."""
    import torch

    total_ms = real = null = 0.0
    for i, (en, ne, ang, fr, bm) in enumerate(conds):
        c = capi.Context(sweep_config(capi, local, ne, 5000 + 100 * rank + i, converge=False, phases=PHASES))
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, T_GAS, en, ang, fr, bm)
        c.init_ensemble()
        c.advance(args.relax)
        flush.add_(1.0)
        torch.cuda.synchronize()
        c.advance(1)
        stream = torch.cuda.ExternalStream(c.stream(), device=local)
        r0 = c.advance(0)
        for _ in range(args.plain_steps):
            flush.add_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            c.advance(1)
            e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
        r1 = c.advance(0)
        real += r1.real_collisions - r0.real_collisions
        null += r1.null_collisions - r0.null_collisions
        c.close()
    return dict(total_ms=total_ms, real=real, null=null)


def _sweep_e2e_batched(capi, ps, conds, local, rank):
    import torch

    torch.cuda.synchronize()
    w0 = time.perf_counter()
    b = capi.Batch(local, len(conds))
    ctxs = []
    for i, (en, ne, ang, fr, bm) in enumerate(conds):
        c = capi.Context(sweep_config(capi, local, ne, 7000 + 100 * rank + i, converge=True, phases=PHASES))
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, T_GAS, en, ang, fr, bm)
        b.add(c)
        ctxs.append(c)
    res, st, rep = b.run()
    rates = [c.process_results()[:2] for c in ctxs]
    w1 = time.perf_counter()
    for c in ctxs:
        c.close()
    del b
    return dict(wall=w1 - w0, results=res, status=st, rates=rates, report=rep)


def _sweep_e2e_plain(capi, ps, conds, local, rank):
    import torch

    torch.cuda.synchronize()
    w0 = time.perf_counter()
    res, rates, h2d, d2h, steps = [], [], 0.0, 0.0, 0
    for i, (en, ne, ang, fr, bm) in enumerate(conds):
        c = capi.Context(sweep_config(capi, local, ne, 7000 + 100 * rank + i, converge=True, phases=PHASES))
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, T_GAS, en, ang, fr, bm)
        r = c.solve()
        rates.append(c.process_results()[:2])
        tm = c.timing()
        h2d += tm.h2d_bytes
        d2h += tm.d2h_bytes
        steps += r.sync_steps
        res.append(r)
        c.close()
    w1 = time.perf_counter()
    return dict(wall=w1 - w0, results=res, rates=rates, h2d=h2d, d2h=d2h, steps=steps)


def _sweep_served(capi, ps, conds, local, rank, args):
    import numpy as np

    srv = capi.Server(local, len(conds))
    rng = np.random.default_rng(SWEEP_SEED + 1)
    order = rng.permutation(len(conds))
    gaps = rng.exponential(args.arrival_ms * 1e-3, len(conds))
    ids = {}
    w0 = time.perf_counter()
    for k, i in enumerate(order):
        time.sleep(float(gaps[k]))
        en, ne, ang, fr, bm = conds[i]
        ids[i] = srv.submit(sweep_config(capi, local, ne, 7000 + 100 * rank + int(i), converge=True, phases=PHASES),
                            ps, ps.gas_first, ps.gas_last, ps.gas_fraction, N_GAS, T_GAS, en, ang, fr, bm)
    sts = {i: srv.wait(j, 600.0) for i, j in ids.items()}
    w1 = time.perf_counter()
    rep = srv.report()
    srv.stop()
    lat = [s.end_time - s.submit_time for s in sts.values()]
    real = sum(s.result.real_collisions for s in sts.values())
    span = max(s.end_time for s in sts.values()) - min(s.submit_time for s in sts.values())
    errors = [f"E/N {conds[i][0]:.4g} Td, {conds[i][1]} electrons: status {s.status}: {s.error.decode(errors='replace')}"
              for i, s in sts.items() if s.state != capi.JOB_DONE]
    return dict(wall=w1 - w0, latencies=lat, real=real, span=span, errors=errors,
                failed=sum(s.state != capi.JOB_DONE for s in sts.values()),
                results=[sts[i].result for i in range(len(conds))], intervals=rep.intervals, busy=rep.busy_seconds,
                peak_footprint=rep.peak_footprint_bytes)


def _largest_deviation(conds, batched, plain, zs):
    """The condition whose batched and plain mean energies differ by the most
    standard errors: E/N, electrons, both mean energies and errors."""
    i = max(range(len(zs)), key=lambda k: zs[k])
    rb, rp = batched["results"][i], plain["results"][i]
    return {"E/N_Td": float(conds[i][0]), "electrons": int(conds[i][1]), "angle_deg": conds[i][2],
            "freq_hz": conds[i][3], "B/N_Hx": conds[i][4],
            "batched_eV": [float(rb.mean_energy), float(rb.mean_energy_err)],
            "plain_eV": [float(rp.mean_energy), float(rp.mean_energy_err)]}


def _accuracy(conds, batched, plain):
    """Convergence and agreement of the batched solves with the plain ones."""
    import numpy as np

    rel_err, zs, rel_dev, rate_dev = [], [], [], []
    for i in range(len(conds)):
        rb, rp = batched["results"][i], plain["results"][i]
        rel_err.append(rb.mean_energy_err / rb.mean_energy)
        zs.append(abs(rb.mean_energy - rp.mean_energy) / max(np.hypot(rb.mean_energy_err, rp.mean_energy_err), 1e-300))
        rel_dev.append(abs(rb.mean_energy / rp.mean_energy - 1.0))
        cb, qb = batched["rates"][i]
        cp, qp = plain["rates"][i]
        for p in range(len(qb)):
            if cb[p] >= 2000 and cp[p] >= 2000 and qp[p] > 0:
                sig = np.sqrt(1.0 / cb[p] + 1.0 / cp[p])
                rate_dev.append(abs(qb[p] / qp[p] - 1.0) / sig)
    return {"max_mean_energy_rel_err": float(max(rel_err)),
            "mean_energy_batched_vs_plain_max_sigmas": float(max(zs)),
            "mean_energy_batched_vs_plain_median_sigmas": float(np.median(zs)),
            "mean_energy_batched_vs_plain_max_rel": float(max(rel_dev)),
            "largest_sigmas_at": _largest_deviation(conds, batched, plain, zs),
            "rates_batched_vs_plain_median_poisson_sigmas": float(np.median(rate_dev)) if rate_dev else None,
            "rates_compared": len(rate_dev),
            "criterion": f"each condition stops when its mean-energy standard error < {SWEEP_ERR:.1%} "
                         "(50-block batch means, BoltzmannMC.C:1743-1767)"}


PRECISION_ELECTRONS = 1_000_000
REPEAT_SEEDS = 8


def _quantities(r):
    """(name, value, error) of the swarm parameters the precision study
    compares (E along -z: drift along +z)."""
    return [("mean_energy", r.mean_energy, r.mean_energy_err), ("flux_v_z", r.flux_v[2], r.flux_v_err[2]),
            ("bulk_v_z", r.bulk_v[2], r.bulk_v_err[2]), ("flux_D_xx", r.flux_d[0], r.flux_d_err[0]),
            ("flux_D_zz", r.flux_d[8], r.flux_d_err[8]), ("bulk_D_xx", r.bulk_d[0], r.bulk_d_err[0]),
            ("bulk_D_zz", r.bulk_d[8], r.bulk_d_err[8])]


def _ref_quantities(x):
    return [("mean_energy", x[0], x[1]), ("flux_v_z", x[4], x[7]), ("bulk_v_z", x[16], x[19]),
            ("flux_D_xx", x[8], x[11]), ("flux_D_zz", x[10], x[13]), ("bulk_D_xx", x[20], x[23]),
            ("bulk_D_zz", x[22], x[25])]


def _precision_study(capi, ps, conds, local):
    """The device's FP32 path against the reference's FP64 path on eight
    points of the sweep (tests/golden/sweep_fp64.json, made by
    tests/golden/make_sweep_fp64.py: the reference built from its sources,
    1e5 electrons, 1e4 integration intervals): the same conditions solved in
    one batch with 1e6 electrons and 1e4 integration intervals; per point and
    quantity the relative error and its size in combined standard errors;
    every rate coefficient with at least 1e4 counts in both runs. Plus seeded
    repeats of the sweep's largest condition solved to its 0.5 % criterion:
    the scatter of their mean energies against the batch-means errors they
    report (short runs: 50 blocks of a few intervals each, far shorter than
    the energy relaxation, so the reported errors understate the scatter)."""
    import numpy as np

    path = os.path.join(ROOT, "tests", "golden", "sweep_fp64.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        ref = json.load(f)["points"]
    b = capi.Batch(local, len(ref) + REPEAT_SEEDS)
    ctxs = []
    for k, rec in enumerate(ref):
        cfg = capi.default_config(device=local, seed=9100 + k, n_electrons=float(PRECISION_ELECTRONS), n_interp=10000,
                                  init_temp_ratio=KT_INIT, req_integration_points=1e4, max_coll_before_ss=300.0,
                                  max_seconds=300.0)
        c = capi.Context(cfg)
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, T_GAS, rec["red_field"])
        b.add(c)
        ctxs.append(c)
    big = max(range(len(conds)), key=lambda i: conds[i][1])
    for k in range(REPEAT_SEEDS):
        c = capi.Context(sweep_config(capi, local, conds[big][1], 9300 + k, converge=True))
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, T_GAS, conds[big][0])
        b.add(c)
        ctxs.append(c)
    t0 = time.perf_counter()
    res, st, _ = b.run()
    wall = time.perf_counter() - t0
    points, worst = [], {}
    n_ok = n_all = 0
    for k, rec in enumerate(ref):
        r = res[k]
        x = rec["result"]
        cnt, rate, _, _ = ctxs[k].process_results()
        pt = {"E/N_Td": rec["red_field"], "status": int(st[k])}
        for (name, gv, ge), (_, rv, re) in zip(_quantities(r), _ref_quantities(x)):
            if abs(rv) < 5.0 * re:
                continue
            rel = gv / rv - 1.0
            sig = (gv - rv) / float(np.hypot(ge, re))
            pt[name] = {"gpu": gv, "gpu_err": ge, "ref": rv, "ref_err": re, "rel_err": rel, "sigmas": sig}
            ok = abs(rel) <= 5e-3 or abs(sig) <= 2.0
            n_ok += ok
            n_all += 1
            w = worst.setdefault(name, {"max_abs_rel_err": 0.0, "max_abs_sigmas": 0.0})
            w["max_abs_rel_err"] = max(w["max_abs_rel_err"], abs(rel))
            w["max_abs_sigmas"] = max(w["max_abs_sigmas"], abs(sig))
        rr = np.array(rec["rate"])
        t_int = x[31] - x[30]
        # the device divides counts by the simulated electron-time, the
        # reference by N x integrated time (BoltzmannMC.C:1632); their ratio,
        # from the largest process's count and rate
        pb = int(np.argmax(cnt))
        et_ratio = (float(cnt[pb]) / (rate[pb] * ps.rel_dens[pb] * N_GAS)
                    / (PRECISION_ELECTRONS * (r.final_time - r.ss_time))) if rate[pb] > 0 else float("nan")
        pt["electron_time_over_N_T"] = et_ratio
        devs = []
        for p in range(ps.n):
            if rr[p] <= 0 or ps.rel_dens[p] <= 0:
                continue
            c_ref = rr[p] * t_int * rec["n_electrons"] * ps.rel_dens[p] * N_GAS
            if c_ref < 1e4 or cnt[p] < 1e4:
                continue
            rel = rate[p] / rr[p] - 1.0
            sig = rel / float(np.sqrt(1.0 / c_ref + 1.0 / float(cnt[p])))
            devs.append((abs(rel), abs(sig), p, float(cnt[p]), c_ref, rel, sig, ps.eloss[p], int(ps.ptype[p]),
                         rate[p] * et_ratio / rr[p] - 1.0))
            ok = abs(rel) <= 5e-3 or abs(sig) <= 2.0
            n_ok += ok
            n_all += 1
        if devs:
            pt["rates"] = {"compared": len(devs), "max_abs_rel_err": max(d[0] for d in devs),
                           "max_abs_sigmas": max(d[1] for d in devs),
                           "median_rel_err": float(np.median([d[5] for d in devs])),
                           "median_rel_err_per_N_T": float(np.median([d[9] for d in devs])),
                           "largest": [{"process": d[2], "type": d[8], "threshold_eV": d[7], "gpu_counts": d[3],
                                        "ref_counts": d[4], "rel_err": d[5], "sigmas": d[6],
                                        "rel_err_per_N_T": d[9]}
                                       for d in sorted(devs, key=lambda d: -d[1])[:3]]}
            w = worst.setdefault("rates", {"max_abs_rel_err": 0.0, "max_abs_sigmas": 0.0})
            w["max_abs_rel_err"] = max(w["max_abs_rel_err"], pt["rates"]["max_abs_rel_err"])
            w["max_abs_sigmas"] = max(w["max_abs_sigmas"], pt["rates"]["max_abs_sigmas"])
        pt["power_balance_rel_err"] = {"gpu": r.power_balance_rel_err, "ref": x[29]}
        points.append(pt)
    rep_res = res[len(ref):]
    me = np.array([r.mean_energy for r in rep_res])
    errs = np.array([r.mean_energy_err for r in rep_res])
    repeats = {"E/N_Td": conds[big][0], "electrons": conds[big][1], "seeds": REPEAT_SEEDS,
               "mean_energy_scatter_eV": float(np.std(me, ddof=1)),
               "median_reported_error_eV": float(np.median(errs)),
               "scatter_over_reported": float(np.std(me, ddof=1) / np.median(errs)),
               "median_integration_points": float(np.median([r.integration_points for r in rep_res]))}
    for c in ctxs:
        c.close()
    del b
    return {"reference": "FP64, the reference built from its sources, 1e5 electrons, 1e4 integration intervals "
                         "(tests/golden/sweep_fp64.json)",
            "device": f"FP32 push, FP64 tallies, {PRECISION_ELECTRONS} electrons, 1e4 integration intervals, batched",
            "criterion": "|rel err| <= 0.5 % or |dev| <= 2 combined standard errors",
            "rates_note": "rates divide counts by the simulated electron-time; rel_err_per_N_T divides by "
                          "N x integrated time as the reference does (BoltzmannMC.C:1632). With ionization the "
                          "reference re-simulates part of the interval for slots a secondary takes over mid-interval, "
                          "so its electron-time exceeds N x time by a share between 0 and the device's; the "
                          "reference's rates lie between the two device figures. Rate sigmas are Poisson only "
                          "and ignore the EEDF's own fluctuation, which dominates at low E/N",
            "within_criterion": f"{n_ok} of {n_all}", "worst": worst, "points": points,
            "seeded_repeats": repeats, "wall_s": wall}


# FP32 + SFU operations the method needs (the algorithmic count of the
# batched path's issue roofline): a free flight 1 lg2 + ~10 FP32 plus the
# field's sin/cos (AC 2 pairs, crossed B 1 pair and a half-angle sine); a null
# test ~6 FMA around its table loads; a real collision ~log2(P) x 2 FMA for the
# process choice + 2 sqrt + 1 rcp + 1 sin/cos pair + ~25 FMA.
OPS_FLIGHT = {"dc": 11.0, "ac": 15.0, "b": 14.0}
OPS_NULL_TEST = 6.0


def ops_real(n_processes):
    import math
    return 2.0 * math.ceil(math.log2(max(n_processes, 2))) + 2.0 + 1.0 + 2.0 + 25.0


# ncu counters of one batched DC advance launch over the sweep (1.98e7
# electrons, collision-stash shape 512 x 2, the same launch as above): warp
# instructions per electron-interval issued to the FMA, ALU and XU (SFU) pipes
NCU_PIPE_PER_ELECTRON = {"fma": 181978916 / 19795598, "alu": 244863326 / 19795598, "xu": 12198627 / 19795598}


def issue_roofline(real, null, electron_steps, kernel_ms, n_processes, flight_ops, sm_mhz):
    """Algorithmic FP32 + SFU operations of the advance over its device time,
    against the lanes' nominal rate (152 SMs x 128 FP32 lanes x the SM clock
    sampled during the run; no measured FP32 peak exists for this machine)."""
    ops = (flight_ops + OPS_NULL_TEST) * (real + null) + ops_real(n_processes) * real + flight_ops * electron_steps
    achieved = ops / (kernel_ms * 1e-3) / 1e12
    peak = 152 * 128 * sm_mhz * 1e6 / 1e12
    # the same rate counted as the FMA + XU pipes issue it (ncu warp
    # instructions per electron-interval x 32 lanes), over the same peak
    pipe = (NCU_PIPE_PER_ELECTRON["fma"] + NCU_PIPE_PER_ELECTRON["xu"]) * 32.0 * electron_steps
    pipe_achieved = pipe / (kernel_ms * 1e-3) / 1e12
    return {"bound": "issue (FP32 + SFU)", "achieved": achieved, "peak": peak, "unit": "Top/s",
            "frac": achieved / peak, "ops_per_electron_interval": ops / max(electron_steps, 1.0),
            "peak_source": "nominal: 152 SMs x 128 FP32 lanes x sampled SM clock",
            "pipe_issue": {"achieved": pipe_achieved, "frac": pipe_achieved / peak,
                           "source": "ncu sm__inst_executed_pipe_fma + _xu per electron-interval x 32 lanes, "
                                     "times this run's electron-intervals over its advance time"},
            "ncu_pipe_warp_instructions_per_electron_interval": NCU_PIPE_PER_ELECTRON,
            "note": "the advance issues more ALU (integer: random numbers, lane bookkeeping) than FMA "
                    "instructions at ~18 of 32 lanes active, about half of the issue slots busy (latency-bound: "
                    "state and table loads); the method's own FP32 + SFU work is a few % of the lanes' rate"}


def run_gpu_sweep(args):
    import torch

    from lokigpu import build as gbuild
    from lokigpu import capi

    rank, world, local = _init_ranks()
    if not os.path.exists(capi.library_path()):
        gbuild.build()
    ps = sweep_processes()
    field = args.workload == "field"
    conds = field_conditions() if field else sweep_conditions()
    clocks = ClockSampler(local)
    clocks.start()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    tb = _sweep_timed_batched(capi, ps, conds, local, rank, args, flush)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    total_ms, real, null = tb["total_ms"], tb["real"], tb["null"]
    if world > 1:
        total_ms, real, null = aggregate_ranks(total_ms, real, null, torch.device("cuda", local))
    value = real / (total_ms * 1e-3)
    tp = _sweep_timed_plain(capi, ps, conds, local, rank, args, flush) if not args.no_plain else None
    e2e_b = _sweep_e2e_batched(capi, ps, conds, local, rank) if not args.no_e2e else None
    e2e_p = _sweep_e2e_plain(capi, ps, conds, local, rank) if not (args.no_e2e or args.no_plain) else None
    srv = _sweep_served(capi, ps, conds, local, rank, args) if not args.no_served else None
    prec = _precision_study(capi, ps, conds, local) if (rank == 0 and not (args.no_precision or field)) else None
    stream = None
    if rank == 0 and not (args.no_served or field) and args.stream_requests > 0:
        stream = serve_stream(capi, local, args.stream_requests, args.stream_arrival_ms, args.request_cap_s,
                              args.slots, args.plain_requests)

    peak, peak_kind = measured_peaks()
    achieved = STATE_BYTES_PER_ELECTRON_STEP * tb["electron_steps"] / (tb["adv_ms"] * 1e-3) / 1e9 if tb["adv_ms"] > 0 else 0.0
    electrons = sum(c[1] for c in conds)
    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cores = os.cpu_count() or 1
            smp = []
            rounds = (len(conds) + cores - 1) // cores
            for k in range(rounds):
                _, sample, _, got = cpu_sample(args.cpu_seconds / rounds, cores, args.workload, offset=k * cores)
                smp += got
            cpu = {"value": cpu_sweep_rate(smp, cores), "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": sample + f"; {rounds} rounds cover every condition"}
        e2e = None
        if e2e_b:
            rep = e2e_b["report"]
            real_b = sum(r.real_collisions for r in e2e_b["results"])
            e2e = {"value": real_b / e2e_b["wall"], "unit": UNIT,
                   "h2d_bytes_per_step": rep.h2d_bytes / max(rep.intervals, 1),
                   "d2h_bytes_per_step": rep.d2h_bytes / max(rep.intervals, 1),
                   "scope": f"64 contexts created, processes uploaded, lgpu_batch_run to convergence, rates read back; "
                            f"{rep.intervals} batched intervals, {e2e_b['wall']:.2f} s wall",
                   "failed": int(sum(1 for s in e2e_b["status"] if s != 0)),
                   "max_energy_eV": max(r.max_eedf_energy for r in e2e_b["results"]) / 1.2}
        plain = None
        if tp:
            plain = {"value": tp["real"] / (tp["total_ms"] * 1e-3), "unit": UNIT,
                     "timed_intervals_per_condition": args.plain_steps,
                     "ms_per_interval_avg": tp["total_ms"] / (args.plain_steps * len(conds))}
            if e2e_p:
                real_p = sum(r.real_collisions for r in e2e_p["results"])
                plain["e2e"] = {"value": real_p / e2e_p["wall"], "unit": UNIT, "wall_s": e2e_p["wall"],
                                "h2d_bytes_per_step": e2e_p["h2d"] / max(e2e_p["steps"], 1),
                                "d2h_bytes_per_step": e2e_p["d2h"] / max(e2e_p["steps"], 1)}
        served = None
        if srv:
            served = {"p50_s": _percentile(srv["latencies"], 50), "p99_s": _percentile(srv["latencies"], 99),
                      "value": srv["real"] / srv["span"], "unit": UNIT, "jobs": len(conds), "failed": srv["failed"],
                      "arrivals": f"Poisson, mean gap {args.arrival_ms} ms, seeded order",
                      "latency": "submit to results on the host (lgpu_server_wait)", "span_s": srv["span"],
                      "peak_footprint_gb": srv["peak_footprint"] / 1e9, "errors": srv["errors"]}
        ratio = {}
        if plain:
            ratio["device_timed"] = value / plain["value"]
            if e2e and "e2e" in plain:
                ratio["e2e"] = e2e["value"] / plain["e2e"]["value"]
                if served:
                    ratio["served_over_plain_e2e"] = served["value"] / plain["e2e"]["value"]
        if stream and stream.get("served_over_plain"):
            ratio["served_stream_over_plain"] = stream["served_over_plain"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "field32_n2o2_crossedB_AC" if field else "sweep64_n2o2_1-1000Td",
                       "conditions": len(conds), "electrons_total": electrons,
                       "electrons_range": [FIELD_ELECTRONS] * 2 if field else list(SWEEP_NE_RANGE),
                       "E/N_Td": [1.0, 1000.0], "gas_density": N_GAS,
                       "fields": ("DC 100 Td at 90 degrees to B along z, B/N 0..2000 Hx (16); AC 150 Td rms at "
                                  "omega/N 1e-18..1e-14 m^3/s (16), 64 phase bins") if field else "DC at 180 degrees",
                       "processes": int(ps.n), "mixture": "N2-like 0.8 + O2-like 0.2 (synthetic, seeded)",
                       "method": f"batched: one launch sequence per interval for all {len(conds)} conditions",
                       "relax_intervals": args.relax, "l2": "256 MiB flush before every timed step",
                       "null_collisions_per_s": null / (total_ms * 1e-3),
                       "host_ms_per_step": tb["host_ms"] / args.steps,
                       "secondaries_per_step": tb["secondaries"] / args.steps,
                       "spilled_per_step": tb["spilled"] / args.steps,
                       "autotuned": {"threads_per_block": tb["shape"][0], "blocks_per_sm": tb["shape"][1],
                                     "electrons_per_warp_claim": tb["shape"][2],
                                     "collision_stash_records_per_warp": tb["shape"][3],
                                     "collision_turn_threshold": tb["real_batch"],
                                     "table_staging": {1.0: "block bounds in shared memory, rows from L2",
                                                       0.0: "rows from L2"}.get(tb["coarse"], "tuning"),
                                     "scope": "on-line, per mixture (largest process count, table points, "
                                              "field branches, thermal targets)"},
                       "collision_turn_threshold": tb["real_batch"], "coarse_null_test": tb["coarse"],
                       "regrids_per_step": tb["regrids"] / max(args.steps, 1)},
            "plain": plain, "batched_over_plain": ratio or None, "served": served, "served_stream": stream,
            "accuracy": _accuracy(conds, e2e_b, e2e_p) if (e2e_b and e2e_p) else None,
            "precision": prec,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": SWEEP_DRAM_BYTES_PER_ELECTRON_STEP * electrons,
                         "traffic_source": "ncu dram__bytes_read+write of the batched DC advance, one sweep interval",
                         "kernel": "k_advance_batch", "peak_source": peak_kind,
                         "algorithmic_bytes": f"{STATE_BYTES_PER_ELECTRON_STEP} B per electron-interval",
                         "kernel_ms_per_interval": tb["adv_ms"] / max(tb["intervals"], 1),
                         "issue": issue_roofline(tb["real"], tb["null"], tb["electron_steps"], tb["adv_ms"], ps.n,
                                                 0.5 * (OPS_FLIGHT["ac"] + OPS_FLIGHT["b"]) if field
                                                 else OPS_FLIGHT["dc"], (clk or {}).get("sm_mhz") or 2070.0)},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(tb["launches"]), "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ------------------------------------------------------------ serving stream
def serve_requests(n, seed=SWEEP_SEED + 7):
    """A seeded request stream: each request a mixture of 1-5 random gases
    (10-40 processes on 100-400-point grids, to 1e4 eV), E/N log-uniform in
    1..1000 Td, DC (60 %), crossed DC B with B/N 100..2000 Hx (20 %) or AC with
    omega/N log-uniform 1e-16..1e-14 m^3/s (20 %), electrons log-uniform in
    1e4..max_electrons."""
    import numpy as np
    from lokigpu import synth

    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        ng = int(rng.integers(1, 6))
        fr = rng.dirichlet(np.ones(ng))
        gases = [synth.random_gas(int(seed * 1000 + 10 * i + g), f"R{i}G{g}", float(fr[g]), e_max=1e4)
                 for g in range(ng)]
        en = float(10 ** rng.uniform(0.0, 3.0))
        kind = rng.random()
        angle, freq, red_mag = 180.0, 0.0, 0.0
        if kind < 0.2:
            angle, red_mag = 90.0, float(rng.uniform(100.0, 2000.0))
        elif kind < 0.4:
            freq = float(10 ** rng.uniform(-16.0, -14.0)) * N_GAS / (2.0 * np.pi)
        ne = int(round(10 ** rng.uniform(4.0, np.log10(SERVE_MAX_ELECTRONS))))
        out.append(dict(gases=gases, en=en, angle=angle, freq=freq, red_mag=red_mag, ne=ne, seed=9000 + i))
    return out


SERVE_MAX_ELECTRONS = 4e6


def serve_stream(capi, local, n_requests, arrival_ms, cap_s, slots, plain_requests):
    """The request stream of random mixtures through lgpu_server: every
    request converged to 0.5 % mean-energy error (or stopped at cap_s of wall
    time), Poisson arrivals with a mean gap of arrival_ms; then the first
    plain_requests requests solved one after the other with lgpu_solve (the
    plain path) for comparison. Returns the served block of the bench line."""
    import numpy as np
    import torch

    from lokigpu import synth

    reqs = serve_requests(n_requests)
    sets = [synth.flatten(r["gases"]) for r in reqs]
    rng = np.random.default_rng(SWEEP_SEED + 11)
    gaps = rng.exponential(arrival_ms * 1e-3, len(reqs))
    srv = capi.Server(local, slots)
    ids = []
    for r, ps, gap in zip(reqs, sets, gaps):
        time.sleep(float(gap))
        cfg = sweep_config(capi, local, r["ne"], r["seed"], converge=True)
        cfg.n_phases = 16
        cfg.max_seconds = cap_s
        ids.append(srv.submit(cfg, ps, ps.gas_first, ps.gas_last, ps.gas_fraction, N_GAS, T_GAS, r["en"],
                              r["angle"], r["freq"], r["red_mag"]))
    sts = [srv.wait(j, 3600.0) for j in ids]
    rep = srv.report()
    srv.stop()
    done = [s for s in sts if s.state == capi.JOB_DONE]
    capped = sum(1 for s in done if s.result.capped)
    lat = [s.end_time - s.submit_time for s in done]
    svc = [s.end_time - s.start_time for s in done]
    real = sum(s.result.real_collisions for s in done)
    span = max(s.end_time for s in sts) - min(s.submit_time for s in sts)
    errors = [f"request {i}: status {s.status}: {s.error.decode(errors='replace')}"
              for i, s in enumerate(sts) if s.state != capi.JOB_DONE]
    torch.cuda.synchronize()
    k = min(plain_requests, len(reqs))
    p0 = time.perf_counter()
    real_p = 0.0
    for r, ps in zip(reqs[:k], sets[:k]):
        cfg = sweep_config(capi, local, r["ne"], r["seed"], converge=True)
        cfg.n_phases = 16
        cfg.max_seconds = cap_s
        c = capi.Context(cfg)
        c.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c.set_conditions(N_GAS, T_GAS, r["en"], r["angle"], r["freq"], r["red_mag"])
        real_p += c.solve().real_collisions
        c.close()
    p1 = time.perf_counter()
    served = real / span
    plain = real_p / (p1 - p0) if k else None
    return {"workload": "serve_random_mixtures", "requests": len(reqs),
            "arrivals": f"Poisson, mean gap {arrival_ms} ms (faster than the device serves them: the rate "
                        f"measures capacity)", "slots": slots,
            "mixtures": "1-5 random gases, 10-40 processes each on 100-400-point grids",
            "E/N_Td": [1.0, 1000.0], "fields": "DC, crossed B (20 %), AC (20 %)",
            "electrons_range": [1e4, SERVE_MAX_ELECTRONS],
            "convergence": f"mean-energy standard error < {SWEEP_ERR:.1%}",
            "value": served, "unit": UNIT,
            "p50_s": _percentile(lat, 50), "p99_s": _percentile(lat, 99),
            "latency": "submit to results on the host (lgpu_server_wait): queueing plus service",
            "service_p50_s": _percentile(svc, 50), "service_p99_s": _percentile(svc, 99),
            "completed": len(done), "capped": capped, "cap_s": cap_s, "failed": len(reqs) - len(done),
            "errors": errors[:10], "span_s": span, "intervals": rep.intervals, "busy_s": rep.busy_seconds,
            "peak_footprint_gb": rep.peak_footprint_bytes / 1e9,
            "plain_first_requests": {"requests": k, "value": plain, "unit": UNIT, "wall_s": p1 - p0,
                                     "note": "the first requests solved one after the other with lgpu_solve"},
            "served_over_plain": served / plain if plain else None}


def run_gpu_serve(args):
    """Served request stream: latency percentiles, throughput, and the plain
    sequential path on the first requests for comparison."""
    from lokigpu import build as gbuild
    from lokigpu import capi

    rank, world, local = _init_ranks()
    if not os.path.exists(capi.library_path()):
        gbuild.build()
    clocks = ClockSampler(local)
    clocks.start()
    blk = serve_stream(capi, local, args.requests, args.arrival_ms, args.request_cap_s, args.slots,
                       args.plain_requests)
    clk = clocks.stop()
    if rank == 0:
        line = {
            "metric": METRIC, "value": blk["value"], "unit": UNIT, "n_gpus": world, "steps": blk["requests"],
            "warmup": 0, "ms_per_step": 1e3 * blk["span_s"] / blk["requests"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {k: blk[k] for k in ("workload", "requests", "arrivals", "slots", "mixtures", "E/N_Td",
                                           "electrons_range", "convergence")},
            "served": blk, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


def run_gpu_n2(args):
    import torch

    from lokigpu import build as gbuild
    from lokigpu import capi

    rank, world, local = _init_ranks()
    if not os.path.exists(capi.library_path()):
        gbuild.build()
    ps = n2_processes()

    def make_ctx(seed):
        cfg = capi.default_config(device=local, seed=seed, n_electrons=float(args.electrons), n_interp=10000,
                                  init_temp_ratio=KT_INIT)
        ctx = capi.Context(cfg)
        ctx.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        ctx.set_conditions(N_GAS, T_GAS, E_N)
        return ctx

    clocks = ClockSampler(local)
    clocks.start()                         # sampled over the relaxation and the timed steps
    ctx = make_ctx(1000 + rank)
    ctx.init_ensemble()
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    ctx.advance(args.relax)                # relaxation towards steady state (untimed)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    for _ in range(args.warmup):
        flush.add_(1.0)
        torch.cuda.synchronize()
        ctx.advance(1)

    r0 = ctx.advance(0)
    t0 = ctx.timing()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    total_ms = 0.0
    for _ in range(args.steps):
        flush.add_(1.0)                    # L2 flush (256 MiB written), outside the timed region
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.advance(1)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    r1 = ctx.advance(0)
    t1 = ctx.timing()
    real = r1.real_collisions - r0.real_collisions
    null = r1.null_collisions - r0.null_collisions
    if world > 1:
        total_ms, real, null = aggregate_ranks(total_ms, real, null, torch.device("cuda", local))
    value = real / (total_ms * 1e-3)

    adv_ms = t1.advance_ms - t0.advance_ms
    adv_n = t1.advance_launches - t0.advance_launches
    adv_steps = t1.electron_steps - t0.electron_steps
    peak, peak_kind = measured_peaks()
    achieved = STATE_BYTES_PER_ELECTRON_STEP * adv_steps / (adv_ms * 1e-3) / 1e9 if adv_ms > 0 else 0.0
    launches = int(t1.kernel_launches - t0.kernel_launches)

    # end to end through the C ABI from host buffers: process upload, start
    # ensemble, the solve loop and the result read-back
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        cfg = capi.default_config(device=local, seed=77 + rank, n_electrons=float(args.electrons), n_interp=10000,
                                  init_temp_ratio=KT_INIT, req_integration_points=200,
                                  max_coll_before_ss=20.0, max_seconds=120.0)
        c2 = capi.Context(cfg)
        c2.set_processes(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
        c2.set_conditions(N_GAS, T_GAS, E_N)
        res = c2.solve()
        c2.process_results()
        c2.distributions()
        w1 = time.perf_counter()
        tm = c2.timing()
        steps = max(res.sync_steps, 1)
        e2e = {"value": res.real_collisions / (w1 - w0), "unit": UNIT,
               "h2d_bytes_per_step": tm.h2d_bytes / steps, "d2h_bytes_per_step": tm.d2h_bytes / steps,
               "scope": f"lgpu_create..lgpu_solve..result read-back, {res.sync_steps} intervals, "
                        f"{res.integration_points} integration points, {w1 - w0:.2f} s wall"}
        c2.close()

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            v, sample, cores, _ = cpu_sample(args.cpu_seconds, os.cpu_count() or 1, "n2_200td")
            cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "n2_like_dc200Td_1e6e", "electrons": args.electrons, "E/N_Td": E_N,
                       "gas_density": N_GAS, "processes": int(ps.n),
                       "method": "plain (one synchronisation interval per step)",
                       "relax_intervals": args.relax, "l2": "256 MiB flush before every timed step",
                       "null_collisions_per_s": null / (total_ms * 1e-3)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": DRAM_BYTES_PER_ELECTRON_STEP * args.electrons,
                         "traffic_source": "ncu dram__bytes_read+write of k_advance at 4e6 electrons, scaled per electron",
                         "kernel": "k_advance", "peak_source": peak_kind,
                         "algorithmic_bytes": f"{STATE_BYTES_PER_ELECTRON_STEP} B per electron-interval",
                         "kernel_ms_per_launch": adv_ms / max(adv_n, 1)},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="sweep", choices=["sweep", "field", "n2_200td", "serve"])
    ap.add_argument("--requests", type=int, default=100, help="serve: requests in the stream")
    ap.add_argument("--stream-requests", type=int, default=500,
                    help="sweep: requests of the random-mixture stream served after the sweep (0: none)")
    ap.add_argument("--stream-arrival-ms", type=float, default=2.0, help="sweep: mean gap of the stream's arrivals")
    ap.add_argument("--request-cap-s", type=float, default=60.0, help="serve: wall-time cap of one request")
    ap.add_argument("--slots", type=int, default=64, help="serve: jobs advanced together")
    ap.add_argument("--plain-requests", type=int, default=8, help="serve: requests also solved one by one")
    ap.add_argument("--electrons", type=int, default=N_ELECTRONS, help="n2_200td only")
    ap.add_argument("--relax", type=int, default=None)
    ap.add_argument("--plain-steps", type=int, default=20, help="sweep: timed plain intervals per condition")
    ap.add_argument("--arrival-ms", type=float, default=20.0, help="sweep: mean gap of the served arrivals")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-precision", action="store_true", help="skip the study against the FP64 reference")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--schedule", default="",
                    help="sweep/field: pin the batched advance's schedule 'shape,threshold,coarse' (default: tuned)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.steps is None:
        args.steps = 200 if args.workload in ("sweep", "field") else 2000
    if args.relax is None:
        args.relax = 200 if args.workload in ("sweep", "field") else 400
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "serve":
        return run_gpu_serve(args)
    global PHASES
    PHASES = FIELD_PHASES if args.workload == "field" else 100
    return run_gpu_sweep(args) if args.workload in ("sweep", "field") else run_gpu_n2(args)


if __name__ == "__main__":
    sys.exit(main())
