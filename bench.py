#!/usr/bin/env python3
"""Benchmark of the electron Monte Carlo hot path on GB300.

Workload: the synthetic N2-like molecular gas (elastic with screened-Coulomb
anisotropy, 1 rotational and 8 vibrational <-> levels, 20 electronic levels,
ionization at 15.6 eV with equal energy sharing; seeded smooth cross sections
on 200-point log grids, Boltzmann populations at 300 K), DC E/N = 200 Td,
N = 3.22e22 m^-3, 1e6 electrons, FP32 push with FP64 tallies.

A step is one synchronisation interval of the plain method over the whole
ensemble: every electron flies and collides up to the synchronisation time,
population control runs, and the ensemble is sampled (moments). The metric is
real collisions per second. The ensemble is relaxed for a number of untimed
intervals first, then W warm-up steps, then K timed steps; an L2 flush (a
256 MiB write) precedes every timed step and is outside the timed region.

--impl reference times the CPU implementation of the same path on the host
cores: the reference built from its own sources when present (oracle/_ref),
else the C restatement (oracle/), on a bounded sample of the same workload.
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
E_N = 200.0
N_ELECTRONS = 1_000_000
STATE_BYTES_PER_ELECTRON_STEP = 64  # 32 B state read + 32 B written per electron per interval
# DRAM bytes per electron and interval of k_advance, from one ncu capture of the
# same kernel on 4e6 electrons (profiles/k_advance_n2_dc200.md): 130.5 MB read +
# 73.6 MB written; traffic grows in proportion to the electrons advanced
DRAM_BYTES_PER_ELECTRON_STEP = (130.535168e6 + 73.571328e6) / 4.0e6
WORKLOAD = "n2_like_dc200Td_1e6e"


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


def workload_processes():
    from lokigpu import synth

    return synth.flatten([synth.n2_like_gas()])


# --------------------------------------------------------------------- CPU arm
def cpu_sample(seconds: float, threads: int, n_electrons: int = 100_000, warm_intervals: int = 300):
    """Times the CPU restatement of the reference's path (oracle/) on the host
    cores: the same gas and field, n_electrons electrons, rate measured after
    warm_intervals intervals so it is taken near steady state like the GPU's."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O

    ps = workload_processes()
    off = np.concatenate([[0], np.cumsum([len(e) for e in ps.raw_e])]).astype(np.int32)
    arrays = dict(ptype=ps.ptype, is_super=ps.is_super, sampler=ps.sampler, sampler_p0=ps.sampler_p0,
                  sampler_p1=ps.sampler_p1, superw=ps.superw, emin=ps.emin, emax=ps.emax, rel_dens=ps.rel_dens,
                  mass=ps.mass, red_mass=ps.red_mass, eloss=ps.eloss, wparam=ps.wparam, raw_off=off[:-1],
                  raw_len=np.array([len(e) for e in ps.raw_e], np.int32), raw_e=np.concatenate(ps.raw_e),
                  raw_v=np.concatenate(ps.raw_v), gas_first=ps.gas_first, gas_last=ps.gas_last,
                  gas_frac=ps.gas_fraction, energy_max_elastic=ps.energy_max_elastic)
    pr = O.OracleProcs(arrays, 10000)
    f = O.make_fields(N_GAS, T_GAS, E=(0.0, 0.0, -E_N * 1e-21 * N_GAS))
    cfg = O.default_run_config(n_electrons, n_threads=threads, seed=3, max_seconds=seconds,
                               mark_sync_step=warm_intervals, req_integration_points=1e12)
    st, res, _ = O.run(pr, f, cfg)
    if res.mark_elapsed > 0 and res.elapsed > res.mark_elapsed:
        real = res.real_collisions - res.mark_real_collisions
        dt = res.elapsed - res.mark_elapsed
        sample = (f"{n_electrons} electrons, same gas and field, intervals {warm_intervals + 1}..{res.sync_steps} "
                  f"({dt:.1f} s of a {seconds:.0f} s run, C restatement of the reference path)")
    else:
        real, dt = res.real_collisions, res.elapsed
        sample = f"{n_electrons} electrons, same gas and field, first {res.sync_steps} intervals ({dt:.1f} s)"
    return real / dt, sample, threads


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    t0 = time.time()
    rates = []
    sample = ""
    per_step = max(3.0, min(20.0, 60.0 / max(1, args.steps + args.warmup)))
    for i in range(args.warmup + args.steps):
        r, sample, _ = cpu_sample(per_step, threads, warm_intervals=100)
        if i >= args.warmup:
            rates.append(r)
    v = sum(rates) / len(rates)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * (time.time() - t0) / (args.steps + args.warmup),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "electrons": 100_000, "impl_detail": "C restatement of the reference path (oracle/), OpenMP"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------- GPU arm
def aggregate_ranks(total_ms, real, null, device):
    """Replicas only: every rank advances its own ensemble; the job time is the
    slowest rank's, the collisions are summed over ranks."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    c = torch.tensor([real, null], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t[0]), float(c[0]), float(c[1])


def run_gpu_arm(args):
    import torch

    from lokigpu import build as gbuild
    from lokigpu import capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    if not os.path.exists(capi.library_path()):
        gbuild.build()
    ps = workload_processes()

    def make_ctx(seed):
        cfg = capi.default_config(device=local, seed=seed, n_electrons=float(args.electrons), n_interp=10000,
                                  init_temp_ratio=1.0 / (8.617333262e-5 * T_GAS))  # start Maxwellian at kT = 1 eV
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
                                  init_temp_ratio=1.0 / (8.617333262e-5 * T_GAS), req_integration_points=200,
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

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            v, sample, cores = cpu_sample(args.cpu_seconds, os.cpu_count() or 1)
            cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "electrons": args.electrons, "E/N_Td": E_N, "gas_density": N_GAS,
                       "processes": int(ps.n), "method": "plain (one synchronisation interval per step)",
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
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--electrons", type=int, default=N_ELECTRONS)
    ap.add_argument("--relax", type=int, default=400)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
