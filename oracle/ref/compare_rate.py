"""Real-collision rate of the reference built from source against the oracle port.

The benchmark's CPU baseline times the oracle (the C restatement in
oracle/loki_oracle.c) because the reference's sources are not on the GPU
machine. This script, run where they are (after `make -C oracle/ref`), times
both on the same case and threads - the sweep's N2-like/O2-like mixture at
100 Td with 1e4 electrons - so the baseline can be read against the reference
itself:

    OMP_NUM_THREADS=8 python oracle/ref/compare_rate.py [--threads 8] [--seconds 20]

The reference runs a full solve (steady state, then 5000 integration points)
and its rate is real collisions over its own elapsedTime, as MCSimDetails.txt
reports it (Output.h:800-820); the port runs the same interval loop for the
given seconds.
"""
import argparse
import ctypes
import multiprocessing as mp
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
for p in (os.path.join(ROOT, "loki-mc_gb300", "python"), os.path.join(ROOT, "tests", "golden"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def reference_rate(n_electrons):
    import make_golden as mg
    from lokigpu import synth

    gases = [synth.n2_like_gas(fraction=0.8, e_max=1e4), synth.o2_like_gas(fraction=0.2, e_max=1e4)]
    tmp = tempfile.mkdtemp(prefix="rate_")
    setup = synth.write_case(tmp, gases, pressure_pa=3.22e22 * mg.KB * 300.0, red_field=100.0,
                             n_electrons=n_electrons, kte_init_ev=1.0, sharing="equalSharing",
                             extra_numerics={"nInterpPoints": "10000", "nIntegrationPoints": "5000",
                                             "maxCollisionsBeforeSteadyState": "1000"})
    lib = mg.open_ref(tmp, setup)
    lib.ref_rng_seed(ctypes.c_uint64(5))
    r = np.zeros(39)
    rate = np.zeros(lib.ref_n_processes())
    lib.ref_solve(mg.ptr(r), mg.ptr(rate))
    return float(r[26]), float(r[28]), float(r[0])  # real collisions, elapsed s, mean energy eV


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--seconds", type=float, default=20.0)
    ap.add_argument("--electrons", type=int, default=10000)
    a = ap.parse_args()
    os.environ["OMP_NUM_THREADS"] = str(a.threads)
    with mp.get_context("spawn").Pool(1) as pool:
        real, elapsed, me = pool.apply(reference_rate, (float(a.electrons),))
    print(f"reference: {real:.4g} real collisions in {elapsed:.1f} s = {real / elapsed:.4g}/s "
          f"({a.threads} threads, mean energy {me:.4g} eV)")
    import bench

    v, sample, cores = bench.cpu_sample(a.seconds, a.threads, "sweep", n_electrons=a.electrons)
    print(f"oracle port: {v:.4g}/s on {cores} threads ({sample})")


if __name__ == "__main__":
    main()
