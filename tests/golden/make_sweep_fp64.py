"""FP64 reference solves of eight points of the 64-point E/N sweep, for the
precision study of bench.py (the per-quantity error of the device's FP32
path against the reference's FP64 one).

Run where the reference source tree is at hand (never on the GPU machine):

    make -C oracle/ref REF=<reference Code/>
    python tests/golden/make_sweep_fp64.py      # writes tests/golden/sweep_fp64.json
    python tests/golden/make_sweep_fp64.py --only 3   # one point (index into INDICES)

Each point is the reference built from its own sources (oracle/_ref/
libref_harness.so, seeded generator), solving the sweep's mixture
(make_golden.case_gases("sweep")) at one E/N of logspace(0, 3, 64) with 1e5
electrons started at kT = 1 eV, 1e4 integration intervals, the default 1e4
table points. Recorded per point: the swarm parameters with their batch-means
errors, the rate coefficients (collision counts follow from them), the power
terms and the power balance. Points already in the file are kept.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import multiprocessing as mp
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

INDICES = (0, 9, 18, 27, 36, 45, 54, 63)
N_ELECTRONS = 1e5
NUMERICS = {"nIntegrationPoints": "1E4", "maxCollisionsBeforeSteadyState": "300", "nInterpPoints": "10000"}
OUT = os.path.join(HERE, "sweep_fp64.json")


def solve_point(idx):
    td = float(np.logspace(0.0, 3.0, 64)[idx])
    tmp = tempfile.mkdtemp(prefix=f"sweep_{idx}_")
    _, _, setup = mg.write_inputs("sweep", tmp, n_electrons=N_ELECTRONS, extra=NUMERICS, red_field=td)
    lib = mg.open_ref(tmp, setup)
    lib.ref_rng_seed(ctypes.c_uint64(500 + idx))
    P = lib.ref_n_processes()
    r = np.zeros(39)
    rate = np.zeros(P)
    lib.ref_solve(mg.ptr(r), mg.ptr(rate))
    gain, loss = np.zeros(P), np.zeros(P)
    lib.ref_get_power(mg.ptr(gain), mg.ptr(loss))
    return dict(index=idx, red_field=td, n_electrons=N_ELECTRONS, numerics=NUMERICS, seed=500 + idx,
                result=r.tolist(), rate=rate.tolist(), power_gain=gain.tolist(), power_loss=loss.tolist())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", type=int, default=None, help="position in INDICES")
    a = ap.parse_args()
    todo = list(INDICES) if a.only is None else [INDICES[a.only]]
    have = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            have = {p["index"]: p for p in json.load(f)["points"]}
    with mp.get_context("spawn").Pool(1) as pool:
        for rec in pool.imap(solve_point, [i for i in todo if i not in have]):
            have[rec["index"]] = rec
            print(f"E/N {rec['red_field']:.4g} Td: mean energy {rec['result'][0]:.5g} eV "
                  f"({rec['result'][28]:.0f} s)", flush=True)
            with open(OUT, "w") as f:
                json.dump(dict(points=[have[k] for k in sorted(have)],
                               result_layout="oracle/ref/harness.cpp: ref_solve"), f)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
