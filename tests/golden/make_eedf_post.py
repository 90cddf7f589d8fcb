"""Generates tests/golden/eedf_post_*.npz: the reference's own end-of-job
post-processing of an EEDF, to pin the device's (BoltzmannMC.C:2186-2266,
2268-2384; Collision.C:355-397).

Run in a checkout that has the reference source tree (never on the GPU machine):

    make -C oracle/ref REF=<reference Code/>
    python tests/golden/make_eedf_post.py

Each case runs a short seeded solve of the reference built from its own
sources (oracle/_ref/libref_harness.so) on a synthetic mixture and records:
the EEDF it ends with (and the energy grid it lies on), the collision behind
every MC process as the end-of-job routines read it (raw integral and
momentum-transfer cross sections, target or product density, threshold, mass
ratio, statistical-weight ratio), the field frequencies and gas density, and
what the reference computed from them: the EEDF-convolved rate coefficient of
every process (under AC also from each phase's EEDF), the two-term swarm
parameters and the total momentum-transfer cross section on the grid nodes. The comparison is
deterministic: the device post-processes the same EEDF.
"""
from __future__ import annotations

import ctypes
import multiprocessing as mp
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

D = ctypes.c_double
TWOTERM_KEYS = ("totalIonRateCoeff", "totalAttRateCoeff", "momTransfFreq", "energyRelaxFreq",
                "energyRelaxFreqClassic", "redDiffCoeffEnergy_eedf", "redMobCoeffEnergy_eedf", "redDiffCoeff_eedf",
                "redMobCoeff_DC_eedf", "characEnergy_eedf", "redMobCoeff_xx_real_eedf", "redMobCoeff_xx_imag_eedf",
                "redMobCoeff_xy_real_eedf", "redMobCoeff_xy_imag_eedf", "redMobCoeff_zz_real_eedf",
                "redMobCoeff_zz_imag_eedf")
SHORT = {"nIntegrationPoints": "500", "nInterpPoints": "2000", "maxCollisionsBeforeSteadyState": "100"}
CASES = {
    "atomic_dc100": ("atomic", {}, SHORT),
    "n2_dc200": ("n2", {"red_field": 200.0}, SHORT),
    "mix_dc300": ("mix", {"red_field": 300.0}, SHORT),
    "mix_b100": ("mix", {"red_field": 100.0, "red_mag": 1000.0, "angle": 90.0}, SHORT),
    "mix_ac150": ("mix", {"red_field": 150.0, "freq": 3.22e22 * 1e-14 / (2 * np.pi)},
                  dict(SHORT, nIntegrationPhases="16")),
    "screen_dc100": ("screen", {}, SHORT),
}


def run(name, seed):
    case, over, numerics = CASES[name]
    out_path = os.path.join(HERE, f"eedf_post_{name}.npz")
    tmp = tempfile.mkdtemp(prefix=f"eedf_post_{name}_")
    _, meta, setup = mg.write_inputs(case, tmp, n_electrons=2e4, extra=numerics, **over)
    lib = mg.open_ref(tmp, setup)
    lib.ref_swarm_param.restype = D
    lib.ref_rng_seed(ctypes.c_uint64(seed))
    P = lib.ref_n_processes()
    r = np.zeros(39)
    lib.ref_solve(mg.ptr(r), mg.ptr(np.zeros(P)))
    proc = mg.dump_processes(lib)  # after the solve has set the relative densities (BoltzmannMC.C:439-455)
    nc = lib.ref_n_eedf_cells()
    cells, eedf = np.zeros(nc), np.zeros(nc)
    lib.ref_get_eedf(mg.ptr(cells), mg.ptr(eedf))
    grid = np.zeros(5)
    lib.ref_get_twoterm_grid(mg.ptr(grid))
    scal = np.zeros((P, 6))
    ni, nm = np.zeros(P, np.int32), np.zeros(P, np.int32)
    ie, iv, me, mv = [], [], [], []
    for p in range(P):
        a, b = ctypes.c_int(), ctypes.c_int()
        lib.ref_twoterm_sizes(p, ctypes.byref(a), ctypes.byref(b))
        ni[p], nm[p] = a.value, b.value
        bufs = [np.zeros(a.value), np.zeros(a.value), np.zeros(b.value), np.zeros(b.value)]
        s = np.zeros(6)
        lib.ref_get_twoterm(p, mg.ptr(s), *[mg.ptr(x) for x in bufs])
        scal[p] = s
        ie.append(bufs[0]), iv.append(bufs[1]), me.append(bufs[2]), mv.append(bufs[3])
    rates = np.zeros(P)
    lib.ref_get_eedf_rates(mg.ptr(rates))
    swarm = np.array([lib.ref_swarm_param(k.encode()) for k in TWOTERM_KEYS])
    mt = np.zeros(int(grid[4]) + 1)
    lib.ref_get_total_mt(mg.ptr(mt))
    extra = {}
    n_ph = lib.ref_n_phases_periodic()
    if n_ph > 0:
        # AC: the per-phase EEDFs and the rate coefficients from each (BoltzmannMC.C:2276-2330)
        z = [np.zeros(n_ph) for _ in range(2)] + [np.zeros(3 * n_ph)] * 2 + [np.zeros(9 * n_ph)] * 2
        per = np.zeros(n_ph * nc)
        lib.ref_get_periodic(*[mg.ptr(x) for x in z], mg.ptr(per))
        rp = np.zeros(n_ph * P)
        lib.ref_get_eedf_rates_periodic(mg.ptr(rp))
        extra = dict(eedf_periodic=per.reshape(n_ph, nc), rates_periodic=rp.reshape(n_ph, P))
    np.savez_compressed(out_path, case=name, max_eedf_energy=r[38], mean_energy=r[0], cells=cells, eedf=eedf, **extra,
                        grid=grid, twoterm_scalars=scal, int_len=ni, mom_len=nm, int_e=np.concatenate(ie),
                        int_v=np.concatenate(iv), mom_e=np.concatenate(me), mom_v=np.concatenate(mv), rates=rates,
                        swarm_keys=np.array(TWOTERM_KEYS), swarm=swarm, total_mt=mt,
                        **{"proc_" + k: v for k, v in proc.items()})
    return out_path


def main():
    # one fresh process per case: the reference exits on its own errors
    # (Message.C:6-16), and each run changes the working directory
    only = sys.argv[1] if len(sys.argv) > 1 else None
    ctx = mp.get_context("spawn")
    for i, name in enumerate(CASES):
        if only not in (None, name):
            continue
        pr = ctx.Process(target=run, args=(name, 500 + i))
        pr.start()
        pr.join()
        if pr.exitcode != 0:
            raise SystemExit(f"{name}: the reference run failed (exit code {pr.exitcode})")
        print("wrote", f"tests/golden/eedf_post_{name}.npz")


if __name__ == "__main__":
    main()
