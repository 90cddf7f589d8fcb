"""Generates the golden vectors in tests/golden/ from the reference itself.

Run in a checkout that has the reference source tree (never on the GPU machine):

    make -C oracle/ref REF=<reference Code/>   # builds oracle/_ref/libref_harness.so
    python tests/golden/make_golden.py      # writes tests/golden/*.npz
    python tests/golden/make_golden.py --stats   # also the long seeded solves

Each case writes the synthetic mixture as LXCat + setup files into a scratch
directory, loads the reference engine built from its own sources
(oracle/_ref/libref_harness.so, see oracle/ref/harness.cpp) in a fresh
process, and records:

* the flattened per-process arrays the reference builds
  (BoltzmannMC.C:29-271) and its interpolated tables (BoltzmannMC.C:561-615);
* free flights in each field branch of accelerateElectron
  (BoltzmannMC.C:804-905): DC, AC, DC E + B, cyclotron resonance, AC + B;
* collision events of performCollision (BoltzmannMC.C:907-1280) driven by a
  recorded stream of uniforms, cold and thermal, for each ionization
  energy-sharing mode, with the number of uniforms consumed;
* with --stats, full seeded solves (BoltzmannMC.C:273-297) whose swarm
  parameters, rate coefficients, power terms and distributions (EEDF, EADF,
  anisotropies, EVDF, periodic averages, as cumulative probabilities on
  sub-grids of the reference's own cells) pin the statistical parity tests;
  --stats-only runs just those, --only NAME one case.
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
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "loki-mc_gb300", "python"))
sys.path.insert(0, os.path.dirname(HERE))
from lokigpu import synth  # noqa: E402
from lokigpu import constants as C  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libref_harness.so")
KB = C.BOLTZMANN
D = ctypes.c_double
VP = ctypes.c_void_p


def ptr(a):
    return a.ctypes.data_as(VP)


# --------------------------------------------------------------------------- cases

def case_gases(name):
    if name == "atomic":
        return [synth.atomic_gas()], dict(N=3.22e22, red_field=100.0, max_e=100.0, sharing="equalSharing")
    if name == "n2":
        return [synth.n2_like_gas()], dict(N=3.22e22, red_field=200.0, max_e=120.0, sharing="equalSharing")
    if name == "mix":
        n2 = synth.n2_like_gas(fraction=0.8)
        o2 = synth.o2_like_gas(fraction=0.2)
        synth.assign_sampler(o2, "Excitation", "bornDipole")
        synth.assign_sampler(o2, "Vibrational", "surendra")
        synth.assign_sampler(o2, "Rotational", "forward")
        synth.assign_sampler(o2, "Ionization", "momentumConservationIonization")
        synth.assign_sampler(n2, "Ionization", "isotropic")
        return [n2, o2], dict(N=3.22e22, red_field=100.0, max_e=120.0, sharing="equalSharing")
    if name == "screen":
        # screened-Coulomb scattering with the screening energy taken after the
        # energy loss (params[0] = 1) on inelastic processes, where the energy
        # after differs from the incident one (AngularScatteringFunctions.h:56-74)
        n2 = synth.n2_like_gas(fraction=0.8)
        o2 = synth.o2_like_gas(fraction=0.2)
        synth.assign_sampler(n2, "Vibrational", "coulombScreen", (1.0, 1.3))
        synth.assign_sampler(n2, "Excitation", "coulombScreen", (1.0, 2.7))
        synth.assign_sampler(o2, "Excitation", "coulombScreen", (0.0, 0.8))
        return [n2, o2], dict(N=3.22e22, red_field=150.0, max_e=120.0, sharing="equalSharing")
    if name == "sweep":
        # the 64-point E/N sweep's mixture (bench.py: sweep_processes): tables
        # to 1e4 eV, default samplers
        n2 = synth.n2_like_gas(fraction=0.8, e_max=1e4)
        o2 = synth.o2_like_gas(fraction=0.2, e_max=1e4)
        return [n2, o2], dict(N=3.22e22, red_field=100.0, max_e=120.0, sharing="equalSharing")
    raise KeyError(name)


def write_inputs(name, tmp, n_electrons=1e4, extra=None, **over):
    gases, meta = case_gases(name)
    meta = dict(meta, **over)
    numerics = {"nInterpPoints": "2000"}
    numerics.update(extra or {})
    setup = synth.write_case(tmp, gases, pressure_pa=meta["N"] * KB * 300.0, red_field=meta["red_field"],
                             n_electrons=n_electrons, kte_init_ev=1.0, sharing=meta["sharing"],
                             extra_numerics=numerics, red_mag=meta.get("red_mag", 0.0),
                             angle=meta.get("angle", 180.0), freq=meta.get("freq", 0.0),
                             gas_temp=meta.get("gas_temp", "false"))
    return gases, meta, setup


def open_ref(tmp, setup):
    os.chdir(tmp)
    lib = ctypes.CDLL(LIB)
    for fn in ("ref_accelerate", "ref_collide", "ref_set_fields", "ref_set_collision_options", "ref_interpolate",
               "ref_statistical_error"):
        getattr(lib, fn).restype = None
    lib.ref_statistical_error.restype = D
    n = lib.ref_open(setup.encode())
    assert n > 0
    return lib


def dump_processes(lib):
    P = lib.ref_n_processes()
    G = lib.ref_n_gases()
    i32 = lambda: np.zeros(P, np.int32)  # noqa: E731
    f64 = lambda: np.zeros(P, np.float64)  # noqa: E731
    a = dict(ptype=i32(), is_super=i32(), is_elastic=i32(), sampler=i32(), sampler_p0=f64(), sampler_p1=f64(),
             is_momcons=i32(), superw=f64(), emin=f64(), emax=f64(), rel_dens=f64(), mass=f64(), red_mass=f64(),
             eloss=f64(), wparam=f64(), raw_len=i32())
    lib.ref_get_processes(*[ptr(a[k]) for k in ("ptype", "is_super", "is_elastic", "sampler", "sampler_p0",
                                                 "sampler_p1", "is_momcons", "superw", "emin", "emax", "rel_dens",
                                                 "mass", "red_mass", "eloss", "wparam", "raw_len")])
    off = np.concatenate([[0], np.cumsum(a["raw_len"])]).astype(np.int32)
    raw_e = np.zeros(off[-1])
    raw_v = np.zeros(off[-1])
    for p in range(P):
        e = np.zeros(a["raw_len"][p])
        v = np.zeros(a["raw_len"][p])
        lib.ref_get_raw(p, ptr(e), ptr(v))
        raw_e[off[p]:off[p + 1]] = e
        raw_v[off[p]:off[p + 1]] = v
    gf, gl, gfr = np.zeros(G), np.zeros(G), np.zeros(G)
    lib.ref_get_gases(ptr(gf), ptr(gl), ptr(gfr))
    a.update(raw_off=off[:-1].copy(), raw_e=raw_e, raw_v=raw_v, gas_first=gf.astype(np.int32),
             gas_last=gl.astype(np.int32), gas_frac=gfr)
    return a


def scalars(lib):
    s = np.zeros(20)
    lib.ref_get_scalars(ptr(s))
    return s


def dump_tables(lib, P):
    M = lib.ref_table_size()
    grid, nu_tot, nu_max = np.zeros(M), np.zeros(M), np.zeros(M)
    sig, cum = np.zeros(M * P), np.zeros(M * P)
    lib.ref_get_tables(ptr(grid), ptr(sig), ptr(cum), ptr(nu_tot), ptr(nu_max))
    return dict(tab_grid=grid, tab_sig=sig, tab_cum=cum, tab_nu_tot=nu_tot, tab_nu_max=nu_max)


FIELD_BRANCHES = ("dc", "ac", "b", "ecr", "acb")


def field_params(branch, rng, N):
    """E vector (V/m, AC amplitude), f (Hz), B/N (Hx), cyclotron (rad/s)."""
    en = 100e-21 * N
    ang = rng.uniform(0.2, 2.9)
    E = np.array([en * np.sin(ang), 0.0, en * np.cos(ang)])
    if branch == "dc":
        return E, 0.0, 0.0, 0.0
    if branch == "ac":
        return E, 1.3e9, 0.0, 0.0
    if branch == "b":
        return E, 0.0, 300.0, 1.7e9
    if branch == "ecr":
        w = 2.0 * np.pi * 0.9e9
        return E, 0.9e9, 800.0, w
    if branch == "acb":
        return E, 0.6e9, 500.0, 2.6e9
    raise KeyError(branch)


def run_case(name, out_path, seed):
    rng = np.random.default_rng(seed)
    tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
    gases, meta, setup = write_inputs(name, tmp)
    lib = open_ref(tmp, setup)
    lib.ref_eval_nonconstant()   # sets relDensities (BoltzmannMC.C:439-455)
    procs = dump_processes(lib)
    P = len(procs["ptype"])
    sc = scalars(lib)
    lib.ref_interpolate(D(meta["max_e"]))
    tabs = dump_tables(lib, P)
    sc2 = scalars(lib)
    N = sc[0]
    out = dict(procs, **tabs, scalars=sc, scalars_tab=sc2, energy_max_elastic=np.array(sc[2]))

    # ---- free flights
    K = 48
    for b in FIELD_BRANCHES:
        E, fhz, bn, wc = field_params(b, rng, N)
        lib.ref_set_fields(D(E[0]), D(E[1]), D(E[2]), D(fhz), D(bn), D(wc))
        t = rng.uniform(0.0, 2e-7, K)
        dt = 10 ** rng.uniform(-12.5, -9.0, K)
        pos = rng.normal(0.0, 1e-3, (K, 3))
        vel = rng.normal(0.0, 1.0, (K, 3)) * (10 ** rng.uniform(4.5, 6.5, K))[:, None]
        energy = 0.5 * C.ELECTRON_MASS * ((vel[:, 0] ** 2 + vel[:, 1] ** 2) + vel[:, 2] ** 2) / C.ELECTRON_CHARGE
        po, vo, eo, go = pos.copy(), vel.copy(), energy.copy(), np.zeros(K)
        for k in range(K):
            p3, v3 = po[k].copy(), vo[k].copy()
            e1, g1 = np.array([eo[k]]), np.zeros(1)
            lib.ref_accelerate(D(t[k]), D(dt[k]), ptr(p3), ptr(v3), ptr(e1), ptr(g1))
            po[k], vo[k], eo[k], go[k] = p3, v3, e1[0], g1[0]
        out.update({f"acc_{b}_field": np.array([E[0], E[1], E[2], fhz, bn, wc]), f"acc_{b}_t": t,
                    f"acc_{b}_dt": dt, f"acc_{b}_pos": pos, f"acc_{b}_vel": vel, f"acc_{b}_energy": energy,
                    f"acc_{b}_pos_out": po, f"acc_{b}_vel_out": vo, f"acc_{b}_energy_out": eo,
                    f"acc_{b}_gain": go})

    # ---- collisions (cold and thermal; every energy-sharing mode)
    modes = [(0, 0, 0.5), (1, 0, 0.5), (0, 1, 0.0), (0, 2, 0.5), (0, 3, 0.5), (2, 0, 0.5)]
    maxe = meta["max_e"]
    step = sc2[16]
    nu_tot = tabs["tab_nu_tot"]
    K = 400
    for m, (gte, shr, fac) in enumerate(modes):
        lib.ref_set_collision_options(gte, shr, D(fac))
        # energies: log-uniform, a third of them above the highest threshold
        en = np.where(rng.random(K) < 0.35, rng.uniform(16.0, 0.95 * maxe, K), 10 ** rng.uniform(-3, np.log10(0.9 * maxe), K))
        if gte == 2:
            en = np.where(rng.random(K) < 0.5, 10 ** rng.uniform(-3, -0.8, K), en)
        d = rng.normal(size=(K, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        speed = np.sqrt(2.0 * en * C.ELECTRON_CHARGE / C.ELECTRON_MASS)
        vel = d * speed[:, None]
        energy = 0.5 * C.ELECTRON_MASS * ((vel[:, 0] ** 2 + vel[:, 1] ** 2) + vel[:, 2] ** 2) / C.ELECTRON_CHARGE
        idx = np.minimum((energy / step).astype(int) + 1, len(nu_tot) - 1)
        nu = np.maximum(nu_tot[idx], 1e3) * rng.uniform(1.0, 1.25, K)
        U = rng.uniform(1e-12, 1.0 - 1e-12, (K, 16))
        res = np.zeros((K, 11))
        used = np.zeros(K, np.int32)
        for k in range(K):
            u = np.ascontiguousarray(U[k])
            lib.ref_rng_replay(ptr(u), ctypes.c_size_t(16))
            o = np.zeros(11)
            p3 = np.zeros(3)
            v3 = vel[k].copy()
            lib.ref_collide(D(nu[k]), ptr(p3), ptr(v3), D(energy[k]), ptr(o))
            lib.ref_rng_consumed.restype = ctypes.c_size_t
            used[k] = lib.ref_rng_consumed()
            assert lib.ref_rng_overrun() == 0
            res[k] = o
        lib.ref_rng_replay_off()
        out.update({f"col{m}_opts": np.array([gte, shr, fac]), f"col{m}_nu": nu, f"col{m}_vel": vel,
                    f"col{m}_energy": energy, f"col{m}_u": U, f"col{m}_out": res, f"col{m}_used": used})

    # ---- statistical-error helper (MathFunctions.C:211-231) and histogram (MathFunctions.C:61-81)
    a = rng.normal(1.0, 0.1, 1237)
    out["staterr_in"] = a
    out["staterr_out"] = np.array(lib.ref_statistical_error(ptr(a), len(a), D(50.0)))
    x = rng.uniform(0, 12.0, 5000)
    nodes = np.linspace(0.0, 10.0, 101)
    cnt = np.zeros(100)
    lib.ref_histogram(ptr(x), len(x), ptr(nodes), len(nodes), ptr(cnt))
    out.update(hist_x=x, hist_nodes=nodes, hist_counts=cnt)
    np.savez_compressed(out_path, **out)


# ------------------------------------------------------------------ seeded solves

STAT_CASES = {
    # name: (gas case, overrides, numerics); 1e4 integration intervals of 1e5
    # electrons, so that the reference's own batch-means errors are a few
    # 0.01 % on the mean energy and the drift velocities; the reference's
    # default 1e4 table points (a coarser table moves the rates of processes
    # whose cross section jumps at threshold by up to ~1 %, depending on where
    # the threshold falls between the grid points of the run's own table)
    "atomic_dc100": ("atomic", {}, {"nIntegrationPoints": "1E4", "nInterpPoints": "10000",
                                    "maxCollisionsBeforeSteadyState": "1E3"}),
    "n2_dc200": ("n2", {}, {"nIntegrationPoints": "1E4", "nInterpPoints": "10000",
                            "maxCollisionsBeforeSteadyState": "300"}),
    "mix_dc100": ("mix", {}, {"nIntegrationPoints": "1E4", "nInterpPoints": "10000",
                              "maxCollisionsBeforeSteadyState": "300"}),
    # omega/N = 1e-14 m^3/s: a 20 ns field period, so the 1e4 integration
    # intervals (~0.1 ns each) average over some 50 periods
    "mix_ac150": ("mix", {"red_field": 150.0, "freq": 3.22e22 * 1e-14 / (2 * np.pi)},
                  {"nIntegrationPoints": "1E4", "nInterpPoints": "10000", "maxCollisionsBeforeSteadyState": "300",
                   "nIntegrationPhases": "64"}),
    "mix_b100": ("mix", {"red_field": 100.0, "red_mag": 1000.0, "angle": 90.0},
                 {"nIntegrationPoints": "1E4", "nInterpPoints": "10000", "maxCollisionsBeforeSteadyState": "300"}),
    # the field-complex batch's branches on the sweep's mixture: crossed DC
    # magnetic fields (E at 90 degrees to B along z) and an AC field of
    # 150 Td rms (omega/N = 1e-14 m^3/s: a 20 ns period, some 50 periods; at
    # fewer periods the time averages depend on where each run's window ends
    # within a period)
    "field_b500": ("sweep", {"red_field": 100.0, "red_mag": 500.0, "angle": 90.0},
                   {"nIntegrationPoints": "1E4", "nInterpPoints": "10000", "maxCollisionsBeforeSteadyState": "300"}),
    "field_b2000": ("sweep", {"red_field": 100.0, "red_mag": 2000.0, "angle": 90.0},
                    {"nIntegrationPoints": "1E4", "nInterpPoints": "10000", "maxCollisionsBeforeSteadyState": "300"}),
    "field_ac1e-14": ("sweep", {"red_field": 150.0, "freq": 3.22e22 * 1e-14 / (2 * np.pi)},
                      {"nIntegrationPoints": "1E4", "nInterpPoints": "10000", "maxCollisionsBeforeSteadyState": "300",
                       "nIntegrationPhases": "64"}),
    "n2_dc200_thermal": ("n2", {"gas_temp": "smartActivation"},
                         {"nIntegrationPoints": "1E4", "nInterpPoints": "10000",
                          "maxCollisionsBeforeSteadyState": "300"}),
}


def dist_record(lib, cells, eedf):
    """The reference's distributions as cumulative probabilities on sub-grids
    of its own cell nodes (tests/golden_util.py: cdf_at, eadf_mass,
    legendre_mass, evdf_cdf), compact enough to commit."""
    import golden_util as gu

    sz = np.zeros(7, np.int32)
    lib.ref_dist_sizes(sz.ctypes.data_as(VP))
    nE, nC, nR, nA, nPh, cyl, ac = (int(x) for x in sz)
    nodes = gu.energy_nodes(cells)
    e_edges = nodes[::5]
    rec = dict(e_edges=e_edges, eedf_cdf=gu.cdf_at(nodes, gu.eedf_mass(cells, eedf), e_edges))
    if cyl:
        f1, f2 = np.zeros(nE), np.zeros(nE)
        eadf, evdf = np.zeros(nE * nC), np.zeros(nR * nA)
        rc, acc = np.zeros(nR), np.zeros(nA)
        lib.ref_get_anisotropic(ptr(f1), ptr(f2), ptr(eadf), ptr(evdf), ptr(rc), ptr(acc))
        rec["eadf_cdf"] = gu.cdf_at(nodes, gu.eadf_mass(cells, eadf.reshape(nE, nC), 10), e_edges)
        rec["f1_cdf"] = gu.cdf_at(nodes, gu.legendre_mass(cells, f1, 1), e_edges)
        rec["f2_cdf"] = gu.cdf_at(nodes, gu.legendre_mass(cells, f2, 2), e_edges)
        dr, dz = rc[1] - rc[0], acc[1] - acc[0]
        r_edges = (np.arange(nR + 1) * dr)[::4]
        z_edges = (acc[0] - 0.5 * dz + np.arange(nA + 1) * dz)[::4]
        rec.update(r_edges=r_edges, z_edges=z_edges,
                   evdf_cdf=gu.evdf_cdf(rc, acc, evdf.reshape(nR, nA), r_edges, z_edges))
    if ac:
        n, me = np.zeros(nPh), np.zeros(nPh)
        fv, bv, fd, bd = np.zeros(3 * nPh), np.zeros(3 * nPh), np.zeros(9 * nPh), np.zeros(9 * nPh)
        per = np.zeros(nPh * nE)
        lib.ref_get_periodic(ptr(n), ptr(me), ptr(fv), ptr(bv), ptr(fd), ptr(bd), ptr(per))
        per = per.reshape(nPh, nE)
        pe = e_edges[::2]
        rec.update(per_n=n, per_mean_energy=me, per_flux_v=fv.reshape(nPh, 3), per_bulk_v=bv.reshape(nPh, 3),
                   per_flux_d=fd.reshape(nPh, 9), per_bulk_d=bd.reshape(nPh, 9), per_e_edges=pe,
                   per_eedf_cdf=np.stack([gu.cdf_at(nodes, gu.eedf_mass(cells, per[q]), pe) for q in range(nPh)]))
    return rec


def run_stats(name, out_path, seed, n_electrons):
    out_path = os.path.abspath(out_path)  # open_ref changes the working directory
    case, over, numerics = STAT_CASES[name]
    tmp = tempfile.mkdtemp(prefix=f"stats_{name}_")
    gases, meta, setup = write_inputs(case, tmp, n_electrons=n_electrons, extra=numerics, **over)
    lib = open_ref(tmp, setup)
    lib.ref_rng_seed(ctypes.c_uint64(seed))
    P = lib.ref_n_processes()
    r = np.zeros(39)
    rate = np.zeros(P)
    lib.ref_solve(ptr(r), ptr(rate))
    nc = lib.ref_n_eedf_cells()
    cells, eedf = np.zeros(nc), np.zeros(nc)
    lib.ref_get_eedf(ptr(cells), ptr(eedf))
    gain, loss = np.zeros(P), np.zeros(P)
    lib.ref_get_power(ptr(gain), ptr(loss))
    rec = dict(case=case, overrides={k: v for k, v in over.items()}, numerics=numerics, n_electrons=n_electrons,
               seed=seed, result=r.tolist(), rate=rate.tolist(), power_gain=gain.tolist(), power_loss=loss.tolist(),
               eedf_cells=cells.tolist(), eedf=eedf.tolist())
    with open(out_path, "w") as f:
        json.dump(rec, f)
    np.savez_compressed(out_path[:-5] + "_dist.npz", **dist_record(lib, cells, eedf))


def _child(args):
    kind, name, path, seed, ne = args
    if kind == "kin":
        run_case(name, path, seed)
    else:
        run_stats(name, path, seed, ne)
    return path


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--stats", action="store_true")
    ap.add_argument("--stats-only", action="store_true", help="only the seeded solves")
    ap.add_argument("--only", default=None)
    ap.add_argument("--ne", type=float, default=1e5)
    a = ap.parse_args()
    if a.stats_only:
        a.stats = True
    jobs = []
    for i, name in enumerate(("atomic", "n2", "mix", "screen")):
        if a.stats_only or (a.only and name != a.only):
            continue
        jobs.append(("kin", name, os.path.join(HERE, f"kin_{name}.npz"), 1000 + i, 0))
    if a.stats:
        for i, name in enumerate(STAT_CASES):
            if a.only and name != a.only:
                continue
            jobs.append(("stats", name, os.path.join(HERE, f"stats_{name}.json"), 77 + i, a.ne))
    # the seeded solves use every core (OpenMP), one after the other
    ctx = mp.get_context("spawn")
    with ctx.Pool(1 if a.stats else min(len(jobs), 4)) as pool:
        for p in pool.imap_unordered(_child, jobs):
            print("wrote", os.path.relpath(p, ROOT))


if __name__ == "__main__":
    main()
