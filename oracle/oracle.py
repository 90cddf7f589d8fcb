"""ctypes front end of the CPU oracle (oracle/loki_oracle.c).

TEST INFRASTRUCTURE, NOT PRODUCT: imported only by the tests, the smoke check
and the CPU-baseline leg of the benchmark, as the reference results the GPU
path is compared with (never as the thing measured or shipped).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblokioracle.so")
SRC = os.path.join(HERE, "loki_oracle.c")

D = ctypes.c_double
I = ctypes.c_int
P_ = ctypes.POINTER


def build(force: bool = False) -> str:
    """Compiles the oracle with the host C compiler (-O2, OpenMP, no FMA contraction)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-ffp-contract=off", "-shared", SRC, "-o",
                               LIB_PATH, "-lm"])
    return LIB_PATH


class Rng(ctypes.Structure):
    _fields_ = [("s", ctypes.c_uint64 * 4), ("replay", P_(D)), ("n", ctypes.c_size_t), ("pos", ctypes.c_size_t),
                ("overrun", I)]


class Procs(ctypes.Structure):
    _fields_ = [("P", I), ("G", I), ("ptype", P_(I)), ("is_super", P_(I)), ("sampler", P_(I)),
                ("sampler_p0", P_(D)), ("sampler_p1", P_(D)), ("superw", P_(D)), ("emin", P_(D)), ("emax", P_(D)),
                ("rel_dens", P_(D)), ("mass", P_(D)), ("red_mass", P_(D)), ("eloss", P_(D)), ("wparam", P_(D)),
                ("raw_off", P_(I)), ("raw_len", P_(I)), ("raw_e", P_(D)), ("raw_v", P_(D)), ("gas_first", P_(I)),
                ("gas_last", P_(I)), ("gas_frac", P_(D)), ("energy_max_elastic", D), ("M", I), ("max_interp", D),
                ("step", D), ("grid", P_(D)), ("sig", P_(D)), ("cum", P_(D)), ("nu_tot", P_(D)), ("nu_max", P_(D))]


class Fields(ctypes.Structure):
    _fields_ = [("N", D), ("Tg", D), ("gas_energy", D), ("E", D * 3), ("acc", D * 3), ("freq_hz", D), ("omega", D),
                ("red_mag", D), ("omega_c", D), ("gas_temp_effect", I), ("sharing", I), ("sharing_factor", D)]


class CollOut(ctypes.Structure):
    _fields_ = [("chosen", I), ("vel", D * 3), ("energy", D), ("dE", D), ("dE_over_E", D), ("ej_vel", D * 3),
                ("ej_energy", D)]


class RunConfig(ctypes.Structure):
    _fields_ = [("n_electrons", I), ("n_threads", I), ("seed", ctypes.c_uint64), ("init_temp_ratio", D),
                ("sync_x", D), ("sync_oversampling", I), ("min_coll_before_ss", D), ("max_coll_before_ss", D),
                ("max_coll_after_ss", D), ("req_integration_points", D), ("req_ss_times", D), ("req_abs_time", D),
                ("errors_checked", I), ("req_err_energy", D), ("req_err_flux_v", D), ("req_err_flux_d", D),
                ("req_err_bulk_v", D), ("req_err_bulk_d", D), ("req_err_power", D), ("n_energy_cells", I),
                ("n_cos_cells", I), ("n_radial_cells", I), ("n_axial_cells", I), ("n_phases", I),
                ("cylindrical", I), ("max_seconds", D), ("max_sync_steps", ctypes.c_longlong),
                ("mark_sync_step", ctypes.c_longlong), ("mark_seconds", D)]


class RunResult(ctypes.Structure):
    _fields_ = [("mean_energy", D), ("mean_energy_err", D), ("flux_v", D * 3), ("flux_v_err", D * 3),
                ("flux_d", D * 9), ("flux_d_err", D * 9), ("bulk_v", D * 3), ("bulk_v_err", D * 3),
                ("bulk_d", D * 9), ("bulk_d_err", D * 9), ("real_collisions", D), ("null_collisions", D),
                ("coll_at_ss", D), ("null_at_ss", D), ("ss_time", D), ("final_time", D),
                ("integration_points", D), ("trial_freq", D), ("power_field", D), ("power_growth", D),
                ("power_balance_rel_err", D), ("max_eedf_energy", D), ("elapsed", D),
                ("sync_steps", ctypes.c_longlong), ("mark_real_collisions", D), ("mark_null_collisions", D),
                ("mark_elapsed", D), ("mark_sync_steps", ctypes.c_longlong), ("status", I)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.lo_uniform.restype = D
        _lib.lo_interp.restype = D
        _lib.lo_max_accel_energy.restype = D
        _lib.lo_statistical_error.restype = D
        _lib.lo_run.restype = I
    return _lib


def _p(a, t):
    return a.ctypes.data_as(P_(t))


class OracleProcs:
    """Owns the numpy buffers behind a Procs struct."""

    def __init__(self, arrays: dict, M: int):
        a = {}
        for k in ("ptype", "is_super", "sampler", "raw_off", "raw_len", "gas_first", "gas_last"):
            a[k] = np.ascontiguousarray(arrays[k], dtype=np.int32)
        for k in ("sampler_p0", "sampler_p1", "superw", "emin", "emax", "rel_dens", "mass", "red_mass", "eloss",
                  "wparam", "raw_e", "raw_v", "gas_frac"):
            a[k] = np.ascontiguousarray(arrays[k], dtype=np.float64)
        P = len(a["ptype"])
        self.P, self.M = P, M
        self.grid = np.zeros(M)
        self.sig = np.zeros(M * P)
        self.cum = np.zeros(M * P)
        self.nu_tot = np.zeros(M)
        self.nu_max = np.zeros(M)
        self.a = a
        s = Procs()
        s.P, s.G = P, len(a["gas_first"])
        for k in ("ptype", "is_super", "sampler", "raw_off", "raw_len", "gas_first", "gas_last"):
            setattr(s, k, _p(a[k], I))
        for k in ("sampler_p0", "sampler_p1", "superw", "emin", "emax", "rel_dens", "mass", "red_mass", "eloss",
                  "wparam", "raw_e", "raw_v", "gas_frac"):
            setattr(s, k, _p(a[k], D))
        s.energy_max_elastic = float(arrays["energy_max_elastic"])
        s.M = M
        s.max_interp = -1.0
        s.step = 0.0
        for k in ("grid", "sig", "cum", "nu_tot", "nu_max"):
            setattr(s, k, _p(getattr(self, k), D))
        self.s = s

    def build_tables(self, fields: Fields, max_energy: float):
        lib().lo_build_tables(ctypes.byref(self.s), ctypes.byref(fields), D(max_energy))


def make_fields(N, Tg=300.0, E=(0.0, 0.0, 0.0), freq_hz=0.0, red_mag=0.0, omega_c=0.0, gas_temp_effect=0,
                sharing=0, sharing_factor=0.5) -> Fields:
    f = Fields()
    f.N, f.Tg = N, Tg
    f.gas_energy = 1.5 * 1.38064852e-23 * Tg / 1.6021766208e-19
    for k in range(3):
        f.E[k] = E[k]
        f.acc[k] = -1.6021766208e-19 / 9.10938356e-31 * E[k]
    f.freq_hz = freq_hz
    f.omega = freq_hz * 2.0 * np.pi
    f.red_mag = red_mag
    f.omega_c = omega_c
    f.gas_temp_effect = gas_temp_effect
    f.sharing = sharing
    f.sharing_factor = sharing_factor
    return f


def accelerate(fields: Fields, t, dt, pos, vel, energy):
    p = np.ascontiguousarray(pos, dtype=np.float64).copy()
    v = np.ascontiguousarray(vel, dtype=np.float64).copy()
    e = D(energy)
    g = D(0.0)
    lib().lo_accelerate(ctypes.byref(fields), D(t), D(dt), _p(p, D), _p(v, D), ctypes.byref(e), ctypes.byref(g))
    return p, v, e.value, g.value


def collide(procs: OracleProcs, fields: Fields, nu_trial, vel, energy, uniforms):
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    r = Rng()
    lib().lo_rng_replay(ctypes.byref(r), _p(u, D), ctypes.c_size_t(len(u)))
    v = np.ascontiguousarray(vel, dtype=np.float64)
    o = CollOut()
    lib().lo_collide(ctypes.byref(procs.s), ctypes.byref(fields), D(nu_trial), _p(v, D), D(energy),
                     ctypes.byref(r), ctypes.byref(o))
    out = np.array([o.chosen, o.vel[0], o.vel[1], o.vel[2], o.energy, o.dE, o.dE_over_E, o.ej_vel[0], o.ej_vel[1],
                    o.ej_vel[2], o.ej_energy])
    return out, int(r.pos), int(r.overrun)


def statistical_error(a, nbins=50.0):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return lib().lo_statistical_error(_p(a, D), len(a), D(nbins))


def default_run_config(n_electrons, **kw) -> RunConfig:
    c = RunConfig()
    c.n_electrons = int(n_electrons)
    c.n_threads = 1
    c.seed = 1
    c.init_temp_ratio = 0.01
    c.sync_x = 1.0
    c.sync_oversampling = 1
    c.min_coll_before_ss = 0.0
    c.max_coll_before_ss = 1e100
    c.max_coll_after_ss = 1e100
    c.req_integration_points = 200
    c.req_ss_times = 0
    c.req_abs_time = 0
    c.errors_checked = 0
    for k in ("req_err_energy", "req_err_flux_v", "req_err_flux_d", "req_err_bulk_v", "req_err_bulk_d",
              "req_err_power"):
        setattr(c, k, 1e100)
    c.n_energy_cells = 1000
    c.n_cos_cells = 100
    c.n_radial_cells = 200
    c.n_axial_cells = 200
    c.n_phases = 100
    c.cylindrical = 1
    c.max_seconds = 0
    c.max_sync_steps = 0
    c.mark_sync_step = 0
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def run(procs: OracleProcs, fields: Fields, cfg: RunConfig):
    res = RunResult()
    P = procs.P
    rate = np.zeros(P)
    pg = np.zeros(P)
    pl = np.zeros(P)
    eedf = np.zeros(cfg.n_energy_cells)
    cells = np.zeros(cfg.n_energy_cells)
    st = lib().lo_run(ctypes.byref(procs.s), ctypes.byref(fields), ctypes.byref(cfg), ctypes.byref(res),
                      _p(rate, D), _p(pg, D), _p(pl, D), _p(eedf, D), _p(cells, D))
    return st, res, dict(rate=rate, power_gain=pg, power_loss=pl, eedf=eedf, eedf_cells=cells)
