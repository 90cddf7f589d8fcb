"""ctypes binding of the C ABI in include/loki_gpu.h (libloki_gpu.so).

Only plain C types cross the boundary. A missing library or a failing call
raises; there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB_NAME = "libloki_gpu.so"

D = ctypes.c_double
I = ctypes.c_int
LL = ctypes.c_longlong
U64 = ctypes.c_uint64
P_ = ctypes.POINTER

LGPU_OK = 0
STATUS = {0: "OK", 1: "BAD_ARG", 2: "OOM", 3: "ENERGY_ABOVE_TABLE", 4: "TIMEOUT", 5: "CUDA_ERROR", 6: "STATE",
          7: "OVERFLOW", 8: "NO_DEVICE"}

EXPORTED = ("lgpu_config_default", "lgpu_create", "lgpu_destroy", "lgpu_last_error", "lgpu_stream",
            "lgpu_set_processes", "lgpu_set_conditions", "lgpu_init_ensemble", "lgpu_advance", "lgpu_solve",
            "lgpu_get_process_results", "lgpu_get_distributions", "lgpu_get_periodic", "lgpu_get_series",
            "lgpu_get_timing", "lgpu_set_twoterm", "lgpu_eedf_postprocess", "lgpu_eedf_rates",
            "lgpu_build_tables", "lgpu_set_field_raw", "lgpu_replay_flights", "lgpu_replay_collisions",
            "lgpu_replay_collisions_coarse", "lgpu_replay_flights_noalloc",
            "lgpu_batch_create", "lgpu_batch_destroy", "lgpu_batch_last_error", "lgpu_batch_add", "lgpu_batch_run",
            "lgpu_batch_start", "lgpu_batch_step", "lgpu_batch_stream", "lgpu_batch_set_schedule",
            "lgpu_server_start", "lgpu_server_submit", "lgpu_server_poll", "lgpu_server_wait",
            "lgpu_server_job_rates", "lgpu_server_job_eedf", "lgpu_server_cancel", "lgpu_server_forget", "lgpu_server_report_get", "lgpu_server_last_error",
            "lgpu_server_stop",
            "lgpu_request_parse", "lgpu_request_jobs", "lgpu_request_job", "lgpu_request_free",
            "lgpu_server_submit_request")

JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED, JOB_CANCELLED = 0, 1, 2, 3, 4


class LokiGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("device", I), ("seed", U64), ("n_electrons", D), ("n_interp", I), ("gas_temperature_effect", I),
                ("sharing", I), ("init_temp_ratio", D), ("min_coll_before_ss", D), ("max_coll_before_ss", D),
                ("max_coll_after_ss", D), ("req_integration_points", D), ("req_ss_times", D), ("req_abs_time", D),
                ("errors_checked", I), ("req_err_mean_energy", D), ("req_err_flux_v", D), ("req_err_flux_d", D),
                ("req_err_bulk_v", D), ("req_err_bulk_d", D), ("req_err_power", D), ("n_energy_cells", I),
                ("n_cos_cells", I), ("n_radial_cells", I), ("n_axial_cells", I), ("n_phases", I), ("sync_x", D),
                ("sync_oversampling", I), ("max_seconds", D), ("max_sync_steps", LL), ("advance_real_batch", I),
                ("advance_queue", I)]


class Process(ctypes.Structure):
    _fields_ = [("type", I), ("is_super", I), ("is_elastic", I), ("sampler", I), ("sampler_p0", D),
                ("sampler_p1", D), ("superw", D), ("emin", D), ("emax", D), ("rel_dens", D), ("mass", D),
                ("eloss", D), ("wparam", D), ("raw_len", I), ("raw_e", P_(D)), ("raw_v", P_(D))]


class Gas(ctypes.Structure):
    _fields_ = [("first", I), ("last", I), ("fraction", D)]


class Conditions(ctypes.Structure):
    _fields_ = [("gas_density", D), ("gas_temperature", D), ("reduced_field_td", D), ("field_angle_deg", D),
                ("excitation_freq_hz", D), ("reduced_mag_field_hx", D)]


class Result(ctypes.Structure):
    _fields_ = [("mean_energy", D), ("mean_energy_err", D), ("flux_v", D * 3), ("flux_v_err", D * 3),
                ("flux_d", D * 9), ("flux_d_err", D * 9), ("bulk_v", D * 3), ("bulk_v_err", D * 3),
                ("bulk_d", D * 9), ("bulk_d_err", D * 9), ("power_field", D), ("power_growth", D),
                ("power_balance_rel_err", D), ("ss_time", D), ("final_time", D), ("trial_freq", D),
                ("max_eedf_energy", D), ("real_collisions", D), ("null_collisions", D), ("coll_at_ss", D),
                ("null_at_ss", D), ("integration_points", LL), ("sampling_points", LL),
                ("first_integration_index", LL), ("sync_steps", LL), ("elapsed", D), ("capped", I)]


class StepReport(ctypes.Structure):
    _fields_ = [("time", D), ("trial_freq", D), ("max_energy", D), ("mean_energy", D), ("real_collisions", D),
                ("null_collisions", D), ("sync_steps", LL)]


class Timing(ctypes.Structure):
    _fields_ = [("advance_ms", D), ("advance_launches", LL), ("electron_steps", D), ("kernel_launches", LL),
                ("h2d_bytes", D), ("d2h_bytes", D)]


class TwotermProcess(ctypes.Structure):
    _fields_ = [("kind", I), ("ion", I), ("density", D), ("threshold", D), ("mass_ratio", D), ("stat_ratio", D),
                ("n_int", I), ("n_mom", I), ("int_e", P_(D)), ("int_v", P_(D)), ("mom_e", P_(D)),
                ("mom_v", P_(D))]


# lgpu_eedf_params, in field order, with the reference's swarmParam keys
EEDF_PARAM_KEYS = ("totalIonRateCoeff", "totalAttRateCoeff", "momTransfFreq", "energyRelaxFreq",
                   "energyRelaxFreqClassic", "redDiffCoeffEnergy_eedf", "redMobCoeffEnergy_eedf", "redDiffCoeff_eedf",
                   "redMobCoeff_DC_eedf", "characEnergy_eedf", "redMobCoeff_xx_real_eedf",
                   "redMobCoeff_xx_imag_eedf", "redMobCoeff_xy_real_eedf", "redMobCoeff_xy_imag_eedf",
                   "redMobCoeff_zz_real_eedf", "redMobCoeff_zz_imag_eedf")


class EedfParams(ctypes.Structure):
    _fields_ = [(k, D) for k in ("tot_ion_rate", "tot_att_rate", "mom_transf_freq", "energy_relax_freq",
                                 "energy_relax_freq_classic", "red_diff_energy", "red_mob_energy", "red_diff",
                                 "red_mob_dc", "charac_energy", "red_mob_xx_re", "red_mob_xx_im", "red_mob_xy_re",
                                 "red_mob_xy_im", "red_mob_zz_re", "red_mob_zz_im")]

    def values(self):
        return np.array([getattr(self, f[0]) for f in self._fields_])


def twoterm_array(procs):
    """(lgpu_twoterm_process array, arrays it points into) from dicts with
    kind (0 elastic, 1 inelastic, 2 superelastic copy), ion (1 ionization,
    2 attachment), density, threshold, mass_ratio, stat_ratio and the raw
    tables int_e, int_v, mom_e, mom_v (mom_* may be absent: the integral
    table)."""
    arr = (TwotermProcess * len(procs))()
    keep = []
    for k, q in enumerate(procs):
        t = arr[k]
        t.kind, t.ion = int(q["kind"]), int(q.get("ion", 0))
        t.density, t.threshold = float(q["density"]), float(q["threshold"])
        t.mass_ratio, t.stat_ratio = float(q.get("mass_ratio", 0.0)), float(q.get("stat_ratio", 0.0))
        tabs = [np.ascontiguousarray(q[n], dtype=np.float64) for n in ("int_e", "int_v")]
        if q.get("mom_e") is not None:
            tabs += [np.ascontiguousarray(q[n], dtype=np.float64) for n in ("mom_e", "mom_v")]
        keep.append(tabs)
        t.n_int = len(tabs[0])
        t.int_e, t.int_v = tabs[0].ctypes.data_as(P_(D)), tabs[1].ctypes.data_as(P_(D))
        if len(tabs) == 4:
            t.n_mom = len(tabs[2])
            t.mom_e, t.mom_v = tabs[2].ctypes.data_as(P_(D)), tabs[3].ctypes.data_as(P_(D))
    return arr, keep


class BatchReport(ctypes.Structure):
    _fields_ = [("intervals", LL), ("kernel_launches", LL), ("elapsed", D), ("real_collisions", D),
                ("null_collisions", D), ("advance_ms", D), ("electron_steps", D), ("h2d_bytes", D),
                ("d2h_bytes", D), ("host_ms", D), ("secondaries", D), ("spilled", D), ("attached", D),
                ("real_batch", D), ("coarse_null_test", D), ("regrids", D), ("advance_threads", D),
                ("advance_blocks_per_sm", D), ("advance_chunk", D), ("advance_stash", D)]


class Job(ctypes.Structure):
    _fields_ = [("config", Config), ("procs", P_(Process)), ("n_procs", I), ("gases", P_(Gas)), ("n_gases", I),
                ("emax_elastic", D), ("conditions", Conditions), ("twoterm", P_(TwotermProcess))]


class JobStatus(ctypes.Structure):
    _fields_ = [("state", I), ("status", I), ("submit_time", D), ("start_time", D), ("end_time", D),
                ("footprint_bytes", D), ("result", Result), ("error", ctypes.c_char * 256)]


class ServerReport(ctypes.Structure):
    _fields_ = [("submitted", LL), ("completed", LL), ("failed", LL), ("running", LL), ("queued", LL),
                ("intervals", LL), ("real_collisions", D), ("null_collisions", D), ("busy_seconds", D),
                ("peak_footprint_bytes", D)]


_lib = None


def library_path() -> str:
    return os.path.join(PKG_DIR, LIB_NAME)


def load(path: str | None = None):
    """Loads libloki_gpu.so (built by ``lokigpu.build``); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or library_path()
    if not os.path.exists(p):
        raise LokiGpuError(8, f"{p} is missing: build it with __graft_entry__.build() or lokigpu.build.build()")
    lib = ctypes.CDLL(p)
    lib.lgpu_config_default.argtypes = [P_(Config)]
    lib.lgpu_config_default.restype = None
    lib.lgpu_create.argtypes = [P_(Config), P_(ctypes.c_void_p)]
    lib.lgpu_destroy.argtypes = [ctypes.c_void_p]
    lib.lgpu_last_error.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    lib.lgpu_stream.argtypes = [ctypes.c_void_p]
    lib.lgpu_stream.restype = ctypes.c_void_p
    lib.lgpu_set_processes.argtypes = [ctypes.c_void_p, P_(Process), I, P_(Gas), I, D]
    lib.lgpu_set_conditions.argtypes = [ctypes.c_void_p, P_(Conditions)]
    lib.lgpu_init_ensemble.argtypes = [ctypes.c_void_p]
    lib.lgpu_advance.argtypes = [ctypes.c_void_p, I, P_(StepReport)]
    lib.lgpu_solve.argtypes = [ctypes.c_void_p, P_(Result)]
    lib.lgpu_get_process_results.argtypes = [ctypes.c_void_p, P_(ctypes.c_ulonglong), P_(D), P_(D), P_(D), I]
    lib.lgpu_get_distributions.argtypes = [ctypes.c_void_p] + [P_(D)] * 9
    lib.lgpu_set_twoterm.argtypes = [ctypes.c_void_p, P_(TwotermProcess), I]
    lib.lgpu_eedf_postprocess.argtypes = [ctypes.c_void_p, P_(D), I, D, P_(EedfParams), P_(D), I]
    lib.lgpu_eedf_rates.argtypes = [ctypes.c_void_p, P_(D), I, I, D, P_(D), I]
    lib.lgpu_get_periodic.argtypes = [ctypes.c_void_p] + [P_(D)] * 6
    lib.lgpu_get_series.argtypes = [ctypes.c_void_p, I, P_(D), LL]
    lib.lgpu_get_series.restype = LL
    lib.lgpu_get_timing.argtypes = [ctypes.c_void_p, P_(Timing)]
    lib.lgpu_build_tables.argtypes = [ctypes.c_void_p, D, P_(D), P_(D), P_(ctypes.c_float), P_(ctypes.c_float)]
    lib.lgpu_set_field_raw.argtypes = [ctypes.c_void_p, P_(D), D, D, D]
    lib.lgpu_replay_flights.argtypes = [ctypes.c_void_p, I] + [P_(D)] * 8
    lib.lgpu_replay_collisions.argtypes = [ctypes.c_void_p, I, P_(D), P_(D), P_(D), P_(D), I, P_(D), P_(I)]
    lib.lgpu_replay_collisions_coarse.argtypes = lib.lgpu_replay_collisions.argtypes
    lib.lgpu_replay_flights_noalloc.argtypes = [I, P_(D), D, D, D, I] + [P_(D)] * 8
    VP = ctypes.c_void_p
    lib.lgpu_batch_create.argtypes = [I, I, P_(VP)]
    lib.lgpu_batch_destroy.argtypes = [VP]
    lib.lgpu_batch_last_error.argtypes = [VP, ctypes.c_char_p, ctypes.c_size_t]
    lib.lgpu_batch_add.argtypes = [VP, VP]
    lib.lgpu_batch_run.argtypes = [VP, P_(Result), P_(I), I, P_(BatchReport)]
    lib.lgpu_batch_start.argtypes = [VP]
    lib.lgpu_batch_step.argtypes = [VP, I, P_(I), P_(BatchReport)]
    lib.lgpu_batch_stream.argtypes = [VP]
    lib.lgpu_batch_stream.restype = VP
    lib.lgpu_batch_set_schedule.argtypes = [VP, I, I, I]
    lib.lgpu_server_start.argtypes = [I, I, D, P_(VP)]
    lib.lgpu_server_submit.argtypes = [VP, P_(Job), P_(LL)]
    lib.lgpu_server_poll.argtypes = [VP, LL, P_(JobStatus)]
    lib.lgpu_server_wait.argtypes = [VP, LL, D, P_(JobStatus)]
    lib.lgpu_server_job_rates.argtypes = [VP, LL, P_(ctypes.c_ulonglong), P_(D), I]
    lib.lgpu_server_job_eedf.argtypes = [VP, LL, P_(EedfParams), P_(D), I]
    lib.lgpu_server_cancel.argtypes = [VP, LL]
    lib.lgpu_server_forget.argtypes = [VP, LL]
    lib.lgpu_server_report_get.argtypes = [VP, P_(ServerReport)]
    lib.lgpu_server_last_error.argtypes = [VP, ctypes.c_char_p, ctypes.c_size_t]
    lib.lgpu_server_stop.argtypes = [VP]
    CP = ctypes.c_char_p
    lib.lgpu_request_parse.argtypes = [CP, I, P_(CP), P_(CP), P_(VP), CP, ctypes.c_size_t]
    lib.lgpu_request_jobs.argtypes = [VP]
    lib.lgpu_request_job.argtypes = [VP, I, P_(Job)]
    lib.lgpu_request_free.argtypes = [VP]
    lib.lgpu_request_free.restype = None
    lib.lgpu_server_submit_request.argtypes = [VP, VP, P_(LL), I]
    _lib = lib
    return lib


def dptr(a):
    return None if a is None else a.ctypes.data_as(P_(D))


def default_config(**kw) -> Config:
    c = Config()
    load().lgpu_config_default(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def replay_flights_noalloc(device, E, freq_hz, red_mag, cyclotron, t, dt, pos, vel):
    """lgpu_replay_flights_noalloc: free flights staged through the library's
    static device array, without a context or any device allocation."""
    lib = load()
    n = len(t)
    t = np.ascontiguousarray(t, np.float64)
    dt = np.ascontiguousarray(dt, np.float64)
    pos = np.ascontiguousarray(pos, np.float64).reshape(n, 3)
    vel = np.ascontiguousarray(vel, np.float64).reshape(n, 3)
    e = np.ascontiguousarray(E, np.float64)
    po, vo, eo, go = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n), np.zeros(n)
    rc = lib.lgpu_replay_flights_noalloc(int(device), dptr(e), float(freq_hz), float(red_mag), float(cyclotron), n,
                                         dptr(t), dptr(dt), dptr(pos), dptr(vel), dptr(po), dptr(vo), dptr(eo), dptr(go))
    if rc != LGPU_OK:
        raise LokiGpuError(rc, "lgpu_replay_flights_noalloc failed")
    return po, vo, eo, go


def _struct_dtype(st):
    """A numpy record type with the layout of a ctypes structure of ints,
    doubles and pointers (pointers as unsigned addresses)."""
    names, formats, offsets = [], [], []
    for name, ct in st._fields_:
        names.append(name)
        formats.append(np.int32 if ct is I else (np.float64 if ct is D else np.uintp))
        offsets.append(getattr(st, name).offset)
    return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": ctypes.sizeof(st)})


_PROCESS_DTYPE = None


def process_arrays(ps, gas_first, gas_last, gas_fraction):
    """lgpu_process / lgpu_gas arrays of a ProcessSet-like object (see
    synth.ProcessSet); the third value holds the arrays the structs point to.
    The records are filled column by column (a mixture of 65 processes in
    tens of microseconds, where a per-field loop took about half a
    millisecond per context)."""
    global _PROCESS_DTYPE
    if _PROCESS_DTYPE is None:
        _PROCESS_DTYPE = _struct_dtype(Process)
    n = ps.n
    rec = np.zeros(n, dtype=_PROCESS_DTYPE)
    for name, src, t in (("type", ps.ptype, np.int32), ("is_super", ps.is_super, np.int32),
                         ("is_elastic", ps.is_elastic, np.int32), ("sampler", ps.sampler, np.int32),
                         ("sampler_p0", ps.sampler_p0, np.float64), ("sampler_p1", ps.sampler_p1, np.float64),
                         ("superw", ps.superw, np.float64), ("emin", ps.emin, np.float64),
                         ("emax", ps.emax, np.float64), ("rel_dens", ps.rel_dens, np.float64),
                         ("mass", ps.mass, np.float64), ("eloss", ps.eloss, np.float64),
                         ("wparam", ps.wparam, np.float64)):
        rec[name] = np.asarray(src, dtype=t)[:n]
    raw_e = [np.ascontiguousarray(x, dtype=np.float64).ravel() for x in ps.raw_e[:n]]
    raw_v = [np.ascontiguousarray(x, dtype=np.float64).ravel() for x in ps.raw_v[:n]]
    len_e = np.array([len(x) for x in raw_e], dtype=np.int64)
    len_v = np.array([len(x) for x in raw_v], dtype=np.int64)
    e_all = np.concatenate(raw_e + [np.zeros(1)])
    v_all = np.concatenate(raw_v + [np.zeros(1)])
    off_e = np.concatenate([[0], np.cumsum(len_e)[:-1]]) if n else np.zeros(0, np.int64)
    off_v = np.concatenate([[0], np.cumsum(len_v)[:-1]]) if n else np.zeros(0, np.int64)
    rec["raw_len"] = np.where(np.asarray(ps.is_super[:n]) != 0, 0, len_e).astype(np.int32)
    rec["raw_e"] = e_all.ctypes.data + 8 * off_e.astype(np.uint64)
    rec["raw_v"] = v_all.ctypes.data + 8 * off_v.astype(np.uint64)
    arr = rec.ctypes.data_as(P_(Process))
    G = len(gas_first)
    gs = (Gas * G)()
    for g in range(G):
        gs[g].first = int(gas_first[g])
        gs[g].last = int(gas_last[g])
        gs[g].fraction = float(gas_fraction[g])
    return arr, gs, [rec, e_all, v_all]


class Context:
    """Owns one lgpu_ctx (one swarm condition)."""

    def __init__(self, cfg: Config):
        self.lib = load()
        self.h = ctypes.c_void_p()
        rc = self.lib.lgpu_create(ctypes.byref(cfg), ctypes.byref(self.h))
        self.cfg = cfg
        self._keep = []
        self.check(rc)

    def last_error(self) -> str:
        buf = ctypes.create_string_buffer(1024)
        self.lib.lgpu_last_error(self.h, buf, 1024)
        return buf.value.decode(errors="replace")

    def check(self, rc):
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())

    def close(self):
        if self.h:
            self.lib.lgpu_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_processes(self, ps, gas_first, gas_last, gas_fraction):
        """ps: a ProcessSet-like object (see synth.ProcessSet)."""
        arr, gs, keep = process_arrays(ps, gas_first, gas_last, gas_fraction)
        self._keep = keep
        self.check(self.lib.lgpu_set_processes(self.h, arr, ps.n, gs, len(gas_first), float(ps.energy_max_elastic)))
        self.P = ps.n

    def set_conditions(self, N, Tg=300.0, red_field=0.0, angle=180.0, freq_hz=0.0, red_mag=0.0):
        c = Conditions(N, Tg, red_field, angle, freq_hz, red_mag)
        self.check(self.lib.lgpu_set_conditions(self.h, ctypes.byref(c)))

    def init_ensemble(self):
        self.check(self.lib.lgpu_init_ensemble(self.h))

    def advance(self, n):
        r = StepReport()
        self.check(self.lib.lgpu_advance(self.h, int(n), ctypes.byref(r)))
        return r

    def solve(self) -> Result:
        r = Result()
        self.check(self.lib.lgpu_solve(self.h, ctypes.byref(r)))
        return r

    def process_results(self):
        P = self.P
        cnt = (ctypes.c_ulonglong * P)()
        rate, gain, loss = np.zeros(P), np.zeros(P), np.zeros(P)
        self.check(self.lib.lgpu_get_process_results(self.h, cnt, dptr(rate), dptr(gain), dptr(loss), P))
        return np.array(cnt[:], dtype=np.uint64), rate, gain, loss

    def set_twoterm(self, procs):
        """The collision behind each MC process for the EEDF post-processing
        (see twoterm_array)."""
        arr, keep = twoterm_array(procs)
        self.check(self.lib.lgpu_set_twoterm(self.h, arr, len(procs)))
        del keep

    def eedf_postprocess(self, eedf=None, max_energy=0.0):
        """(EedfParams, rates): the EEDF-convolved rate coefficients and the
        two-term swarm parameters, on the device, of the given EEDF or (None)
        the context's own."""
        out = EedfParams()
        rate = np.zeros(self.P)
        if eedf is None:
            self.check(self.lib.lgpu_eedf_postprocess(self.h, None, 0, 0.0, ctypes.byref(out), dptr(rate), self.P))
        else:
            e = np.ascontiguousarray(eedf, dtype=np.float64)
            self.check(self.lib.lgpu_eedf_postprocess(self.h, dptr(e), len(e), float(max_energy), ctypes.byref(out),
                                                      dptr(rate), self.P))
        return out, rate

    def eedf_rates(self, eedf=None, max_energy=0.0):
        """EEDF-convolved rate coefficients [n_eedf, P] of the rows of eedf,
        or (None) of the context's per-phase EEDFs under AC."""
        if eedf is None:
            n = max(self.cfg.n_phases, 1)
            rate = np.zeros((n, self.P))
            self.check(self.lib.lgpu_eedf_rates(self.h, None, 0, 0, 0.0, dptr(rate), self.P))
            return rate
        e = np.ascontiguousarray(np.atleast_2d(eedf), dtype=np.float64)
        rate = np.zeros((e.shape[0], self.P))
        self.check(self.lib.lgpu_eedf_rates(self.h, dptr(e), e.shape[0], e.shape[1], float(max_energy), dptr(rate),
                                            self.P))
        return rate

    def distributions(self):
        c = self.cfg
        nEC, nCos, nR, nA, nPh = c.n_energy_cells, c.n_cos_cells, c.n_radial_cells, c.n_axial_cells, c.n_phases
        out = dict(eedf_cells=np.zeros(nEC), eedf=np.zeros(nEC), efadf=np.zeros(nEC), esadf=np.zeros(nEC),
                   eadf=np.zeros((nEC, nCos)), evdf=np.zeros((nR, nA)), radial_cells=np.zeros(nR),
                   axial_cells=np.zeros(nA), eedf_periodic=np.zeros((nPh, nEC)))
        self.check(self.lib.lgpu_get_distributions(self.h, *[dptr(out[k]) for k in (
            "eedf_cells", "eedf", "efadf", "esadf", "eadf", "evdf", "radial_cells", "axial_cells", "eedf_periodic")]))
        return out

    def periodic(self):
        nPh = self.cfg.n_phases
        out = dict(n=np.zeros(nPh), mean_energy=np.zeros(nPh), flux_v=np.zeros((nPh, 3)),
                   bulk_v=np.zeros((nPh, 3)), flux_d=np.zeros((nPh, 9)), bulk_d=np.zeros((nPh, 9)))
        self.check(self.lib.lgpu_get_periodic(self.h, *[dptr(out[k]) for k in (
            "n", "mean_energy", "flux_v", "bulk_v", "flux_d", "bulk_d")]))
        return out

    def series(self, which, width):
        n = self.lib.lgpu_get_series(self.h, which, None, 0)
        rows = self.lib.lgpu_get_series(self.h, which, None, 1 << 40)
        out = np.zeros(rows * width)
        got = self.lib.lgpu_get_series(self.h, which, dptr(out), rows)
        if got < 0:
            self.check(-got)
        del n
        return out.reshape(rows, width) if width > 1 else out

    def timing(self) -> Timing:
        t = Timing()
        self.check(self.lib.lgpu_get_timing(self.h, ctypes.byref(t)))
        return t

    def stream(self) -> int:
        return self.lib.lgpu_stream(self.h) or 0

    def build_tables(self, max_energy, M, P):
        nu_tot, nu_max = np.zeros(M), np.zeros(M)
        sig = np.zeros(M * P, np.float32)
        cum = np.zeros(M * P, np.float32)
        self.check(self.lib.lgpu_build_tables(self.h, float(max_energy), dptr(nu_tot), dptr(nu_max),
                                              sig.ctypes.data_as(P_(ctypes.c_float)),
                                              cum.ctypes.data_as(P_(ctypes.c_float))))
        return nu_tot, nu_max, sig, cum

    def set_field_raw(self, E, freq_hz, red_mag, cyclotron):
        e = np.ascontiguousarray(E, dtype=np.float64)
        self.check(self.lib.lgpu_set_field_raw(self.h, dptr(e), float(freq_hz), float(red_mag), float(cyclotron)))

    def replay_flights(self, t, dt, pos, vel):
        n = len(t)
        t = np.ascontiguousarray(t, np.float64)
        dt = np.ascontiguousarray(dt, np.float64)
        pos = np.ascontiguousarray(pos, np.float64).reshape(n, 3)
        vel = np.ascontiguousarray(vel, np.float64).reshape(n, 3)
        po, vo, eo, go = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n), np.zeros(n)
        self.check(self.lib.lgpu_replay_flights(self.h, n, dptr(t), dptr(dt), dptr(pos), dptr(vel), dptr(po),
                                                dptr(vo), dptr(eo), dptr(go)))
        return po, vo, eo, go

    def replay_collisions(self, nu, vel, energy, uniforms, coarse=False):
        """lgpu_replay_collisions, or with coarse=True
        lgpu_replay_collisions_coarse (the advance kernels' null test)."""
        n = len(nu)
        nu = np.ascontiguousarray(nu, np.float64)
        vel = np.ascontiguousarray(vel, np.float64).reshape(n, 3)
        energy = np.ascontiguousarray(energy, np.float64)
        u = np.ascontiguousarray(uniforms, np.float64).reshape(n, -1)
        out = np.zeros((n, 11))
        used = np.zeros(n, np.int32)
        fn = self.lib.lgpu_replay_collisions_coarse if coarse else self.lib.lgpu_replay_collisions
        self.check(fn(self.h, n, dptr(nu), dptr(vel), dptr(energy), dptr(u), u.shape[1], dptr(out),
                      used.ctypes.data_as(P_(I))))
        return out, used


class Batch:
    """Owns one lgpu_batch: many contexts solved with one launch sequence per
    synchronisation interval."""

    def __init__(self, device=0, max_slots=64):
        self.lib = load()
        self.h = ctypes.c_void_p()
        self.ctxs = []
        rc = self.lib.lgpu_batch_create(int(device), int(max_slots), ctypes.byref(self.h))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())

    def last_error(self) -> str:
        buf = ctypes.create_string_buffer(1024)
        self.lib.lgpu_batch_last_error(self.h, buf, 1024)
        return buf.value.decode(errors="replace")

    def add(self, ctx: Context):
        rc = self.lib.lgpu_batch_add(self.h, ctx.h)
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())
        self.ctxs.append(ctx)

    def start(self):
        rc = self.lib.lgpu_batch_start(self.h)
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())

    def step(self, n=1):
        """n batched intervals: (contexts still running, BatchReport of the call)."""
        running = I()
        rep = BatchReport()
        rc = self.lib.lgpu_batch_step(self.h, int(n), ctypes.byref(running), ctypes.byref(rep))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())
        return running.value, rep

    def stream(self) -> int:
        return self.lib.lgpu_batch_stream(self.h)

    def set_schedule(self, shape, real_batch=20, coarse=1):
        """Pins the advance's launch shape, collision-turn threshold and
        coarse null test (shape -1: tune them on line again)."""
        rc = self.lib.lgpu_batch_set_schedule(self.h, int(shape), int(real_batch), int(coarse))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())

    def run(self):
        """Solves every added context: (results, status codes, BatchReport)."""
        n = len(self.ctxs)
        res = (Result * max(n, 1))()
        st = (I * max(n, 1))()
        rep = BatchReport()
        rc = self.lib.lgpu_batch_run(self.h, res, st, n, ctypes.byref(rep))
        self.ctxs = []
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())
        return [res[i] for i in range(n)], [st[i] for i in range(n)], rep

    def close(self):
        if self.h:
            self.lib.lgpu_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Owns one lgpu_server: continuous batching of submitted swarm jobs."""

    def __init__(self, device=0, max_slots=64, memory_budget_bytes=0.0):
        self.lib = load()
        self.h = ctypes.c_void_p()
        rc = self.lib.lgpu_server_start(int(device), int(max_slots), float(memory_budget_bytes), ctypes.byref(self.h))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, self.last_error())

    def last_error(self) -> str:
        buf = ctypes.create_string_buffer(1024)
        self.lib.lgpu_server_last_error(self.h, buf, 1024)
        return buf.value.decode(errors="replace")

    def submit(self, cfg: Config, ps, gas_first, gas_last, gas_fraction, N, Tg=300.0, red_field=0.0, angle=180.0,
               freq_hz=0.0, red_mag=0.0, twoterm=None) -> int:
        """twoterm: per process dicts (twoterm_array) for the EEDF
        post-processing at the job's end, or None."""
        arr, gs, keep = process_arrays(ps, gas_first, gas_last, gas_fraction)
        tt = None
        if twoterm is not None:
            tt, tkeep = twoterm_array(twoterm)
            keep = (keep, tkeep, tt)
        job = Job(cfg, ctypes.cast(arr, P_(Process)), ps.n, ctypes.cast(gs, P_(Gas)), len(gas_first),
                  float(ps.energy_max_elastic), Conditions(N, Tg, red_field, angle, freq_hz, red_mag),
                  ctypes.cast(tt, P_(TwotermProcess)) if tt is not None else None)
        jid = LL()
        rc = self.lib.lgpu_server_submit(self.h, ctypes.byref(job), ctypes.byref(jid))
        del keep  # the server copied every array
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_submit failed")
        return jid.value

    def job_eedf(self, job_id, n_procs):
        """(EedfParams, EEDF-convolved rates) of a finished job submitted with
        two-term inputs (lgpu_server_job_eedf)."""
        out = EedfParams()
        rates = np.zeros(n_procs)
        rc = self.lib.lgpu_server_job_eedf(self.h, LL(job_id), ctypes.byref(out), dptr(rates), int(n_procs))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_job_eedf failed")
        return out, rates

    def submit_request(self, req: "Request") -> list:
        """lgpu_server_submit_request: every job of a parsed request."""
        n = len(req)
        ids = (LL * max(n, 1))()
        rc = self.lib.lgpu_server_submit_request(self.h, req.h, ids, n)
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_submit_request failed")
        return list(ids[:n])

    def poll(self, jid) -> JobStatus:
        st = JobStatus()
        rc = self.lib.lgpu_server_poll(self.h, int(jid), ctypes.byref(st))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_poll failed")
        return st

    def wait(self, jid, timeout_s=0.0) -> JobStatus:
        st = JobStatus()
        rc = self.lib.lgpu_server_wait(self.h, int(jid), float(timeout_s), ctypes.byref(st))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_wait: job not finished")
        return st

    def rates(self, jid, n):
        counts = np.zeros(n, np.uint64)
        rate = np.zeros(n)
        rc = self.lib.lgpu_server_job_rates(self.h, int(jid), counts.ctypes.data_as(P_(ctypes.c_ulonglong)),
                                            dptr(rate), int(n))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_job_rates failed")
        return counts, rate

    def cancel(self, jid):
        rc = self.lib.lgpu_server_cancel(self.h, int(jid))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_cancel failed")

    def forget(self, jid):
        rc = self.lib.lgpu_server_forget(self.h, int(jid))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_server_forget failed")

    def report(self) -> ServerReport:
        r = ServerReport()
        self.lib.lgpu_server_report_get(self.h, ctypes.byref(r))
        return r

    def stop(self):
        if self.h:
            self.lib.lgpu_server_stop(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


class Request:
    """lgpu_request: the jobs of a setup file and its LXCat files, parsed by
    the library (no file access: the texts are passed in)."""

    def __init__(self, setup_text: str, files: dict):
        self.lib = load()
        self.h = ctypes.c_void_p()
        names = list(files)
        n = len(names)
        cn = (ctypes.c_char_p * max(n, 1))(*[k.encode() for k in names])
        ct = (ctypes.c_char_p * max(n, 1))(*[files[k].encode() for k in names])
        err = ctypes.create_string_buffer(1024)
        rc = self.lib.lgpu_request_parse(setup_text.encode(), n, cn, ct, ctypes.byref(self.h), err, 1024)
        if rc != LGPU_OK:
            raise LokiGpuError(rc, err.value.decode(errors="replace"))

    def __len__(self):
        return self.lib.lgpu_request_jobs(self.h)

    def job(self, k) -> Job:
        j = Job()
        rc = self.lib.lgpu_request_job(self.h, int(k), ctypes.byref(j))
        if rc != LGPU_OK:
            raise LokiGpuError(rc, "lgpu_request_job failed")
        return j

    def twoterm(self, k=0):
        """The collision behind each process of job k, as the EEDF
        post-processing reads it: dicts of twoterm_array's fields."""
        j = self.job(k)
        out = []
        for p in range(j.n_procs):
            t = j.twoterm[p]
            out.append(dict(kind=t.kind, ion=t.ion, density=t.density, threshold=t.threshold,
                            mass_ratio=t.mass_ratio, stat_ratio=t.stat_ratio,
                            int_e=np.ctypeslib.as_array(t.int_e, (t.n_int,)).copy(),
                            int_v=np.ctypeslib.as_array(t.int_v, (t.n_int,)).copy(),
                            mom_e=np.ctypeslib.as_array(t.mom_e, (t.n_mom,)).copy(),
                            mom_v=np.ctypeslib.as_array(t.mom_v, (t.n_mom,)).copy()))
        return out

    def processes(self, k=0):
        """The flattened processes of job k as numpy arrays (the field names
        of synth.ProcessSet)."""
        j = self.job(k)
        P = j.n_procs
        q = [j.procs[p] for p in range(P)]
        out = {f: np.array([getattr(x, f) for x in q]) for f in
               ("type", "is_super", "is_elastic", "sampler", "sampler_p0", "sampler_p1", "superw", "emin", "emax",
                "rel_dens", "mass", "eloss", "wparam", "raw_len")}
        out["raw_e"] = [np.ctypeslib.as_array(x.raw_e, (x.raw_len,)).copy() if x.raw_len else np.zeros(0) for x in q]
        out["raw_v"] = [np.ctypeslib.as_array(x.raw_v, (x.raw_len,)).copy() if x.raw_len else np.zeros(0) for x in q]
        out["gas_first"] = np.array([j.gases[g].first for g in range(j.n_gases)])
        out["gas_last"] = np.array([j.gases[g].last for g in range(j.n_gases)])
        out["gas_frac"] = np.array([j.gases[g].fraction for g in range(j.n_gases)])
        out["energy_max_elastic"] = j.emax_elastic
        return out

    def close(self):
        if self.h:
            self.lib.lgpu_request_free(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
