"""The C ABI library without a GPU: it loads, exports every entry point that
include/loki_gpu.h declares, fills the reference's defaults
(Code/LoKI-MC/Headers/BoltzmannMC.h:50-104) and reports a missing device
as a status code instead of falling back to anything."""
import ctypes
import os
import re

import pytest

from lokigpu import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "loki_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^(?:int|void|long long|void\*)\s+\**(lgpu_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    names = declared_symbols()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(capi.EXPORTED)


def test_defaults_match_reference():
    c = capi.default_config()
    assert c.n_interp == 10000           # interpolCrossSectionSize
    assert c.init_temp_ratio == 0.01     # initialElecTempOverGasTemp
    assert c.req_integration_points == 200
    assert (c.n_energy_cells, c.n_cos_cells, c.n_radial_cells, c.n_axial_cells) == (1000, 100, 200, 200)
    assert c.n_phases == 100
    assert c.sync_x == 1.0 and c.sync_oversampling == 1
    assert c.max_coll_before_ss == 1e100 and c.min_coll_before_ss == 0


def test_status_codes_without_device():
    lib = capi.load()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a CUDA device is present")
    except ImportError:
        pass
    cfg = capi.default_config()
    h = ctypes.c_void_p()
    rc = lib.lgpu_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == 8  # LGPU_ERR_NO_DEVICE
    buf = ctypes.create_string_buffer(256)
    lib.lgpu_last_error(h, buf, 256)
    assert b"no CUDA device" in buf.value
    lib.lgpu_destroy(h)
    assert lib.lgpu_create(None, ctypes.byref(h)) == 1  # LGPU_ERR_BAD_ARG
    assert lib.lgpu_solve(None, None) == 1


def test_process_records_carry_every_field_and_table():
    """The lgpu_process records the front end builds column by column hold
    each process's fields, and their raw pointers read back each process's
    own cross-section table (a superelastic copy has none)."""
    import numpy as np

    from lokigpu import synth

    ps = synth.flatten([synth.n2_like_gas(fraction=0.8), synth.o2_like_gas(fraction=0.2)])
    arr, gs, keep = capi.process_arrays(ps, ps.gas_first, ps.gas_last, ps.gas_fraction)
    assert ctypes.sizeof(capi.Process) == capi._PROCESS_DTYPE.itemsize
    for p in range(ps.n):
        q = arr[p]
        assert (q.type, q.is_super, q.is_elastic, q.sampler) == (int(ps.ptype[p]), int(ps.is_super[p]),
                                                                 int(ps.is_elastic[p]), int(ps.sampler[p]))
        for name, src in (("sampler_p0", ps.sampler_p0), ("sampler_p1", ps.sampler_p1), ("superw", ps.superw),
                          ("emin", ps.emin), ("emax", ps.emax), ("rel_dens", ps.rel_dens), ("mass", ps.mass),
                          ("eloss", ps.eloss), ("wparam", ps.wparam)):
            assert getattr(q, name) == float(src[p]), (p, name)
        e = np.asarray(ps.raw_e[p], dtype=np.float64)
        v = np.asarray(ps.raw_v[p], dtype=np.float64)
        assert q.raw_len == (0 if ps.is_super[p] else len(e))
        assert [q.raw_e[k] for k in range(len(e))] == list(e)
        assert [q.raw_v[k] for k in range(len(v))] == list(v)
    assert [(g.first, g.last, g.fraction) for g in gs] == [
        (int(a), int(b), float(c)) for a, b, c in zip(ps.gas_first, ps.gas_last, ps.gas_fraction)]
