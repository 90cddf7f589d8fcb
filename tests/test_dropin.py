"""The drop-in entry point (loki-mc_gb300/adapter/) builds with the
reference's own sources and runs a setup up to the GPU backend: without a
device it must stop the reference's way (Message::error, errorLog.txt), with
no CPU fallback. Needs the reference source tree; skipped elsewhere."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("LOKI_REFERENCE_CODE", "")


@pytest.mark.skipif(not (REF and os.path.isdir(REF)), reason="LOKI_REFERENCE_CODE (the reference's Code/) not set")
def test_dropin_reaches_the_backend(tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a CUDA device is present: the run would not stop at the backend")
    except ImportError:
        pass
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "dropin"])
    sys.path.insert(0, os.path.join(ROOT, "loki-mc_gb300", "python"))
    from lokigpu import synth

    synth.write_case(str(tmp_path), [synth.atomic_gas()], pressure_pa=3.22e22 * 1.38064852e-23 * 300,
                     red_field=100.0, n_electrons=1000, kte_init_ev=1.0,
                     extra_numerics={"backend": "gpu", "nIntegrationPoints": "500"})
    r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "lokimc_gpu"), "case.in", "1"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=120)
    log = (tmp_path / "errorLog.txt").read_text()
    assert "lgpu_create: no CUDA device" in log, r.stdout[-2000:]


@pytest.mark.skipif(not (REF and os.path.isdir(REF)), reason="LOKI_REFERENCE_CODE (the reference's Code/) not set")
@pytest.mark.parametrize("name", ["reid_dc", "mix_b", "mix_ac"])
def test_dropin_comparison_passes_two_reference_seeds(name, tmp_path):
    """The bounds of the drop-in comparison on the GPU (test_dropin_gpu.py)
    calibrated on the reference itself: two runs of the reference built from
    source with different seeds of its generator must pass them."""
    import test_dropin_gpu as T

    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}"])
    bases = []
    for seed in (11, 22):
        d = tmp_path / f"s{seed}"
        T._write(str(d), name, gpu=False)
        env = dict(os.environ, LOKI_ORACLE_SEED=str(seed))
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "lokimc"), "case.in", "4"], cwd=d, env=env,
                       capture_output=True, timeout=1800, check=True)
        bases.append(str(d / "Output" / name))
    failures = T.compare_outputs(*bases)
    assert not failures, "\n".join(failures[:40])
