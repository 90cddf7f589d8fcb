"""The batched passes' chunk layout (loki-mc_gb300/csrc/lgpu_chunks.h) on the host.

The moment and distribution passes of a batch cut all conditions' electrons
into chunks listed full chunks first, then remainders largest first, and take
them in snake order over the blocks. tests/chunk_layout_check.cpp compiles the
same header with g++ and walks the layout as the kernels do: every electron of
every included condition exactly once, none of an excluded one, and on
sweep-like sets of conditions no block more than one chunk above the mean.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_chunk_layout_covers_every_electron_once(tmp_path):
    exe = tmp_path / "chunk_layout_check"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "loki-mc_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "chunk_layout_check.cpp"), "-o", str(exe)])
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0 and run.stdout.strip().endswith("ok"), run.stdout[-2000:]
