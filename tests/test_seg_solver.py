"""The segmented recurrences of the few-wavefunction chain solver (k_chain_seg in qpc_chain.cuh), replayed
on the host with the engine's own seg_spike: forward and backward solves against the sequential ones, for
B-spline degrees 5..8 and segment layouts with short last segments (tests/cpp/seg_replay.cu)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_segmented_recurrences_match_sequential(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if not nvcc:
        pytest.skip("no CUDA compiler")
    exe = str(tmp_path / "seg_replay")
    csrc = os.path.join(ROOT, "qpc-tdse-cpc_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", csrc, os.path.join(ROOT, "tests", "cpp", "seg_replay.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout.split("\n")
    rows = [l.split() for l in out if l.strip()]
    assert len(rows) == 5
    for P, N, Q, Ls, ef, eb in rows:
        assert int(N) - (int(Q) - 1) * int(Ls) >= int(P)       # the last segment holds a full carry
        assert float(ef) < 1e-14 and float(eb) < 1e-14, (P, N, Q)
