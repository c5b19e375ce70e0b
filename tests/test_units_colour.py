"""The bank-group order of the batched k-wide unit products (colour_wave in
units.cuh), checked on the host: compiled with nvcc as host code and run on
seeded waves (tests/native/colour_wave_check.cu)."""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import ROOT


def test_colour_wave_is_a_proper_colouring(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.which(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "colour_wave_check"
    csrc = ROOT / "plsqr3.2013.09_gb300" / "csrc"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", str(csrc), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "native" / "colour_wave_check.cu"), "-o", str(exe)],
                   check=True, capture_output=True, timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
