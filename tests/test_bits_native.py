"""The integer-pipe float64 <-> float32 conversions of the FP32-local kernel,
compiled for the host from the same header and checked against exact casts
(round-to-nearest-even, halfway cases, zeros, infinities, NaN)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_bit_conversions_match_exact_casts(tmp_path):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc) and shutil.which('nvcc') is None:
        pytest.skip('nvcc not available')
    exe = tmp_path / 'bits_check'
    subprocess.run([nvcc, '-O2', '-std=c++17', os.path.join(HERE, 'native', 'bits_check.cu'),
                    '-o', str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
