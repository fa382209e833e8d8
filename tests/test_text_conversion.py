"""The decimal conversion code of the state I/O kernels (golikov_2d_gb300/csrc/gd_text.cuh)
against the C library: "%.6g" formatting byte for byte and correctly rounded parsing bit for
bit, on random bit patterns, typical magnitudes, exact ties, powers of ten, subnormals and
long digit strings.  The header is compiled for the host here (it is __host__ __device__);
the GPU tests check the kernels themselves."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_format_and_parse_match_libc(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "text_conversion")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "text_conversion.cpp")],
                   check=True)
    r = subprocess.run([exe, "100000"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:]
