"""The library's Float16C codec, compiled for the host from its CUDA header, equals the oracle's
restatement of src/utils/custom_fp.mojo:36-101 on every 16-bit code (decode) and every 32-bit
float pattern (encode).  The GPU tests check the device build of the same functions."""
import shutil
import subprocess
from pathlib import Path

import pytest

import oracle

HERE = Path(__file__).resolve().parent


def test_codec_exhaustive(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    lib = oracle.build()
    exe = tmp_path / "codec_exhaustive"
    subprocess.run([gxx, "-O2", "-std=c++17", "-fopenmp", "-x", "c++", str(HERE / "codec_exhaustive.cpp"), "-o",
                    str(exe), f"-L{lib.parent}", "-llbm_oracle", f"-Wl,-rpath,{lib.parent}"], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "decode mismatches 0, encode mismatches 0" in res.stdout
