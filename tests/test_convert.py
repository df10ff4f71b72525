"""The integer-pipe FP64 <-> FP32 conversions used by the mixed form (dg_convert.cuh) equal the
IEEE round-to-nearest-even conversions bit for bit; checked on the host, where the same integer
expressions compile (no GPU needed)."""
import shutil
import subprocess
from pathlib import Path

import pytest

SRC = Path(__file__).resolve().parent / "native" / "convert_check.cpp"


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
def test_integer_pipe_conversions_match_ieee(tmp_path):
    exe = tmp_path / "convert_check"
    subprocess.run(["g++", "-O2", "-std=c++17", str(SRC), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout
    narrowed = int(out.stdout.split("narrowed ")[1].split()[0])
    assert narrowed > 9_000_000
