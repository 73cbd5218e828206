"""CPU check of the z-chunk model shared by the streaming kernels
(wave_chunks in clk_internal.h): tests/wave_chunks_check.cpp asserts the
counts it picks for the measured cases and that a choice never costs more
waves x planes than one chunk per tile."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_wave_chunks(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    cuda_inc = next((p for p in (Path("/usr/local/cuda/include"),) if (p / "cuda_runtime_api.h").exists()), None)
    if cxx is None or cuda_inc is None:
        pytest.skip("no C++ compiler or CUDA headers")
    exe = tmp_path / "wave_chunks_check"
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-I", str(ROOT / "include"), "-I", str(cuda_inc),
                        "-I", str(ROOT / "clij-opencl-kernels_gb300" / "csrc"), "-o", str(exe),
                        str(ROOT / "tests" / "wave_chunks_check.cpp")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-2000:]
