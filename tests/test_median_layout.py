"""CPU check of the staged median kernels' shared-memory layouts
(clk_median_impl.cuh): tests/median_layout_check.cu replays the staging of
every CTA over a range of image extents (cp.async vectors inside the row,
edge-pixel fills outside it), records which clamped image pixel each
shared-memory element holds, and checks that every read of the tile bodies
stays inside its buffer and finds the pixel of the reference's clamped read;
it also replays the z-pair loops' plane rings.  A read one column off or a
ring buffer reused one pair early makes it fail."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return None


def test_median_layout(tmp_path):
    cc = nvcc()
    if cc is None:
        pytest.skip("nvcc not found")
    exe = tmp_path / "median_layout_check"
    r = subprocess.run([cc, "-O1", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                        "--expt-relaxed-constexpr", "-I", str(ROOT / "include"),
                        "-I", str(ROOT / "clij-opencl-kernels_gb300" / "csrc"), "-o", str(exe),
                        str(ROOT / "tests" / "median_layout_check.cu")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-2000:]
