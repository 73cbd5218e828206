"""CPU check of the register-ring separable kernels' address arithmetic
(clk_sep3.cuh): tests/sep3_layout_check.cu recomputes every thread's
shared-memory and global offsets for every instantiated operation, radius
and Z radius over a range of image extents (border tiles included) and
checks that each access stays inside its buffer and its staged row.  The
kernels' shared-memory accesses cannot be bounds-checked on the device here
(no sanitizer), and an access past a buffer but inside the CTA's shared
memory would not fault; this check covers that."""
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


def test_sep3_layout(tmp_path):
    cc = nvcc()
    if cc is None:
        pytest.skip("nvcc not found")
    exe = tmp_path / "sep3_layout_check"
    r = subprocess.run([cc, "-O1", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                        "--expt-relaxed-constexpr", "-I", str(ROOT / "include"),
                        "-I", str(ROOT / "clij-opencl-kernels_gb300" / "csrc"), "-o", str(exe),
                        str(ROOT / "tests" / "sep3_layout_check.cu")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-2000:]
