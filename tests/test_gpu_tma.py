"""The opt-in TMA staging of the fused separable kernels (CLK_SEP2_TMA=1,
read once per process): a child process runs integer min/max/mean, the
integer and float Gaussians and float min/max through it and compares with
the oracle bit for bit (float outputs of the Gaussian within the FP64
tolerance)."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/clij-opencl-kernels_gb300"); sys.path.insert(0, sys.argv[1] + "/tests")
import torch
import clk
from conftest import random_image
from oracle import oracle as O
O.port()
rng = np.random.default_rng(41)
bad = []
def run(kernel, a, ddt, N, s):
    d = torch.empty(a.shape, dtype=clk.torch_dtype(O.dtype_code(ddt)), device="cuda")
    clk.separable(kernel, torch.from_numpy(a).cuda(), d, N, s)
    torch.cuda.synchronize()
    return d.cpu().numpy()
for shp in ((9, 70, 128), (3, 33, 64)):
    for dt in (np.uint16, np.uint8, np.float32):
        a = random_image(rng, shp, dt)
        for R in (2, 5):
            N, s = (2 * R + 1, 2 * R + 1, 5), (R / 2.0, R / 2.0, 1.0)
            for k in ("minimum_separable_3d", "maximum_separable_3d", "mean_separable_3d", "gaussian_blur_separable_3d"):
                if dt == np.float32 and k == "mean_separable_3d":
                    continue
                for ddt in ((dt, np.float32) if k.startswith("gaussian") and dt != np.float32 else (dt,)):
                    got = run(k, a, ddt, N, s)
                    if ddt == np.float32 and k.startswith("gaussian"):
                        val, scale = O.fp64(k, a, N, s)
                        ok = bool((np.abs(got.astype(np.float64) - val) <= 1e-5 * np.maximum(np.abs(val), scale)).all())
                    else:
                        ok = got.tobytes() == O.separable(k, a, ddt, N, s).tobytes()
                    if not ok:
                        bad.append([k, list(shp), str(np.dtype(dt)), str(np.dtype(ddt)), R])
print(json.dumps({"bad": bad}))
"""


def test_tma_staging_matches_oracle():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    env = dict(os.environ, CLK_SEP2_TMA="1")
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["bad"] == [], res["bad"]
