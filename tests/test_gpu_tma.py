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


TIMEOUT_CHILD = r"""
import json, os, sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/clij-opencl-kernels_gb300")
import torch
import clk
from clk import _lib as L
from oracle import oracle as O
O.port()
rng = np.random.default_rng(5)
a = rng.integers(0, 65536, size=(12, 70, 128)).astype(np.uint16)
src = torch.from_numpy(a).cuda()
want = O.separable("maximum_separable_3d", a, np.uint16, (7, 7, 3), (3, 3, 1))
res = {}
def call():
    d = torch.zeros(a.shape, dtype=torch.uint16, device="cuda")
    try:
        clk.separable("maximum_separable_3d", src, d, (7, 7, 3), (3.0, 3.0, 1.0))
        torch.cuda.synchronize()
        return "ok", d.cpu().numpy()
    except L.ClkError as e:
        torch.cuda.synchronize()
        return e.status, None
# 1: every first wait runs out at once; the kernel drains its copies, sets
# the flag and returns; the call itself returned before the kernel ran
os.environ["CLK_TMA_WAIT_POLLS"] = "0"
res["first"] = call()[0]
# 2: the next call reports the earlier launch as timed out
res["second"] = call()[0]
# 3: with the normal limit the staging works again
del os.environ["CLK_TMA_WAIT_POLLS"]
res["third"], got = call()
res["third_matches_oracle"] = got is not None and got.tobytes() == want.tobytes()
res["fourth"] = call()[0]
res["timeout_code"] = L.TIMEOUT
print(json.dumps(res))
"""


def test_tma_wait_limit_runs_out_and_reports_timeout():
    # The bounded wait of the TMA staging, made to run out on purpose with a
    # poll limit of 0 (the copies themselves are real and land): the CTA
    # drains them, flags the launch, and the next call returns CLK_TIMEOUT;
    # afterwards the context is fine and results are correct.
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    env = dict(os.environ, CLK_SEP2_TMA="1")
    r = subprocess.run([sys.executable, "-c", TIMEOUT_CHILD, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["first"] == "ok", res
    assert res["second"] == res["timeout_code"], res
    assert res["third"] == "ok" and res["third_matches_oracle"], res
    assert res["fourth"] == "ok", res
