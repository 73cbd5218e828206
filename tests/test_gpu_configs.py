"""GPU parity at the benchmark sizes, against the oracle.

* the 256x256x64 uint16 blob stack (200 blobs): gaussian_blur_separable_3d
  sigma (2,2,1), N = (13,13,7), to float;
* the 1024x1024x256 uint16 blob stack (20k blobs) and its uint8 mask
  (> 400): every filter of the plain suite, each as the bench runs it;
* a 2048x2048x40 float32 slab of the large-halo stack (blobs + N(0,20)
  noise; both z borders inside the slab): gaussian sigma (10,10,5),
  maximum r (15,15,7), median_sphere r=2.

Integer, min/max and median outputs are compared bit for bit; float outputs
within |gpu - fp64| <= 1e-5 * max(|fp64|, scale) of the FP64 oracle (scale:
the filter applied to |src|, the forward-error bound of any float32
evaluation).  Each float case also reports its plain maximum relative error
max |gpu - fp64| / |fp64| over voxels with |fp64| > 1, against the FP64
oracle and against the reference-order float32 result; set
CLK_PARITY_REPORT=<file> to collect those figures as JSON lines.

The oracle runs on every host core (OpenMP); the whole file takes about a
minute of host time on 16 cores.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REL_TOL = 1e-5
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import clk
    from clk import synth
    clk.load()
    return torch, clk, synth


def report(case, **fields):
    path = os.environ.get("CLK_PARITY_REPORT")
    line = {"case": case, **fields}
    print(json.dumps(line))
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(line) + "\n")


def float_check(case, got, val, scale, ref_f32=None):
    """Scaled-bound pass/fail plus the plain relative errors."""
    got = got.astype(np.float64)
    err = np.abs(got - val)
    ok = err <= REL_TOL * np.maximum(np.abs(val), scale)
    big = np.abs(val) > 1.0
    rel = float((err[big] / np.abs(val[big])).max()) if big.any() else 0.0
    fields = {"voxels": int(got.size), "max_rel_err_vs_fp64": rel,
              "max_scaled_err_vs_fp64": float((err / np.maximum(np.maximum(np.abs(val), scale), 1e-30)).max()),
              "scaled_bound_pass": bool(ok.all())}
    if ref_f32 is not None:
        r = ref_f32.astype(np.float64)
        rb = np.abs(r) > 1.0
        fields["max_rel_err_vs_reference_order_f32"] = float((np.abs(got[rb] - r[rb]) / np.abs(r[rb])).max())
        fields["reference_order_max_rel_err_vs_fp64"] = float((np.abs(r[big] - val[big]) / np.abs(val[big])).max())
    report(case, **fields)
    assert ok.all(), (case, fields)


# ---------------------------------------------------------------- 256x256x64


def test_gaussian_256x256x64_u16_to_f32(env, oracle):
    torch, clk, synth = env
    img = synth.blobs((64, 256, 256), 200, seed=1, dtype=torch.uint16)
    out = torch.empty(img.shape, dtype=torch.float32, device="cuda")
    N, s = (13, 13, 7), (2.0, 2.0, 1.0)
    clk.separable("gaussian_blur_separable_3d", img, out, N, s)
    torch.cuda.synchronize()
    a = img.cpu().numpy()
    val, scale = oracle.fp64("gaussian_blur_separable_3d", a, N, s, nthreads=NT)
    impl = "ref" if oracle.ref_available() else "port"
    ref = oracle.separable("gaussian_blur_separable_3d", a, np.float32, N, s, impl=impl, nthreads=NT)
    float_check("gaussian s(2,2,1) 256x256x64 u16->f32", out.cpu().numpy(), val, scale, ref)


# ---------------------------------------------------------------- 1024x1024x256

# (name, kind, kernel, params, source, dst pixel type): the plain suite, each
# filter called the way the benchmark calls it
SUITE = [
    ("gaussian_blur s(3,3,1.5)", "sep", "gaussian_blur_separable_3d", ((19, 19, 11), (3.0, 3.0, 1.5)), "img",
     np.float32),
    ("mean_box r(5,5,2)", "sep", "mean_separable_3d", ((11, 11, 5), (5.0, 5.0, 2.0)), "img", np.uint16),
    ("minimum_box r(5,5,2)", "sep", "minimum_separable_3d", ((11, 11, 5), (5.0, 5.0, 2.0)), "img", np.uint16),
    ("maximum_box r(5,5,2)", "sep", "maximum_separable_3d", ((11, 11, 5), (5.0, 5.0, 2.0)), "img", np.uint16),
    ("median_box r1", "exec", "median_box_3d", (3, 3, 3), "img", np.uint16),
    ("median_sphere r2", "exec", "median_sphere_3d", (5, 5, 5), "img", np.uint16),
    ("sobel_3d", "exec", "sobel_3d", (), "img", np.float32),
    ("erode_sphere r1", "morph", "erode_sphere_3d", 1, "mask", np.uint8),
    ("erode_sphere r2", "morph", "erode_sphere_3d", 2, "mask", np.uint8),
    ("dilate_sphere r1", "morph", "dilate_sphere_3d", 1, "mask", np.uint8),
    ("dilate_sphere r2", "morph", "dilate_sphere_3d", 2, "mask", np.uint8),
]


@pytest.fixture(scope="module")
def stack(env):
    torch, clk, synth = env
    img = synth.blobs((256, 1024, 1024), 20000, seed=2, dtype=torch.uint16)
    mask = synth.mask_of(img, 400.0)
    return {"img": img, "mask": mask, "img_np": img.cpu().numpy(), "mask_np": mask.cpu().numpy()}


@pytest.mark.parametrize("name,kind,kernel,params,srcn,ddt", SUITE, ids=[t[0] for t in SUITE])
def test_suite_1024x1024x256(env, oracle, stack, name, kind, kernel, params, srcn, ddt):
    torch, clk, synth = env
    from clk.api import torch_dtype
    from oracle.oracle import dtype_code
    src, a = stack[srcn], stack[srcn + "_np"]
    out = torch.empty(src.shape, dtype=torch_dtype(dtype_code(ddt)), device="cuda")
    if kind == "sep":
        clk.separable(kernel, src, out, params[0], params[1])
    elif kind == "exec":
        p = {"src": src, "dst": out}
        p.update(dict(zip(("Nx", "Ny", "Nz"), params)))
        clk.execute(kernel, p)
    elif params == 1:
        clk.execute(kernel, {"src": src, "dst": out})
    else:
        clk.morphology(kernel, src, out, params)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    del out
    if ddt == np.float32:
        if kind == "sep":
            val, scale = oracle.fp64(kernel, a, params[0], params[1], nthreads=NT)
        else:
            val, scale = oracle.fp64(kernel, a, nthreads=NT)
        float_check(f"{name} 1024x1024x256", got, val, scale)
        return
    if kind == "sep":
        want = oracle.separable(kernel, a, ddt, params[0], params[1], nthreads=NT)
    elif kind == "exec":
        want = oracle.execute(kernel, a, ddt, list(params), nthreads=NT)
    else:
        want = a
        for _ in range(params):
            want = oracle.execute(kernel, want, np.uint8, nthreads=NT)
    mism = int(np.count_nonzero(got != want))
    report(f"{name} 1024x1024x256", voxels=int(got.size), mismatches=mism)
    assert mism == 0, (name, mism)


# ---------------------------------------------------------------- 2048x2048x40 f32


@pytest.fixture(scope="module")
def slab(env):
    torch, clk, synth = env
    img = synth.blobs((40, 2048, 2048), 2000, seed=7, dtype=torch.float32, poisson=False, noise_sigma=20.0)
    return img, img.cpu().numpy()


def test_large_halo_gaussian_slab(env, oracle, slab):
    torch, clk, synth = env
    img, a = slab
    out = torch.empty_like(img)
    N, s = (61, 61, 31), (10.0, 10.0, 5.0)
    clk.separable("gaussian_blur_separable_3d", img, out, N, s)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    del out
    val, scale = oracle.fp64("gaussian_blur_separable_3d", a, N, s, nthreads=NT)
    float_check("gaussian s(10,10,5) 2048x2048x40 f32", got, val, scale)


@pytest.mark.parametrize("kind", ["maximum r(15,15,7)", "median_sphere r2"])
def test_large_halo_exact_slab(env, oracle, slab, kind):
    torch, clk, synth = env
    img, a = slab
    out = torch.empty_like(img)
    if kind.startswith("maximum"):
        N, s = (31, 31, 15), (15.0, 15.0, 7.0)
        clk.separable("maximum_separable_3d", img, out, N, s)
        want = oracle.separable("maximum_separable_3d", a, np.float32, N, s, nthreads=NT)
    else:
        clk.execute("median_sphere_3d", {"src": img, "dst": out, "Nx": 5, "Ny": 5, "Nz": 5})
        want = oracle.execute("median_sphere_3d", a, np.float32, [5, 5, 5], nthreads=NT)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    mism = int(np.count_nonzero(got.view(np.uint32) != want.view(np.uint32)))
    report(f"{kind} 2048x2048x40 f32", voxels=int(got.size), mismatches=mism)
    assert mism == 0, (kind, mism)
