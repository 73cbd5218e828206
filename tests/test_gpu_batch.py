"""GPU tests of the batch engine (clk_batch_*): a pipeline over many
images of uneven shape and pixel type, one persistent launch per step and
pixel type, replayed from a CUDA graph.  Batched results must equal the
per-image plain calls bit for bit; integer images must also equal the
oracle applied step by step."""
import numpy as np
import pytest

from conftest import random_image

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clk():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import clk as m
    m.load()
    return m


def make_images(rng, n, dtypes):
    imgs = []
    for k in range(n):
        dt = dtypes[k % len(dtypes)]
        if k % 2:
            shp = (int(rng.integers(3, 17)), int(rng.integers(16, 90)), int(rng.integers(16, 130)))
        else:
            shp = (int(rng.integers(16, 150)), int(rng.integers(16, 200)))
        if k % 5 == 0:  # some even widths for the register-window paths, some odd
            shp = shp[:-1] + (shp[-1] | 1,)
        elif k % 5 == 1:
            shp = shp[:-1] + (shp[-1] & ~1,)
        a = random_image(rng, shp, dt)
        if np.dtype(dt) == np.float32:
            a = np.abs(a)  # no -0.0 in float medians
        imgs.append(a)
    return imgs


CHAIN_TOPHAT = lambda clk: [clk.op_separable("gaussian_blur_separable", (13, 13, 13), (2.0, 2.0, 2.0)),  # noqa: E731
                            clk.op_separable("minimum_separable", (9, 9, 9), (4.0, 4.0, 4.0)),
                            clk.op_separable("maximum_separable", (9, 9, 9), (4.0, 4.0, 4.0)),
                            clk.op_kernel("median_box", (3, 3, 3))]
CHAIN_MIXED = lambda clk: [clk.op_separable("mean_separable", (5, 5, 3), (2.0, 2.0, 1.0)),  # noqa: E731
                           clk.op_morphology("dilate_sphere", 2),
                           clk.op_kernel("median_sphere", (5, 5, 5)),
                           clk.op_separable("gaussian_blur_separable", (7, 7, 1), (1.0, 1.0, 0.0))]


def run_both(clk, ops, imgs, tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("CLK_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    srcs = [torch.from_numpy(a).cuda() for a in imgs]
    out_b = [torch.empty_like(s) for s in srcs]
    out_p = [torch.empty_like(s) for s in srcs]
    b = clk.Batch(ops, srcs, out_b)
    b.run()
    b.run()  # a second replay gives the same result
    torch.cuda.synchronize()
    got = [t.cpu().numpy() for t in out_b]
    b.close()
    bp = clk.Batch(ops, srcs, out_p)
    bp.run_plain()
    torch.cuda.synchronize()
    want = [t.cpu().numpy() for t in out_p]
    return got, want, b


@pytest.mark.parametrize("chain", ["tophat", "mixed"])
def test_batched_equals_plain(clk, chain, tmp_path, monkeypatch):
    rng = np.random.default_rng(51)
    imgs = make_images(rng, 30, [np.uint8, np.uint16, np.float32, np.int16, np.int8])
    ops = CHAIN_TOPHAT(clk) if chain == "tophat" else CHAIN_MIXED(clk)
    got, want, b = run_both(clk, ops, imgs, tmp_path, monkeypatch)
    for k, (g, w) in enumerate(zip(got, want)):
        assert g.tobytes() == w.tobytes(), (chain, k, imgs[k].shape, imgs[k].dtype)
    assert (tmp_path / "tune.json").exists()
    # the tuner chose, per step, a work-item depth and, for the integer
    # separable steps, a tile body (0: register-window 64x32, 1: generic 64x16)
    import json
    tune = json.loads((tmp_path / "tune.json").read_text())
    tiles = {k: v for k, v in tune.items() if k.endswith("|tile")}
    assert tiles and all(v in (0, 1) for v in tiles.values()), tune
    assert all(k[: -len("|tile")] in tune for k in tiles), tune


def test_batched_tophat_matches_oracle_on_integer_images(clk, oracle, tmp_path, monkeypatch):
    rng = np.random.default_rng(52)
    imgs = make_images(rng, 12, [np.uint8, np.uint16])
    got, _, _ = run_both(clk, CHAIN_TOPHAT(clk), imgs, tmp_path, monkeypatch)
    for k, a in enumerate(imgs):
        nd = a.ndim
        sfx = "_2d" if nd == 2 else "_3d"
        N = (13, 13, 13)[:nd]
        cur = oracle.separable("gaussian_blur_separable" + sfx, a, a.dtype, N, (2.0,) * nd)
        cur = oracle.separable("minimum_separable" + sfx, cur, a.dtype, (9,) * nd, (4.0,) * nd)
        cur = oracle.separable("maximum_separable" + sfx, cur, a.dtype, (9,) * nd, (4.0,) * nd)
        cur = oracle.execute("median_box" + sfx, cur, a.dtype, [3] * nd)
        assert np.array_equal(got[k], cur), (k, a.shape, a.dtype)


def test_batched_medians_on_rows_of_whole_vectors_match_oracle(clk, oracle, tmp_path, monkeypatch):
    # widths of whole 16-byte vectors take the staged bodies (float keys for
    # f32, staged plane tiles for 16-bit pixels), the others the pair bodies
    rng = np.random.default_rng(54)
    imgs = []
    for dt, w in ((np.float32, 36), (np.float32, 64), (np.float32, 38), (np.uint16, 72), (np.uint16, 66),
                  (np.int16, 40), (np.uint8, 48)):
        a = random_image(rng, (int(rng.integers(5, 12)), int(rng.integers(9, 40)), w), dt)
        imgs.append(np.abs(a) if np.dtype(dt) == np.float32 else a)
    for name, N in (("median_sphere", (5, 5, 5)), ("median_box", (3, 3, 3))):
        got, want, _ = run_both(clk, [clk.op_kernel(name, N)], imgs, tmp_path, monkeypatch)
        for k, a in enumerate(imgs):
            ref = oracle.execute(name + "_3d", a, a.dtype, list(N))
            assert got[k].tobytes() == ref.tobytes(), (name, a.shape, a.dtype)
            assert want[k].tobytes() == ref.tobytes(), (name, a.shape, a.dtype)


def test_one_launch_per_step_type_and_body(clk, tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("CLK_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(53)
    imgs = []
    for k in range(40):  # even widths: every image has a batched body
        dt = [np.uint8, np.uint16, np.float32][k % 3]
        shp = (int(rng.integers(4, 12)), int(rng.integers(16, 64)), 2 * int(rng.integers(8, 64)))
        imgs.append(np.abs(random_image(rng, shp, dt)))
    srcs = [torch.from_numpy(a).cuda() for a in imgs]
    dsts = [torch.empty_like(s) for s in srcs]
    b = clk.Batch(CHAIN_TOPHAT(clk), srcs, dsts)
    # steps x pixel types, not steps x images; the median step runs one launch
    # per pixel type and network body (16-bit rows of whole vectors take the
    # staged tiles, other even widths the row pairs)
    assert b.launches <= 4 * 3 + 3, b.launches
    b.close()


def test_per_kernel_launches_give_the_same_integer_results(clk, tmp_path, monkeypatch):
    """The reference's launch pattern (one clk_execute per axis and kernel)
    equals the fused/batched result for integer images."""
    import torch
    monkeypatch.setenv("CLK_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(54)
    imgs = make_images(rng, 14, [np.uint8, np.uint16, np.int16])
    srcs = [torch.from_numpy(a).cuda() for a in imgs]
    out_b = [torch.empty_like(s) for s in srcs]
    b = clk.Batch(CHAIN_TOPHAT(clk), srcs, out_b)
    b.run()
    torch.cuda.synchronize()
    got = [t.cpu().numpy() for t in out_b]
    for t in out_b:
        t.zero_()
    b.run_per_kernel()
    torch.cuda.synchronize()
    for k, t in enumerate(out_b):
        assert np.array_equal(t.cpu().numpy(), got[k]), (k, imgs[k].shape, imgs[k].dtype)
    b.close()
