"""Failure handling on the GPU, made on the host (no GPU fault).

* Out of memory: with CLK_INJECT_ALLOC_FAILURE=1 every device allocation the
  library makes for temporaries reports failure.  clk_separable (pass-by-pass
  form), clk_morphology (three iterations), clk_batch_create and a served
  request with two steps must return CLK_OOM, leave no launch half done,
  and work again once the variable is cleared; calls that need no
  temporaries (the fused separable kernel) are unaffected.
* Cancellation: a request still queued behind a busy slot is cancelled,
  never runs (its output keeps its fill), waiting for it returns
  CLK_CANCELLED; a request already running cannot be cancelled (CLK_BUSY).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import clk
    from clk import _lib as L
    clk.load()
    return torch, clk, L


@pytest.fixture
def inject(monkeypatch):
    monkeypatch.setenv("CLK_INJECT_ALLOC_FAILURE", "1")
    yield
    monkeypatch.delenv("CLK_INJECT_ALLOC_FAILURE", raising=False)


def test_separable_oom_and_recovery(env, oracle, monkeypatch):
    torch, clk, L = env
    rng = np.random.default_rng(3)
    a = rng.integers(0, 256, size=(8, 40, 96)).astype(np.uint8)
    src = torch.from_numpy(a).cuda()
    out = torch.full(a.shape, 7, dtype=torch.uint16, device="cuda")
    monkeypatch.setenv("CLK_INJECT_ALLOC_FAILURE", "1")
    # uint8 -> uint16 has no fused kernel: the passes need temporaries
    with pytest.raises(L.ClkError) as e:
        clk.separable("mean_separable_3d", src, out, (5, 5, 3), (2, 2, 1))
    assert e.value.status == L.OOM
    torch.cuda.synchronize()
    assert bool((out == 7).all()), "a failed call must launch nothing"
    # the fused kernel needs no temporaries: unaffected
    f = torch.empty(a.shape, dtype=torch.uint8, device="cuda")
    clk.separable("maximum_separable_3d", src, f, (5, 5, 3), (2, 2, 1))
    torch.cuda.synchronize()
    assert np.array_equal(f.cpu().numpy(), oracle.separable("maximum_separable_3d", a, np.uint8, (5, 5, 3), (2, 2, 1)))
    monkeypatch.delenv("CLK_INJECT_ALLOC_FAILURE")
    clk.separable("mean_separable_3d", src, out, (5, 5, 3), (2, 2, 1))
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.separable("mean_separable_3d", a, np.uint16, (5, 5, 3), (2, 2, 1)))


def test_morphology_oom(env, oracle, monkeypatch):
    torch, clk, L = env
    rng = np.random.default_rng(4)
    m = (rng.random((10, 33, 64)) < 0.7).astype(np.uint8)
    src = torch.from_numpy(m).cuda()
    out = torch.full(m.shape, 9, dtype=torch.uint8, device="cuda")
    monkeypatch.setenv("CLK_INJECT_ALLOC_FAILURE", "1")
    with pytest.raises(L.ClkError) as e:
        clk.morphology("erode_sphere_3d", src, out, 3)
    assert e.value.status == L.OOM
    torch.cuda.synchronize()
    assert bool((out == 9).all())
    clk.morphology("erode_sphere_3d", src, out, 2)  # fused pair: one step, no temporary
    torch.cuda.synchronize()
    want = m
    for _ in range(2):
        want = oracle.execute("erode_sphere_3d", want, np.uint8)
    assert np.array_equal(out.cpu().numpy(), want)
    monkeypatch.delenv("CLK_INJECT_ALLOC_FAILURE")
    clk.morphology("erode_sphere_3d", src, out, 3)
    torch.cuda.synchronize()
    want = oracle.execute("erode_sphere_3d", want, np.uint8)
    assert np.array_equal(out.cpu().numpy(), want)


def test_batch_create_oom(env, monkeypatch):
    torch, clk, L = env
    imgs = [torch.zeros((8, 32, 64), dtype=torch.uint16, device="cuda") for _ in range(3)]
    outs = [torch.empty_like(t) for t in imgs]
    ops = [clk.op_separable("minimum_separable", (3, 3, 3), (1, 1, 1)),
           clk.op_separable("maximum_separable", (3, 3, 3), (1, 1, 1))]
    monkeypatch.setenv("CLK_INJECT_ALLOC_FAILURE", "1")
    with pytest.raises(L.ClkError) as e:
        clk.Batch(ops, imgs, outs)
    assert e.value.status == L.OOM
    monkeypatch.delenv("CLK_INJECT_ALLOC_FAILURE")
    b = clk.Batch(ops, imgs, outs)
    b.run()
    torch.cuda.synchronize()
    b.close()


def test_server_request_oom(env, oracle, monkeypatch):
    torch, clk, L = env
    rng = np.random.default_rng(5)
    a = rng.integers(0, 4000, size=(6, 30, 64)).astype(np.uint16)
    src = torch.from_numpy(a).cuda()
    out = torch.full(a.shape, 5, dtype=torch.uint16, device="cuda")
    ops = [clk.op_kernel("median_box", (3, 3, 3)), clk.op_separable("mean_separable", (3, 3, 3), (1, 1, 1))]
    srv = clk.Server(slots=2, hbm_budget_bytes=1 << 30)
    try:
        monkeypatch.setenv("CLK_INJECT_ALLOC_FAILURE", "1")
        t = srv.submit(ops, src, out)
        with pytest.raises(L.ClkError) as e:
            srv.wait(t)
        assert e.value.status == L.OOM
        monkeypatch.delenv("CLK_INJECT_ALLOC_FAILURE")
        assert srv.stats()["failed"] == 1
        torch.cuda.synchronize()
        assert bool((out == 5).all())
        srv.wait(srv.submit(ops, src, out))
        torch.cuda.synchronize()
        want = oracle.separable("mean_separable_3d", oracle.execute("median_box_3d", a, np.uint16, (3, 3, 3)),
                                np.uint16, (3, 3, 3), (1, 1, 1))
        assert np.array_equal(out.cpu().numpy(), want)
    finally:
        srv.close()


def test_server_cancel_queued_request(env):
    torch, clk, L = env
    big = torch.randint(0, 60000, (192, 1024, 1024), dtype=torch.int32, device="cuda").to(torch.uint16)
    big_out = torch.empty_like(big)
    small = torch.randint(0, 60000, (8, 64, 64), dtype=torch.int32, device="cuda").to(torch.uint16)
    outs = [torch.full_like(small, 11) for _ in range(4)]
    heavy = [clk.op_kernel("median_sphere", (5, 5, 5)) for _ in range(3)]
    srv = clk.Server(slots=1, hbm_budget_bytes=0)
    try:
        t0 = srv.submit(heavy, big, big_out)  # occupies the only slot for several ms
        ts = [srv.submit([clk.op_kernel("median_box", (3, 3, 3))], small, o) for o in outs]
        srv.cancel(ts[2])
        srv.cancel(ts[3])
        srv.wait(t0)
        srv.wait(ts[0])
        srv.wait(ts[1])
        for t in ts[2:]:
            with pytest.raises(L.ClkError) as e:
                srv.wait(t)
            assert e.value.status == L.CANCELLED
        torch.cuda.synchronize()
        assert bool((outs[2] == 11).all()) and bool((outs[3] == 11).all()), "a cancelled request ran"
        assert not bool((outs[0] == 11).all())
        st = srv.stats()
        assert st["cancelled"] == 2 and st["completed"] == 3
        # running or finished requests cannot be cancelled
        t = srv.submit(heavy, big, big_out)
        import time
        deadline = time.time() + 5
        while srv.stats()["inflight"] == 0 and time.time() < deadline:
            time.sleep(0.0005)
        with pytest.raises(L.ClkError) as e:
            srv.cancel(t)
        assert e.value.status == L.BUSY
        srv.wait(t)
    finally:
        srv.close()
