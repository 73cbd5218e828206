"""GPU tests of the served form (clk_server_*): requests with random
pipelines over images of uneven shape and pixel type, admitted as slots and
HBM budget free up and run concurrently.  Each result must be the same alone
(one slot, one request at a time) and in the mix (many slots, all in flight),
bit for bit; admission must respect the budget; errors surface."""
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


def random_pipeline(clk, rng):
    """1-4 steps from {gaussian s in [1,4], mean r in [1,5], median_box r=1,
    erode/dilate_sphere r in [1,2], sobel}."""
    ops = []
    for _ in range(int(rng.integers(1, 5))):
        k = int(rng.integers(0, 6))
        if k == 0:
            s = float(rng.uniform(1, 4))
            n = 2 * int(np.ceil(3 * s)) + 1
            ops.append(clk.op_separable("gaussian_blur_separable", (n, n, n), (s, s, s)))
        elif k == 1:
            r = int(rng.integers(1, 6))
            ops.append(clk.op_separable("mean_separable", (2 * r + 1,) * 3, (r, r, r)))
        elif k == 2:
            ops.append(clk.op_kernel("median_box", (3, 3, 3)))
        elif k in (3, 4):
            ops.append(clk.op_morphology("erode_sphere" if k == 3 else "dilate_sphere", int(rng.integers(1, 3))))
        else:
            ops.append(clk.op_kernel("sobel"))
    return ops


def make_requests(clk, rng, n):
    import torch
    reqs = []
    for k in range(n):
        dt = [np.uint8, np.uint16, np.float32][k % 3]
        if k % 2:
            shp = (int(rng.integers(3, 20)), int(rng.integers(16, 70)), int(rng.integers(16, 90)))
        else:
            shp = (int(rng.integers(16, 120)), int(rng.integers(16, 150)))
        a = np.abs(random_image(rng, shp, dt))
        reqs.append((random_pipeline(clk, rng), torch.from_numpy(a).cuda()))
    return reqs


def serve(clk, reqs, slots, budget=64 << 30, serial=False):
    import torch
    srv = clk.Server(slots=slots, hbm_budget_bytes=budget)
    outs = [torch.empty_like(src) for _, src in reqs]
    if serial:
        for (ops, src), out in zip(reqs, outs):
            srv.wait(srv.submit(ops, src, out))
    else:
        tickets = [srv.submit(ops, src, out) for (ops, src), out in zip(reqs, outs)]
        for t in tickets:
            srv.wait(t)
    st = srv.stats()
    srv.close()
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs], st


def test_result_same_alone_and_in_the_mix(clk):
    rng = np.random.default_rng(61)
    reqs = make_requests(clk, rng, 48)
    alone, st1 = serve(clk, reqs, slots=1, serial=True)
    mixed, st8 = serve(clk, reqs, slots=8)
    assert st1["completed"] == st8["completed"] == len(reqs)
    for k, (a, m) in enumerate(zip(alone, mixed)):
        assert a.tobytes() == m.tobytes(), (k, reqs[k][1].shape, [o["kernel"] for o in reqs[k][0]])
    assert st8["p50_ms"] > 0 and st8["p99_ms"] >= st8["p50_ms"]


def test_admission_respects_the_budget(clk):
    rng = np.random.default_rng(62)
    reqs = make_requests(clk, rng, 24)
    need = max(2 * ((src.numel() * src.element_size() + 255) // 256 * 256) for _, src in reqs)
    budget = 3 * need
    _, st = serve(clk, reqs, slots=16, budget=budget)
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert 0 < st["bytes_peak"] <= budget


def test_server_errors(clk):
    import torch
    srv = clk.Server(slots=2, hbm_budget_bytes=1024)
    src = torch.zeros((8, 64, 64), dtype=torch.uint16, device="cuda")
    ops = [clk.op_kernel("median_box", (3, 3, 3)), clk.op_kernel("sobel")]
    with pytest.raises(clk.ClkError):  # needs more temporaries than the budget
        srv.submit(ops, src, torch.empty_like(src))
    with pytest.raises(clk.ClkError):
        srv.wait(123456789)
    srv.close()


def oracle_pipeline(clk, oracle, ops, a):
    """The request's steps on the CPU, one oracle call per reference launch:
    separable filters X -> Y (-> Z) with dst-typed temporaries, median and
    sobel as one launch each, radius-r morphology as r launches of the r=1
    kernel; every intermediate in the request's pixel type."""
    from clk import _lib as L
    nd = a.ndim
    sfx = "_2d" if nd == 2 else "_3d"
    cur = a
    for op in ops:
        name = op["kernel"] + sfx
        if op["kind"] == L.OP_SEPARABLE:
            cur = oracle.separable(name, cur, a.dtype, op["N"][:nd], op["s"][:nd])
        elif op["kind"] == L.OP_MORPHOLOGY:
            for _ in range(op["iterations"]):
                cur = oracle.execute(name, cur, a.dtype)
        elif op["kernel"].startswith("median"):
            cur = oracle.execute(name, cur, a.dtype, op["N"][:nd])
        else:
            cur = oracle.execute(name, cur, a.dtype)
    return cur


def test_served_integer_results_match_the_oracle(clk, oracle):
    # Integer requests served in the mix (8 slots, all in flight) against the
    # oracle run step by step: bit for bit.
    import torch
    rng = np.random.default_rng(63)
    reqs = [r for r in make_requests(clk, rng, 60) if r[1].dtype != torch.float32]
    mixed, st = serve(clk, reqs, slots=8)
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for k, ((ops, src), got) in enumerate(zip(reqs, mixed)):
        want = oracle_pipeline(clk, oracle, ops, src.cpu().numpy())
        assert np.array_equal(got, want), (k, src.shape, src.dtype, [o["kernel"] for o in ops])
