"""The oracle restatement against the committed reference outputs."""
import numpy as np

import golden_cases


def test_golden_fixtures_cover_every_kernel(oracle):
    kernels = {c["kernel"] for c, _, _ in golden_cases.load()}
    assert kernels == set(oracle.KERNELS)


def test_port_matches_golden(oracle):
    n = 0
    for c, a, want in golden_cases.load():
        dt = golden_cases.NP[c["dst"]]
        if c["kind"] == "convolve":
            got = oracle.execute(c["kernel"], a, dt, kernel_image=c["kernel_image"])
        elif c["kind"] == "execute":
            ints, floats = golden_cases.split_params(c["params"])
            got = oracle.execute(c["kernel"], a, dt, ints, floats)
        else:
            got = oracle.separable(c["kernel"], a, dt, c["params"]["N"], c["params"]["s"])
        assert got.tobytes() == want.tobytes(), c
        n += 1
    assert n > 800
