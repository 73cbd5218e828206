"""Generate tests/golden/golden.npz from the reference's own kernels.

The reference repository has no tests, fixtures or golden vectors.  These
fixtures are outputs of its .cl kernels themselves, compiled on the host by
oracle/build_ref.py (oracle/_ref), on small seeded inputs: every hot-path
kernel, several pixel-type pairs, border-heavy extents and parameters.  The
committed file lets the oracle and the CUDA library be checked against the
reference where the reference checkout is absent.

    python oracle/build_ref.py <reference checkout> && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"

PAIRS_SEP = [("u16", "u16"), ("u16", "f32"), ("u8", "u8"), ("f32", "f32"), ("i16", "i16"), ("f32", "u8"),
             ("i8", "f32")]
PAIRS_MEDIAN = [("u16", "u16"), ("u8", "u8"), ("f32", "f32"), ("i8", "i8"), ("i16", "i16")]
PAIRS_MORPH = [("u8", "u8"), ("u16", "u16"), ("f32", "f32"), ("u8", "f32"), ("i16", "u8")]
PAIRS_SOBEL = [("u16", "f32"), ("u8", "f32"), ("f32", "f32"), ("i16", "f32"), ("u16", "u16"), ("i8", "i8")]
NP = {"u8": np.uint8, "i8": np.int8, "u16": np.uint16, "i16": np.int16, "f32": np.float32}


def image(rng, shape, dt, binary=False):
    dt = np.dtype(NP[dt])
    if dt == np.float32:
        a = (rng.standard_normal(shape) * 300).astype(np.float32)
    else:
        info = np.iinfo(dt)
        a = rng.integers(info.min, int(info.max) + 1, size=shape).astype(dt)
    if binary:
        a = (a * (rng.random(shape) < 0.85)).astype(dt)
    return a


def main() -> None:
    if not O.ref_available():
        raise SystemExit("build oracle/_ref first: python oracle/build_ref.py")
    rng = np.random.default_rng(20240601)
    arrays, index = {}, []

    def add(kind, kernel, sdt, ddt, params, a, out, kimg=None):
        key = f"c{len(index):04d}"
        arrays[key + "_in"] = a
        arrays[key + "_out"] = out
        if kimg is not None:
            arrays[key + "_k"] = kimg
        index.append({"key": key, "kind": kind, "kernel": kernel, "src": sdt, "dst": ddt, "params": params})

    for k in O.KERNELS:
        is2 = k.endswith("2d")
        if k.startswith("convolve"):
            for shp in ([(10, 13), (1, 6)] if is2 else [(5, 7, 9), (1, 3, 8)]):
                for sdt, ddt in PAIRS_SEP:
                    a = image(rng, shp, sdt)
                    for ks in (((3, 3), (4, 2)) if is2 else ((3, 3, 3), (2, 3, 4))):
                        kimg = rng.standard_normal(ks).astype(np.float32)
                        out = O.execute(k, a, NP[ddt], impl="ref", kernel_image=kimg)
                        add("convolve", k, sdt, ddt, {"kernel_shape": list(ks)}, a, out, kimg)
            continue
        shapes = [(10, 13), (1, 6)] if is2 else [(5, 7, 9), (1, 3, 8)]
        if "slice_by_slice" in k and not k.startswith(("erode", "dilate")):
            pairs = PAIRS_MEDIAN if k.startswith("median") else PAIRS_SEP
            cases = [{"Nx": 3, "Ny": 3}, {"Nx": 5, "Ny": 5}, {"Nx": 5, "Ny": 3}]
        elif "_sphere_" in k and k.startswith(("minimum", "maximum", "mean")):
            pairs = [p for p in PAIRS_SEP if not (k == "minimum_sphere_2d" and p[0] == "f32" and p[1] != "f32")]
            cases = ([{"Nx": 3, "Ny": 3}, {"Nx": 5, "Ny": 5}, {"Nx": 5, "Ny": 3}] if is2 else
                     [{"Nx": 3, "Ny": 3, "Nz": 3}, {"Nx": 5, "Ny": 5, "Nz": 5}, {"Nx": 3, "Ny": 5, "Nz": 1}])
        elif k.startswith("greater_constant"):
            pairs = PAIRS_SEP
            cases = [{"scalar": 400.0}, {"scalar": -2.5}]
        elif k.startswith("copy"):
            pairs, cases = PAIRS_SEP, [{}]
        elif k.startswith(("gaussian", "mean", "minimum", "maximum")):
            pairs = PAIRS_SEP
            cases = [{"dim": d, "N": N, "s": s} for d in ((0, 1) if is2 else (0, 1, 2))
                     for N, s in ((5, 1.0), (8, 2.5))]
        elif k.startswith("median"):
            pairs = PAIRS_MEDIAN
            cases = ([{"Nx": 3, "Ny": 3}, {"Nx": 5, "Ny": 5}, {"Nx": 5, "Ny": 3}] if is2 else
                     [{"Nx": 3, "Ny": 3, "Nz": 3}, {"Nx": 5, "Ny": 5, "Nz": 5}, {"Nx": 3, "Ny": 5, "Nz": 1}])
        elif k.startswith(("erode", "dilate")):
            pairs, cases = PAIRS_MORPH, [{}]
        else:
            pairs, cases = PAIRS_SOBEL, [{}]
        for shp in shapes:
            for sdt, ddt in pairs:
                a = image(rng, shp, sdt, binary=k.startswith(("erode", "dilate")))
                for c in cases:
                    ints = [v for n, v in c.items() if n not in ("s", "scalar")]
                    floats = [v for n, v in c.items() if n in ("s", "scalar")]
                    out = O.execute(k, a, NP[ddt], ints, floats, impl="ref")
                    add("execute", k, sdt, ddt, c, a, out)
    for k in ("gaussian_blur_separable_3d", "mean_separable_3d", "minimum_separable_3d", "maximum_separable_3d",
              "gaussian_blur_separable_2d", "mean_separable_2d", "minimum_separable_2d", "maximum_separable_2d"):
        shp = (11, 14) if k.endswith("2d") else (6, 10, 12)
        for sdt, ddt in (("u16", "u16"), ("u16", "f32"), ("u8", "u8"), ("f32", "f32")):
            a = image(rng, shp, sdt)
            for N, s in (((7, 5, 3), (1.5, 1.0, 0.5)), ((1, 9, 5), (0.0, 2.0, 1.0))):
                out = O.separable(k, a, NP[ddt], N, s, impl="ref")
                add("separable", k, sdt, ddt, {"N": list(N), "s": list(s)}, a, out)
    arrays["index"] = np.frombuffer(json.dumps(index).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"{OUT}: {len(index)} cases, {OUT.stat().st_size / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
