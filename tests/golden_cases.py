"""Loader for tests/golden/golden.npz (outputs of the reference's kernels)."""
import json
import pathlib

import numpy as np

PATH = pathlib.Path(__file__).resolve().parent / "golden" / "golden.npz"
NP = {"u8": np.uint8, "i8": np.int8, "u16": np.uint16, "i16": np.int16, "f32": np.float32}


def load():
    z = np.load(PATH)
    index = json.loads(bytes(z["index"]).decode())
    for c in index:
        if c["key"] + "_k" in z:  # convolve: its float kernel image
            c = dict(c, kernel_image=z[c["key"] + "_k"])
        yield c, z[c["key"] + "_in"], z[c["key"] + "_out"]


FLOAT_PARAMS = ("s", "scalar")


def split_params(params):
    ints = [v for n, v in params.items() if n not in FLOAT_PARAMS]
    floats = [v for n, v in params.items() if n in FLOAT_PARAMS]
    return ints, floats
