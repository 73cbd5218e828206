"""Recipe for oracle/_ref: the reference's own kernels run on the host.

TEST INFRASTRUCTURE ONLY.  The reference (clEsperanto/clij-opencl-kernels) is
OpenCL C source with no host code and no OpenCL platform exists here, so its
hot-path kernels are compiled as C++ against oracle/cl_shim.h, which restates
the preamble (clamp-to-edge buffer reads, saturating convert).  The result,
oracle/_ref/libclkref.so, is both a parity witness for the oracle restatement
(oracle/clk_oracle.cpp) and the "reference" CPU baseline timed by bench.py.

Two steps, so that the second can run where the reference is absent:
  generate(): read kernels/<name>_x.cl from the reference checkout, apply the
      textual pre-pass below, write oracle/_ref/gen/<name>.cpp (one namespace
      per src/dst pixel-type pair).  Needs the reference checkout.
  compile():  g++ -O3 -fopenmp -ffp-contract=off the generated files into
      oracle/_ref/libclkref.so.  Needs only oracle/_ref/gen.
oracle/_ref/ is git-ignored: nothing derived from the reference's text is
committed.

Pre-pass (the only edits; each keeps the kernel's arithmetic unchanged):
  * OpenCL vector literals "(int2)(a,b)" / "(int4)(a,b,c,d)" become
    "int2{a,b}" / "int4{...}" (as C++ they would parse as a cast of a comma
    expression), e.g. gaussian_blur_separable_3d_x.cl:18-19.
  * sobel_3d_x.cl:17-19 "int g?[3][3][3];" become CLK_SOBEL_ARRAY(g?): the same
    arrays followed by one zero int, pinning the out-of-range tap of
    sobel_3d_x.cl:46-49 to 0.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
GEN_DIR = REF_DIR / "gen"
LIB = REF_DIR / "libclkref.so"
# The reference checkout: the argument of build() / generate(), else the
# environment variable CLK_REFERENCE_DIR.  There is no default location.
REFERENCE_ENV = "CLK_REFERENCE_DIR"


def reference_dir(reference: Path | str | None = None) -> Path | None:
    if reference is None:
        reference = os.environ.get(REFERENCE_ENV) or None
    return Path(reference) if reference else None

KERNELS = [
    "gaussian_blur_separable_2d", "gaussian_blur_separable_3d",
    "mean_separable_2d", "mean_separable_3d",
    "minimum_separable_2d", "minimum_separable_3d",
    "maximum_separable_2d", "maximum_separable_3d",
    "median_box_2d", "median_box_3d", "median_sphere_2d", "median_sphere_3d",
    "erode_box_2d", "erode_box_3d", "erode_sphere_2d", "erode_sphere_3d",
    "dilate_box_2d", "dilate_box_3d", "dilate_sphere_2d", "dilate_sphere_3d",
    "sobel_2d", "sobel_3d",
    # the neighbourhood filters either side of the path
    "minimum_sphere_2d", "minimum_sphere_3d", "maximum_sphere_2d", "maximum_sphere_3d",
    "mean_sphere_2d", "mean_sphere_3d",
    "minimum_slice_by_slice_sphere_3d", "maximum_slice_by_slice_sphere_3d", "mean_slice_by_slice_sphere_3d",
    "median_slice_by_slice_box_3d", "median_slice_by_slice_sphere_3d",
    "erode_box_slice_by_slice_3d", "erode_sphere_slice_by_slice_3d",
    "dilate_box_slice_by_slice_3d", "dilate_sphere_slice_by_slice_3d",
    "greater_constant_2d", "greater_constant_3d", "copy_2d", "copy_3d",
    "gradient_x_2d", "gradient_y_2d", "gradient_x_3d", "gradient_y_3d", "gradient_z_3d",
    "laplace_box_2d", "laplace_box_3d", "laplace_diamond_2d", "laplace_diamond_3d",
    "convolve_2d", "convolve_3d",
]
# pixel types in clk_dtype order (include/clk.h)
DTYPES = [("u8", "uint8_t"), ("i8", "int8_t"), ("u16", "uint16_t"),
          ("i16", "int16_t"), ("f32", "float")]


def _vector_literals(text: str) -> str:
    out, i = [], 0
    pat = re.compile(r"\((int2|int4)\)\s*\(")
    while True:
        m = pat.search(text, i)
        if not m:
            out.append(text[i:])
            return "".join(out)
        out.append(text[i:m.start()])
        j, depth = m.end(), 1
        while depth:
            c = text[j]
            depth += (c == "(") - (c == ")")
            j += 1
        out.append(m.group(1) + "{" + _vector_literals(text[m.end():j - 1]) + "}")
        i = j


def _params(text: str, name: str):
    m = re.search(r"__kernel\s+void\s+" + name + r"\s*\((.*?)\)\s*\{", text, re.S)
    if not m:
        raise RuntimeError(f"no __kernel {name}")
    params = []
    for p in m.group(1).split(","):
        p = p.strip()
        ident = re.findall(r"[A-Za-z_]\w*", p)[-1]
        if "IMAGE_" in p:
            params.append(("image", ident))
        elif re.search(r"\bfloat\b", p):
            params.append(("float", ident))
        elif re.search(r"\bint\b", p):
            params.append(("int", ident))
        else:
            raise RuntimeError(f"{name}: unknown parameter {p!r}")
    return params


def generate(reference: Path | str | None = None) -> list[Path]:
    reference = reference_dir(reference)
    if reference is None:
        raise RuntimeError(f"no reference checkout: pass its path or set {REFERENCE_ENV}")
    GEN_DIR.mkdir(parents=True, exist_ok=True)
    files = []
    for k in KERNELS:
        text = (reference / "kernels" / f"{k}_x.cl").read_text()
        text = _vector_literals(text)
        if k == "sobel_3d":
            for g in ("gx", "gy", "gz"):
                text, n = re.subn(r"int\s+" + g + r"\s*\[3\]\[3\]\[3\]\s*;",
                                  f"CLK_SOBEL_ARRAY({g});", text)
                assert n == 1, g
        params = _params(text, k)
        body = [f"// generated by oracle/build_ref.py from kernels/{k}_x.cl",
                '#include "../../cl_shim.h"', '#include "../../ref_loop.h"']
        for sn, st in DTYPES:
            for dn, dt in DTYPES:
                body.append(f"namespace clkcl {{ namespace {k}__{sn}_{dn} {{")
                body.append(f"typedef {st} SRC_T; typedef {dt} DST_T;")
                body.append(text)
                body.append("}}")
        body.append(f'extern "C" int clkref_{k}(int sdt, int ddt, const clkref_call* c) {{')
        body.append("  switch (sdt * 5 + ddt) {")
        for si, (sn, st) in enumerate(DTYPES):
            for di, (dn, dt) in enumerate(DTYPES):
                ns = f"clkcl::{k}__{sn}_{dn}"
                args, ni, nf = [], 0, 0
                for kind, ident in params:
                    if kind == "image":  # src / src1 -> the input, dst -> the output
                        args.append("src" if ident.startswith("src") else ident)
                    elif kind == "int":
                        args.append(f"c->ia[{ni}]"); ni += 1
                    else:
                        args.append(f"c->fa[{nf}]"); nf += 1
                kimg = (" clkcl::clk_img<float> kernelImage{(float*)c->kimg, c->kw, c->kh, c->kd};"
                        if any(ident == "kernelImage" for _, ident in params) else "")
                body.append(
                    f"  case {si * 5 + di}: {{ clkcl::clk_img<{st}> src{{({st}*)c->src, c->sw, c->sh, c->sd}};"
                    f" clkcl::clk_img<{dt}> dst{{({dt}*)c->dst, c->dw, c->dh, c->dd}};{kimg}"
                    f" clkref_loop(c, [&] {{ {ns}::{k}({', '.join(args)}); }}); return 0; }}")
        body.append("  default: return -1;\n  }\n}")
        out = GEN_DIR / f"{k}.cpp"
        out.write_text("\n".join(body) + "\n")
        files.append(out)
    (GEN_DIR / "common.cpp").write_text(
        '#include "../../cl_shim.h"\nthread_local int clkcl::clk_gid[3];\n')
    return files


def compile(jobs: int | None = None, cxx: str = "g++") -> Path:
    srcs = sorted(GEN_DIR.glob("*.cpp"))
    if not srcs:
        raise RuntimeError("oracle/_ref/gen is empty: run generate() where the reference exists")
    flags = ["-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
             "-std=c++17", "-w"]
    objs = []

    def one(src: Path) -> Path:
        obj = src.with_suffix(".o")
        # sobel_3d's out-of-range tap is undefined behaviour in C++ too; at
        # -O2/-O3 g++ folds the constant arrays and exploits it (results then
        # match no memory layout), at -O1 indexing stays flat address
        # arithmetic over the padded arrays, as the pinned policy states.
        extra = (["-O1", "-fno-aggressive-loop-optimizations"] if src.stem == "sobel_3d" else [])
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime,
                                                          (HERE / "cl_shim.h").stat().st_mtime,
                                                          (HERE / "ref_loop.h").stat().st_mtime):
            subprocess.run([cxx, *flags, *extra, "-c", str(src), "-o", str(obj)], check=True)
        return obj

    with cf.ThreadPoolExecutor(jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(one, srcs))
    subprocess.run([cxx, "-shared", "-fopenmp", "-o", str(LIB), *map(str, objs)], check=True)
    return LIB


def build(reference: Path | str | None = None) -> Path | None:
    """Generate (when a reference checkout is given and present) and compile;
    None if neither the reference nor previously generated sources are
    available."""
    reference = reference_dir(reference)
    if reference is not None and (reference / "kernels").is_dir():
        generate(reference)
    if not any(GEN_DIR.glob("*.cpp")):
        return None
    return compile()


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
