"""Generate clk_median_networks.cuh: the comparator networks of the fast
median kernels (clk_median.cu).

    python clij-opencl-kernels_gb300/csrc/gen_median_networks.py

The median of a neighbourhood is an order statistic, so any network that
selects the right rank gives the reference's result exactly for integer
pixels (median_box_3d_x.cl:3-20 sorts and takes element n/2).  The networks
are built from Batcher odd-even merges of already sorted lists and pruned
backwards to the ranks that are actually consumed: a comparator whose min
(or max) is never used becomes a single max (or min), one whose outputs are
both unused disappears; the sphere's final selections end with the identity
for two sorted lists C[k] = min_i max(S[i-1], X[k-i]).  Every network is
checked here on all 0/1 inputs of its sorted-input structure (0-1
principle: exhaustively over the ones-counts of its sorted groups and every
0/1 pattern of its free wires) and on random values.

Networks (V is a SIMD word: two 16-bit lanes, one output each):
  net_sort3            sort three values (a z- or y-column, or an x-row)
  net_merge333         three sorted triples -> sorted 9 (3x3 block of a plane)
  net_merge33          two sorted triples -> sorted 6 (rows shared by a y pair)
  net_merge63          sorted 6 + sorted triple -> sorted 9
  net_merge99_mid      two sorted 9s -> ranks 4..13 of their merge
  net_box27_final      rank 9 of (ranks 4..13 of 18) U (sorted 9) = median of 27
  net_sphere33_final   rank 16 of (sorted 9 U sorted 9 U sorted 9 U 4 U 2) = median of 33
  net_merge99_r1_16    two sorted 9s -> ranks 1..16 (the shared merge of a z pair)
  net_sphere33_pair_final  rank 15 of (ranks 1..16 U sorted 9 U 6) = median of 33
  net_sort4 / net_sort2 helpers
"""
from __future__ import annotations

import itertools
import random
from pathlib import Path

OUT = Path(__file__).resolve().parent / "clk_median_networks.cuh"


def oe_merge(a: list[int], b: list[int], net: list) -> list[int]:
    """Odd-even merge of sorted wire lists a, b; appends comparators (lo, hi)
    (after one, wire lo holds the min) and returns the wires in rank order."""
    if not a:
        return list(b)
    if not b:
        return list(a)
    if len(a) == 1 and len(b) == 1:
        net.append((a[0], b[0]))
        return [a[0], b[0]]
    e = oe_merge(a[0::2], b[0::2], net)
    o = oe_merge(a[1::2], b[1::2], net)
    out = [e[0]]
    i = 0
    while i < len(o) and i + 1 < len(e):
        net.append((o[i], e[i + 1]))
        out += [o[i], e[i + 1]]
        i += 1
    out += o[i:] + e[i + 1:]
    return out


def prune(net, needed):
    """Backward pruning: keep what the needed wires depend on."""
    need = set(needed)
    prog = []
    for lo, hi in reversed(net):
        nl, nh = lo in need, hi in need
        if not (nl or nh):
            continue
        prog.append(("cmp" if nl and nh else ("min" if nl else "max"), lo, hi))
        need |= {lo, hi}
    return list(reversed(prog))


def run(prog, vals):
    a = list(vals)
    for k, lo, hi in prog:
        x, y = a[lo], a[hi]
        if k == "cmp":
            a[lo], a[hi] = min(x, y), max(x, y)
        elif k == "min":
            a[lo] = min(x, y)
        else:
            a[hi] = max(x, y)
    return a


def ops(prog):
    return sum(2 if k == "cmp" else 1 for k, _, _ in prog)


def verify(prog, n, groups, checks, exhaustive=True, trials=20000):
    """groups: sorted input runs (lists of wires); checks(vals, out) -> bool."""
    rng = random.Random(1)

    def make(bits):
        v = list(bits)
        for g in groups:
            s = sorted(v[w] for w in g)
            for w, x in zip(g, s):
                v[w] = x
        return v

    if exhaustive and n <= 22:
        for bits in itertools.product((0, 1), repeat=n):
            v = make(bits)
            assert checks(v, run(prog, v)), (bits,)
    for _ in range(trials):
        v = make([rng.randint(0, 9) for _ in range(n)])
        assert checks(v, run(prog, v)), v


def verify_01_groups(prog, n, groups, rank, out_wire):
    """Exhaustive 0-1 check of a selection network whose inputs are sorted
    groups plus free wires: a sorted 0/1 group is fixed by its count of ones,
    so every 0/1 input of that structure is enumerated (by the 0-1
    principle, a min/max network that selects rank `rank` on all of them
    selects it on every input)."""
    grouped = {w for g in groups for w in g}
    free = [w for w in range(n) if w not in grouped]
    for counts in itertools.product(*[range(len(g) + 1) for g in groups]):
        base = [0] * n
        for g, c in zip(groups, counts):
            for w in g[len(g) - c:]:
                base[w] = 1
        for bits in itertools.product((0, 1), repeat=len(free)):
            v = list(base)
            for w, b in zip(free, bits):
                v[w] = b
            assert run(prog, v)[out_wire] == sorted(v)[rank], (counts, bits)


def emit(name, n, prog, args_doc):
    lines = [f"// {args_doc}", f"// {ops(prog)} min/max operations",
             f"template <class V> CLK_NET_FN void {name}(V (&w)[{n}]) {{"]
    for k, lo, hi in prog:
        if k == "cmp":
            lines.append(f"  {{ const V t = vmin(w[{lo}], w[{hi}]); w[{hi}] = vmax(w[{lo}], w[{hi}]); w[{lo}] = t; }}")
        elif k == "min":
            lines.append(f"  w[{lo}] = vmin(w[{lo}], w[{hi}]);")
        else:
            lines.append(f"  w[{hi}] = vmax(w[{lo}], w[{hi}]);")
    lines.append("}")
    return "\n".join(lines)


def main():
    parts = []
    stats = {}

    # sort3
    net = []
    r = oe_merge(oe_merge([0], [1], net), [2], net)
    assert r == [0, 1, 2] or sorted(r) == [0, 1, 2]
    prog = prune(net, [0, 1, 2])
    order = r
    verify(prog, 3, [], lambda v, o: [o[w] for w in order] == sorted(v))
    stats["sort3"] = ops(prog)
    parts.append(("net_sort3_raw", 3, prog, order, "w[0..2] -> ranks in order " + str(order)))

    # merge333: wires 0-2, 3-5, 6-8 sorted triples -> sorted 9
    net = []
    r = oe_merge(oe_merge([0, 1, 2], [3, 4, 5], net), [6, 7, 8], net)
    prog = prune(net, r)
    verify(prog, 9, [[0, 1, 2], [3, 4, 5], [6, 7, 8]], lambda v, o: [o[w] for w in r] == sorted(v))
    stats["merge333"] = ops(prog)
    parts.append(("net_merge333_raw", 9, prog, r, "three sorted triples w[0..2], w[3..5], w[6..8] -> sorted 9"))

    # merge33: two sorted triples w[0..2], w[3..5] -> sorted 6 (the two rows
    # a y-pair of box-median outputs shares)
    net = []
    r = oe_merge([0, 1, 2], [3, 4, 5], net)
    prog = prune(net, r)
    verify(prog, 6, [[0, 1, 2], [3, 4, 5]], lambda v, o: [o[w] for w in r] == sorted(v))
    stats["merge33"] = ops(prog)
    parts.append(("net_merge33_raw", 6, prog, r, "sorted triples w[0..2], w[3..5] -> sorted 6"))

    # merge63: sorted 6 w[0..5] and sorted triple w[6..8] -> sorted 9 (a
    # 3x3 block from the shared pair of rows and its own third row)
    net = []
    r = oe_merge(list(range(6)), [6, 7, 8], net)
    prog = prune(net, r)
    verify(prog, 9, [list(range(6)), [6, 7, 8]], lambda v, o: [o[w] for w in r] == sorted(v))
    stats["merge63"] = ops(prog)
    parts.append(("net_merge63_raw", 9, prog, r, "sorted 6 w[0..5] and sorted triple w[6..8] -> sorted 9"))

    # merge99_mid: wires 0-8 and 9-17 sorted -> ranks 4..13
    net = []
    r = oe_merge(list(range(9)), list(range(9, 18)), net)
    prog = prune(net, r[4:14])
    verify(prog, 18, [list(range(9)), list(range(9, 18))],
           lambda v, o: [o[w] for w in r[4:14]] == sorted(v)[4:14], exhaustive=True)
    stats["merge99_mid"] = ops(prog)
    parts.append(("net_merge99_mid_raw", 18, prog, r[4:14], "sorted 9s w[0..8], w[9..17] -> ranks 4..13"))

    # box27 final: wires 0-9 = ranks 4..13 of an 18-merge (sorted), 10-18 sorted 9 -> rank 9 of 19
    net = []
    r = oe_merge(list(range(10)), list(range(10, 19)), net)
    prog = prune(net, [r[9]])
    verify(prog, 19, [list(range(10)), list(range(10, 19))], lambda v, o: o[r[9]] == sorted(v)[9])
    stats["box27_final"] = ops(prog)
    parts.append(("net_box27_final_raw", 19, prog, [r[9]], "sorted 10 w[0..9] U sorted 9 w[10..18] -> rank 9"))

    # sphere33 final: 0-8, 9-17 sorted 9 (planes z-1, z+1); 18-26 sorted 9 (plane z);
    # 27-30 four singles (x+-2, y+-2 in plane z); 31, 32 singles (z-2, z+2).
    # The three sorted 9s merged for ranks 10..16 only, the six singles
    # sorted, rank 16 of the union by C[k] = min over i of max(S[i-1],
    # X[k-i]), i = 0..6 (146 operations against 166 for the best pruned
    # merge tree)
    net = []
    x = oe_merge(oe_merge(list(range(9)), list(range(9, 18)), net), list(range(18, 27)), net)
    prog = prune(net, [x[16 - i] for i in range(7)])
    net = []
    s4 = oe_merge(oe_merge([27], [28], net), oe_merge([29], [30], net), net)
    s6 = oe_merge(s4, oe_merge([31], [32], net), net)
    prog += prune(net, s6)
    for i in range(1, 7):
        prog.append(("max", s6[i - 1], x[16 - i]))
    for i in range(1, 7):
        prog.append(("min", x[16], x[16 - i]))
    allr = {16: x[16]}
    verify(prog, 33, [list(range(9)), list(range(9, 18)), list(range(18, 27))],
           lambda v, o: o[allr[16]] == sorted(v)[16], exhaustive=False, trials=200000)
    verify_01_groups(prog, 33, [list(range(9)), list(range(9, 18)), list(range(18, 27))], 16, allr[16])
    stats["sphere33_final"] = ops(prog)
    parts.append(("net_sphere33_final_raw", 33, prog, [allr[16]], "sorted 9 x3 + 4 + 2 singles -> rank 16"))

    # sphere33 in z pairs: outputs z and z+1 share the blocks of planes z and
    # z+1.  Their merge drops rank 0 (below the median: 17 of the 18 are
    # larger, so at most 15 of the other 15 values can be smaller) and rank
    # 17 (above it), keeping ranks 1..16 ...
    net = []
    r = oe_merge(list(range(9)), list(range(9, 18)), net)
    prog = prune(net, r[1:17])
    verify(prog, 18, [list(range(9)), list(range(9, 18))],
           lambda v, o: [o[w] for w in r[1:17]] == sorted(v)[1:17], exhaustive=True)
    stats["merge99_r1_16"] = ops(prog)
    parts.append(("net_merge99_r1_16_raw", 18, prog, r[1:17], "sorted 9s w[0..8], w[9..17] -> ranks 1..16"))

    # ... and each output takes rank 15 of those 16 (w[0..15], sorted), the
    # sorted block of its other plane (w[16..24]), its four in-plane
    # singles (w[25..28]) and its two z singles (w[29], w[30]).  The 16 and
    # the 9 are merged for ranks 9..15 only, the six singles sorted, and
    # rank 15 of the union taken by the selection identity for two sorted
    # lists X (the 25) and S (the 6): C[k] = min over i of max(S[i-1],
    # X[k-i]), i = 0..6, S[-1] = -inf -- 84 operations against 104 for a
    # pruned merge of (16, (9, 6)).
    net = []
    ab = oe_merge(list(range(16)), list(range(16, 25)), net)
    prog = prune(net, [ab[15 - i] for i in range(7)])
    net = []
    s4 = oe_merge(oe_merge([25], [26], net), oe_merge([27], [28], net), net)
    s6 = oe_merge(s4, oe_merge([29], [30], net), net)
    prog += prune(net, s6)
    for i in range(1, 7):  # t_i = max(S[i-1], X[15-i]) in wire X[15-i]
        prog.append(("max", s6[i - 1], ab[15 - i]))
    for i in range(1, 7):  # C[15] = min(t_0 .. t_6) in wire X[15] (t_0 = X[15])
        prog.append(("min", ab[15], ab[15 - i]))
    allr = {15: ab[15]}
    verify(prog, 31, [list(range(16)), list(range(16, 25))],
           lambda v, o: o[allr[15]] == sorted(v)[15], exhaustive=False, trials=200000)
    verify_01_groups(prog, 31, [list(range(16)), list(range(16, 25))], 15, allr[15])
    stats["sphere33_pair_final"] = ops(prog)
    parts.append(("net_sphere33_pair_final_raw", 31, prog, [allr[15]],
                  "sorted 16 w[0..15] U sorted 9 w[16..24] U 6 singles -> rank 15"))

    # 2D: median of 9 from three sorted triples (median_box_2d 3x3)
    net = []
    r = oe_merge(oe_merge([0, 1, 2], [3, 4, 5], net), [6, 7, 8], net)
    prog = prune(net, [r[4]])
    verify(prog, 9, [[0, 1, 2], [3, 4, 5], [6, 7, 8]], lambda v, o: o[r[4]] == sorted(v)[4])
    stats["med9_2d"] = ops(prog)
    parts.append(("net_med9_raw", 9, prog, [r[4]], "three sorted triples -> rank 4"))

    body = ["// clk_median_networks.cuh - GENERATED by gen_median_networks.py; do not edit.",
            "// Pruned odd-even merge networks for the fast median kernels.  Each",
            "// function works in place on w[]; the comment under it lists the wires",
            "// that hold the consumed ranks afterwards.",
            "#pragma once",
            "#ifndef CLK_NET_FN",
            "#define CLK_NET_FN __device__ __forceinline__",
            "#endif",
            "#ifndef CLK_NET_CONST",
            "#define CLK_NET_CONST __device__ constexpr",
            "#endif", ""]
    for name, n, prog, outw, doc in parts:
        body.append(emit(name, n, prog, doc))
        body.append(f"CLK_NET_CONST int {name.replace('_raw', '')}_out[{len(outw)}] = {{{', '.join(map(str, outw))}}};")
        body.append("")
    OUT.write_text("\n".join(body))
    print(OUT, stats)


if __name__ == "__main__":
    main()
