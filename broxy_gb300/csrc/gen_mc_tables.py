"""Generate ``mc_tables.inc`` — the marching-cubes triangulation table.

The per-case triangle lists must match the classic Lorensen/Bourke table that
the reference mesher carries (GMorpho/tables.h:321, ``triTable``), otherwise the
extracted mesh would have a different connectivity.  The table is read from the
reference header once, at development time, and re-encoded here in a compact
form of this project: one 64-bit word per cube case, edge indices packed as
4-bit nibbles (triangle ``t`` uses nibbles ``3t..3t+2``), the length of each
list, and the reference's slot-size count table.

The edge-intersection table (``edgeTable``, tables.h:25) is NOT stored: it is
derived from the cube corner order and checked by the tests.  The per-case
triangle counts are the reference's own ``numTriTable`` (tables.h:61), read
as-is: they size the triangle slots of every cube, and for case 91 the
reference count (4) is one less than the triangles its list holds (5).  The
mesher reproduces the consequence of that mismatch; see ``mc.cu``.

Usage (needs the reference checkout):
    python broxy_gb300/csrc/gen_mc_tables.py /path/to/reference/GMorpho/tables.h
"""
import os
import re
import sys


def parse_tri_table(path):
    src = open(path).read()
    m = re.search(r"triTable\[256 \*16\]\s*=\s*\{(.*?)\};", src, re.S)
    vals = [int(v) for v in re.findall(r"-?\d+", m.group(1))]
    assert len(vals) == 256 * 16
    cases = []
    for c in range(256):
        row = vals[16 * c:16 * c + 16]
        n = row.index(-1) if -1 in row else 16
        assert n % 3 == 0 and n <= 15
        cases.append(row[:n])
    return cases


def parse_tri_counts(path):
    src = open(path).read()
    m = re.search(r"numTriTable\[256\]\s*=\s*\{(.*?)\};", src, re.S)
    vals = [int(v) for v in re.findall(r"\d+", m.group(1))]
    assert len(vals) == 256
    return vals


def main():
    path = sys.argv[1]
    cases = parse_tri_table(path)
    counts = parse_tri_counts(path)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mc_tables.inc")
    with open(out, "w") as f:
        f.write("/* Generated by gen_mc_tables.py: marching-cubes triangle lists,\n"
                "   one 64-bit word per case (4-bit edge ids, 3 per triangle), and\n"
                "   the reference's per-case triangle count (slot size).\n"
                "   Do not edit by hand. */\n")
        f.write("#define GM_MC_TRI_PACKED_INIT { \\\n")
        for c in range(256):
            w = 0
            for i, e in enumerate(cases[c]):
                w |= (e & 0xF) << (4 * i)
            f.write("  0x%016xULL%s \\\n" % (w, "," if c < 255 else ""))
        f.write("}\n")
        f.write("#define GM_MC_TRI_COUNT_INIT { \\\n")
        for c in range(0, 256, 16):
            f.write("  " + ", ".join(str(counts[k]) for k in range(c, c + 16))
                    + ("," if c < 240 else "") + " \\\n")
        f.write("}\n")
        f.write("#define GM_MC_TRI_LEN_INIT { \\\n")
        for c in range(0, 256, 16):
            f.write("  " + ", ".join(str(len(cases[k]) // 3) for k in range(c, c + 16))
                    + ("," if c < 240 else "") + " \\\n")
        f.write("}\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
