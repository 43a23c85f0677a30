"""Generate ``case_tables.h``: the marching-cubes (MC) and dual-marching-cubes (DMC)
case tables in the packed layout the CUDA kernels read.

Conventions that have to match the reference bit for bit (they decide the
vertex/face/patch numbering of the output) are kept as they are there:

* MC corner order for the 8-bit case code (``src/cumc.cu:107``):
  (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1).
* DMC corner order for the case code is Morton order (``src/cudualmc.cu:95-104``):
  corner i sits at (i&1, (i>>1)&1, (i>>2)&1).
* Edge numbering (``src/cumc.cu:109-122`` == ``src/cudualmc.cu:106-119``): edge e starts
  at the cell-local point EDGE_START[e] and runs one step along EDGE_AXIS[e].

Table contents:

* MC triangulation (``src/cumc.cu:143-159``).  It is not a rule-derived table (its
  hexagons use zig-zag strips, not fans), so its triangles are read from the
  reference source when that is present and re-encoded; the committed header
  keeps the packed copy.  Each case is one 64-bit word: bits 0-3 = number of
  triangles (0..5), then 15 four-bit edge ids (three per triangle, in table order).
* DMC patches (``src/cudualmc.cu:121-242, 244-501``), derived here from geometry:
  a patch is a connected set of crossing edges, two crossing edges of one cube
  face being joined when they bound the same corner whose value is >= iso on an
  ambiguous face (the >= iso corners are cut off), or when they are the only two
  crossing edges of the face.  Patches are numbered by the smallest corner index of
  the minority sign they enclose (the >= iso corners when at most four are set,
  the < iso corners otherwise).  A case is "problematic" when it has exactly one
  ambiguous face and a single patch; its resolution direction is that face.
* DMC quad order (``src/cudualmc.cu:504-513``), derived: the four cells around a
  crossing edge along axis a, stepped over the two other axes (b, c) = (a+1, a+2)
  mod 3 in the cyclic order (0,0) (-1,0) (-1,-1) (0,-1) when the edge enters
  (value rises through iso from its start point), and reversed when it exits.

Run ``python gen_tables.py`` (optionally ``--reference DIR``; by default the checkout
named by the environment variable DISO_REFERENCE_SRC, if any) to rewrite the header,
``python gen_tables.py --check`` to compare the committed header with a fresh
derivation (the MC words are compared only when the reference source is present).
"""
from __future__ import annotations

import argparse
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "case_tables.h")
# a reference checkout, when one is on this machine (None otherwise)
DEFAULT_REFERENCE = os.environ.get("DISO_REFERENCE_SRC")

MC_CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
              (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
DMC_CORNERS = [(i & 1, (i >> 1) & 1, (i >> 2) & 1) for i in range(8)]
# edge e: (start point, axis)
EDGES = [((0, 0, 0), 0), ((1, 0, 0), 2), ((0, 0, 1), 0), ((0, 0, 0), 2),
         ((0, 1, 0), 0), ((1, 1, 0), 2), ((0, 1, 1), 0), ((0, 1, 0), 2),
         ((0, 0, 0), 1), ((1, 0, 0), 1), ((1, 0, 1), 1), ((0, 0, 1), 1)]


def edge_endpoints(corners):
    idx = {c: i for i, c in enumerate(corners)}
    out = []
    for start, axis in EDGES:
        end = list(start)
        end[axis] += 1
        out.append((idx[start], idx[tuple(end)]))
    return out


def edge_of(start, axis):
    return EDGES.index((tuple(start), axis))


# ----------------------------------------------------------------------------- DMC
def dmc_patches(code):
    """Patches (lists of edge ids, ascending) of a DMC case, in patch order."""
    ends = edge_endpoints(DMC_CORNERS)
    bit = lambda c: (code >> c) & 1
    crossing = [bit(a) != bit(b) for a, b in ends]
    parent = list(range(12))

    def find(x):
        while parent[x] != x:
            x = parent[x]
        return x

    for axis in range(3):
        for side in range(2):
            face = [c for c in range(8) if DMC_CORNERS[c][axis] == side]
            fe = [e for e, (a, b) in enumerate(ends) if crossing[e] and a in face and b in face]
            if len(fe) == 2:
                parent[find(fe[0])] = find(fe[1])
            elif len(fe) == 4:
                for c in face:
                    if bit(c):
                        inc = [e for e in fe if c in ends[e]]
                        parent[find(inc[0])] = find(inc[1])
    groups = {}
    for e in range(12):
        if crossing[e]:
            groups.setdefault(find(e), []).append(e)
    minority = 1 if bin(code).count("1") <= 4 else 0

    def key(p):
        return min(a if bit(a) == minority else b for a, b in (ends[e] for e in p))

    return sorted((sorted(g) for g in groups.values()), key=key)


def ambiguous_faces(code):
    bit = lambda c: (code >> c) & 1
    out = []
    for axis in range(3):
        for side in range(2):
            a, b, c, d = sorted(c for c in range(8) if DMC_CORNERS[c][axis] == side)
            # a,d and b,c are the diagonals of the face
            if bit(a) == bit(d) and bit(b) == bit(c) and bit(a) != bit(b):
                out.append(2 * axis + side)
    return out


def dmc_problem_dir(code):
    amb = ambiguous_faces(code)
    if len(amb) == 1 and len(dmc_patches(code)) == 1:
        return amb[0]
    return 7


def dmc_word(code):
    patches = dmc_patches(code)
    w = 0
    for p, edges in enumerate(patches):
        for e in edges:
            w |= p << (2 * e)
    w |= len(patches) << 24
    w |= dmc_problem_dir(code) << 28
    for p, edges in enumerate(patches):
        w |= len(edges) << (32 + 4 * p)
    return w


def dmc_quads():
    """For each edge type (axis + 3*exiting): four (db, dc) cell offsets + local edge id."""
    rows = []
    for exiting in (0, 1):
        for axis in range(3):
            b, c = (axis + 1) % 3, (axis + 2) % 3
            ring = [(0, 0), (-1, 0), (-1, -1), (0, -1)]
            if exiting:
                ring = [ring[0], ring[3], ring[2], ring[1]]
            row = []
            for ob, oc in ring:
                off = [0, 0, 0]
                off[b], off[c] = ob, oc
                start = [0, 0, 0]
                start[b], start[c] = -ob, -oc
                row.append((off, edge_of(start, axis)))
            rows.append(row)
    return rows


# ----------------------------------------------------------------------------- MC
def _c_array(src, name):
    m = re.search(r"__constant__\s+int\s+" + name + r"\s*\[[^\]]*\]\s*=\s*\{", src)
    if m is None:
        raise ValueError(f"table {name} not found")
    body = src[m.end():src.index("}", m.end())]
    return [int(v) for v in re.findall(r"-?\d+", body)]


def mc_words_from_reference(reference):
    src = open(os.path.join(reference, "src", "cumc.cu")).read()
    first = _c_array(src, "firstMarchingCubesId")
    ids = _c_array(src, "marchingCubesIds")
    words = []
    for code in range(256):
        tri_ids = ids[first[code]:first[code + 1]]
        assert len(tri_ids) % 3 == 0 and len(tri_ids) <= 15
        w = len(tri_ids) // 3
        for i, e in enumerate(tri_ids):
            w |= e << (4 + 4 * i)
        words.append(w)
    return words


def mc_words_from_header(path=HEADER):
    src = open(path).read()
    m = re.search(r"#define DISO_MC_TRIANGLES \{([^}]*)\}", src)
    return [int(v, 16) for v in re.findall(r"0x([0-9a-fA-F]+)", m.group(1))]


def dmc_words_from_header(path=HEADER):
    src = open(path).read()
    m = re.search(r"#define DISO_DMC_CASES \{([^}]*)\}", src)
    return [int(v, 16) for v in re.findall(r"0x([0-9a-fA-F]+)", m.group(1))]


def mc_check_structure(words):
    """Every triangle edge crosses, and every crossing edge of the case is used."""
    ends = edge_endpoints(MC_CORNERS)
    for code, w in enumerate(words):
        bit = lambda c: (code >> c) & 1
        n = w & 15
        used = {(w >> (4 + 4 * i)) & 15 for i in range(3 * n)}
        crossing = {e for e, (a, b) in enumerate(ends) if bit(a) != bit(b)}
        if used != crossing:
            raise AssertionError(f"MC case {code}: edges {sorted(used)} != crossings {sorted(crossing)}")


# ----------------------------------------------------------------------------- emit
def render(mc_words):
    lines = []
    p = lines.append
    p("// Generated by gen_tables.py -- do not edit.")
    p("// Marching-cubes and dual-marching-cubes case tables in packed form; the")
    p("// generator's docstring gives the encoding and where each table comes from.")
    p("#pragma once")
    p("#include <stdint.h>")
    p("")
    p("// edge e: start point (bit0 = dx, bit1 = dy, bit2 = dz) | axis << 3")
    enc = [s[0] | (s[1] << 1) | (s[2] << 2) | (a << 3) for s, a in EDGES]
    p("#define DISO_EDGE_TABLE {" + ", ".join(str(v) for v in enc) + "}")
    p("")
    p("// edge id of the cell-local edge starting at corner s (bit0 = dx, bit1 = dy, bit2 = dz)")
    p("// along axis a, at index 3 * s + a; 15 where no edge of the cell starts there")
    lut = [15] * 24
    for e, (st, a) in enumerate(EDGES):
        lut[3 * (st[0] | (st[1] << 1) | (st[2] << 2)) + a] = e
    p("#define DISO_EDGE_LOOKUP {" + ", ".join(str(v) for v in lut) + "}")
    p("")
    p("// MC: bits 0-3 triangle count, then 4-bit edge ids, three per triangle")
    p("#define DISO_MC_TRIANGLES {\\")
    for i in range(0, 256, 4):
        p("  " + ", ".join(f"0x{w:016x}ull" for w in mc_words[i:i + 4]) + ",\\")
    p("}")
    p("static const uint64_t kMcTriangles[256] = DISO_MC_TRIANGLES;")
    p("")
    p("// DMC: bits 2e..2e+1 patch of edge e; bits 24-26 patch count; bits 28-30 ambiguity")
    p("// direction (2*axis + (1 if +)) or 7; bits 32+4p..35+4p edge count of patch p")
    dmc = [dmc_word(c) for c in range(256)]
    p("#define DISO_DMC_CASES {\\")
    for i in range(0, 256, 4):
        p("  " + ", ".join(f"0x{w:016x}ull" for w in dmc[i:i + 4]) + ",\\")
    p("}")
    p("static const uint64_t kDmcCase[256] = DISO_DMC_CASES;")
    p("")
    p("// DMC quads: for edge type t = axis + 3*exiting, four entries, each")
    p("// (dx+1) | (dy+1) << 2 | (dz+1) << 4 | local edge << 8 of the neighbour cell")
    q = []
    for row in dmc_quads():
        for off, e in row:
            q.append((off[0] + 1) | ((off[1] + 1) << 2) | ((off[2] + 1) << 4) | (e << 8))
    p("#define DISO_DMC_QUADS {" + ", ".join(str(v) for v in q) + "}")
    p("")
    return "\n".join(lines)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    ap.add_argument("--check", action="store_true")
    args = ap.parse_args(argv)
    have_ref = bool(args.reference) and os.path.exists(os.path.join(args.reference, "src", "cumc.cu"))
    if have_ref:
        mc = mc_words_from_reference(args.reference)
    else:
        mc = mc_words_from_header()
    mc_check_structure(mc)
    text = render(mc)
    if args.check:
        cur = open(HEADER).read()
        if cur != text:
            print("case_tables.h differs from a fresh derivation", file=sys.stderr)
            return 1
        print("case_tables.h up to date" + ("" if have_ref else " (MC words not re-read)"))
        return 0
    open(HEADER, "w").write(text)
    print("wrote", HEADER)
    return 0


if __name__ == "__main__":
    sys.exit(main())
