"""Case tables: the packed header equals a fresh derivation, the DMC tables
derived by rule equal the reference's own tables, and the MC table keeps the
marching-cubes invariants."""
import os
import re
import sys

import pytest

from helpers import ROOT

sys.path.insert(0, os.path.join(ROOT, "diso_gb300", "csrc"))
import gen_tables as G  # noqa: E402

REF = G.DEFAULT_REFERENCE  # a reference checkout named by DISO_REFERENCE_SRC, or None
HAVE_REF = bool(REF) and os.path.exists(os.path.join(REF, "src", "cudualmc.cu"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)
import hash_tables as H  # noqa: E402


def _arr(src, name):
    m = re.search(name + r"\s*(\[[^\]]*\])+\s*=\s*\{", src)
    i, depth, j = m.end() - 1, 0, m.end() - 1
    while True:
        depth += {"{": 1, "}": -1}.get(src[j], 0)
        if depth == 0:
            break
        j += 1
    body = re.sub(r"//[^\n]*", "", src[i:j + 1])
    return [int(v) for v in re.findall(r"-?\d+", body)]


def test_header_up_to_date():
    assert G.main(["--check"]) == 0


def test_mc_table_structure():
    G.mc_check_structure(G.mc_words_from_header())


def test_dmc_patch_invariants():
    ends = G.edge_endpoints(G.DMC_CORNERS)
    for code in range(256):
        pats = G.dmc_patches(code)
        crossing = {e for e, (a, b) in enumerate(ends) if ((code >> a) & 1) != ((code >> b) & 1)}
        assert sorted(e for p in pats for e in p) == sorted(crossing)
        # complementing a code keeps the crossings; the number of patches of an
        # unambiguous case does not depend on the sign convention
        if not G.ambiguous_faces(code):
            assert len(G.dmc_patches(code ^ 0xFF)) == len(pats)
    assert sum(G.dmc_problem_dir(c) != 7 for c in range(256)) == 36


@pytest.mark.skipif(not HAVE_REF, reason="reference source not present")
def test_mc_table_matches_reference():
    src = open(os.path.join(REF, "src", "cumc.cu")).read()
    first, ids = _arr(src, "firstMarchingCubesId"), _arr(src, "marchingCubesIds")
    words = G.mc_words_from_header()
    for code in range(256):
        w = words[code]
        got = [(w >> (4 + 4 * i)) & 15 for i in range(3 * (w & 15))]
        assert got == ids[first[code]:first[code + 1]], code
    locs = _arr(src, r"int mcEdgeLocations")
    for e, (start, axis) in enumerate(G.EDGES):
        assert list(start) + [axis] == locs[4 * e:4 * e + 4]


@pytest.mark.skipif(not HAVE_REF, reason="reference source not present")
def test_dmc_tables_match_reference():
    src = open(os.path.join(REF, "src", "cudualmc.cu")).read()
    fp, fe, ei = _arr(src, "mcFirstPatchIndex"), _arr(src, "mcFirstEdgeIndex"), _arr(src, "mcEdgeIndex")
    prob, off, quad = _arr(src, "problematicConfigs"), _arr(src, "dmcEdgeOffset"), _arr(src, "dmcQuad")
    for code in range(256):
        pats = G.dmc_patches(code)
        ref = [ei[fe[p]:fe[p + 1]] for p in range(fp[code], fp[code + 1])]
        assert pats == ref, code
        d = G.dmc_problem_dir(code)
        assert (255 if d == 7 else d) == prob[code]
        for e in range(12):
            want = next((k for k, p in enumerate(pats) if e in p), -1)
            assert off[12 * code + e] == want
    flat = [v for row in G.dmc_quads() for off3, e in row for v in list(off3) + [e]]
    assert flat == quad


def reference_layout():
    """The reference's case tables (src/cumc.cu:107-175, src/cudualmc.cu:95-513) in
    its own array layout, rebuilt from the tables of this package: the MC words of
    the committed header, the DMC tables derived by rule."""
    words = G.mc_words_from_header()
    first, ids = [0], []
    for w in words:
        tri = [(w >> (4 + 4 * i)) & 15 for i in range(3 * (w & 15))]
        ids += tri
        first.append(len(ids))
    locs = [v for start, axis in G.EDGES for v in list(start) + [axis]]
    fp, fe, ei, prob, off = [0], [0], [], [], []
    for code in range(256):
        pats = G.dmc_patches(code)
        for p in pats:
            ei += list(p)
            fe.append(len(ei))
        fp.append(fp[-1] + len(pats))
        d = G.dmc_problem_dir(code)
        prob.append(255 if d == 7 else d)
        off += [next((k for k, p in enumerate(pats) if e in p), -1) for e in range(12)]
    quad = [v for row in G.dmc_quads() for off3, e in row for v in list(off3) + [e]]
    return {"firstMarchingCubesId": first, "marchingCubesIds": ids, "mcEdgeLocations": locs,
            "mcFirstPatchIndex": fp, "mcFirstEdgeIndex": fe, "mcEdgeIndex": ei, "problematicConfigs": prob,
            "dmcEdgeOffset": off, "dmcQuad": quad}


def test_tables_match_reference_digests():
    """Every case table, rebuilt in the reference's layout, has the length and the
    SHA-256 of the reference's own (tests/golden/reference_tables.json, written from
    a reference checkout by tests/golden/hash_tables.py): the tables are pinned to
    the reference without a checkout on this machine."""
    import json

    want = json.load(open(os.path.join(GOLDEN, "reference_tables.json")))
    got = reference_layout()
    assert set(got) == set(want)
    for name, vals in got.items():
        assert len(vals) == want[name]["length"], name
        assert H.digest(vals) == want[name]["sha256"], name


def test_digest_detects_a_changed_entry():
    vals = reference_layout()["dmcQuad"]
    vals[7] ^= 1
    want = __import__("json").load(open(os.path.join(GOLDEN, "reference_tables.json")))
    assert H.digest(vals) != want["dmcQuad"]["sha256"]
