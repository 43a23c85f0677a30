"""Write tests/golden/reference_tables.json: a SHA-256 digest of each case table
of a reference checkout, so that the tables derived here can be checked against
the reference's without a checkout on the machine (and without copying them).

    python tests/golden/hash_tables.py --ref-src <reference checkout>

Each digest is taken over the table's integers as parsed from the C source
(initialiser order, comments removed), written as JSON (a list of ints, no
spaces).  The tables: firstMarchingCubesId, marchingCubesIds and mcEdgeLocations
of src/cumc.cu; mcFirstPatchIndex, mcFirstEdgeIndex, mcEdgeIndex,
problematicConfigs, dmcEdgeOffset and dmcQuad of src/cudualmc.cu.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_tables.json")
TABLES = {"src/cumc.cu": ["firstMarchingCubesId", "marchingCubesIds", r"int mcEdgeLocations"],
          "src/cudualmc.cu": ["mcFirstPatchIndex", "mcFirstEdgeIndex", "mcEdgeIndex", "problematicConfigs",
                              "dmcEdgeOffset", "dmcQuad"]}


def c_array(src, name):
    """Integers of the initialiser of C array `name` (a regex) in `src`."""
    m = re.search(name + r"\s*(\[[^\]]*\])+\s*=\s*\{", src)
    if m is None:
        raise ValueError(f"table {name} not found")
    i = j = m.end() - 1
    depth = 0
    while True:
        depth += {"{": 1, "}": -1}.get(src[j], 0)
        if depth == 0:
            break
        j += 1
    body = re.sub(r"//[^\n]*", "", src[i:j + 1])
    return [int(v) for v in re.findall(r"-?\d+", body)]


def digest(values):
    return hashlib.sha256(json.dumps([int(v) for v in values], separators=(",", ":")).encode()).hexdigest()


def key(name):
    return name.split()[-1]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=os.environ.get("DISO_REFERENCE_SRC"), required="DISO_REFERENCE_SRC" not in os.environ)
    args = ap.parse_args()
    out = {}
    for path, names in TABLES.items():
        src = open(os.path.join(args.ref_src, path)).read()
        for name in names:
            vals = c_array(src, name)
            out[key(name)] = {"length": len(vals), "sha256": digest(vals)}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
