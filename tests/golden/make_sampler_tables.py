"""Generates tests/golden/sampler_tables.json from the reference's sampler
tables (modules/cpu/math/halton.inl, modules/cpu/math/sobol.inl).

Run in a checkout that has the reference source; the JSON it writes holds a
SHA-256 digest of each table (as little-endian uint32) plus its first 16
values, which is what the tests compare the oracle's regenerated tables
against.  The reference itself is not needed to run the tests.

    python tests/golden/make_sampler_tables.py /path/to/ospray
"""
import hashlib
import json
import os
import re
import sys

import numpy as np


def parse(path, name):
    text = open(path).read()
    m = re.search(r"%s\s*\[[^\]]*\]\s*=\s*\{(.*?)\};" % re.escape(name), text, re.S)
    vals = [int(v.rstrip("uU"), 0) for v in re.findall(r"0x[0-9a-fA-F]+u?|\d+u?", m.group(1))]
    return np.array(vals, dtype=np.uint32)


def main(ref):
    math = os.path.join(ref, "modules", "cpu", "math")
    out = {}
    for fname, names in (("halton.inl", ["halton_perm3", "halton_perm5", "halton_perm7"]),
                         ("sobol.inl", ["Sobol_revMatrices"])):
        for n in names:
            a = parse(os.path.join(math, fname), n)
            out[n] = {"count": int(a.size), "sha256": hashlib.sha256(a.astype("<u4").tobytes()).hexdigest(),
                      "head": [int(x) for x in a[:16]]}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sampler_tables.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["OSPRAY_REFERENCE_DIR"])
