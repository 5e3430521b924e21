#!/usr/bin/env python3
"""Extract the CKD continuum coefficient tables into ``continua.bin``.

The CO2, H2O, N2 and O2 continuum parameterisations of the reference
(``ctmco2``/``ctmh2o``/``ctmn2``/``ctmo2``, src/jurassic.c:886-2917) are
driven by published spectroscopic coefficient tables (CKD continuum data).
Results can only match the reference when these numbers are identical, so
they are taken verbatim as DATA: this script parses the numeric initialisers
out of the reference source and writes them as little-endian float64 arrays.
No code is taken; the library and the oracle evaluate the parameterisations
with their own implementations.

Output layout of continua.bin (all float64, in this order):
  co2296[2001] co2260[2001] co2230[2001]          (ctmco2, jurassic.c:892,1167,1444)
  h2o296[2001] h2o260[2001] h2ofrn[2001]          (ctmh2o, jurassic.c:1753,2087,2421)
  xfcrev[15]                                       (ctmh2o, jurassic.c:2756)
  n2_b[98] n2_beta[98] n2_nu[98]                   (ctmn2,  jurassic.c:2801-2829)
  o2_b[90] o2_beta[90] o2_nu[90]                   (ctmo2,  jurassic.c:2866-2890)

usage: python make_continua.py [/path/to/reference]
"""
import hashlib
import os
import re
import sys

import numpy as np

ORDER = [
    ("ctmco2", "co2296", 2001), ("ctmco2", "co2260", 2001), ("ctmco2", "co2230", 2001),
    ("ctmh2o", "h2o296", 2001), ("ctmh2o", "h2o260", 2001), ("ctmh2o", "h2ofrn", 2001),
    ("ctmh2o", "xfcrev", 15),
    ("ctmn2", "ba", 98), ("ctmn2", "betaa", 98), ("ctmn2", "nua", 98),
    ("ctmo2", "ba", 90), ("ctmo2", "betaa", 90), ("ctmo2", "nua", 90),
]


def _function_body(src, name):
    m = re.search(r"\ndouble\s+%s\s*\(" % name, src)
    if not m:
        raise SystemExit("function %s not found" % name)
    start = src.index("{", m.end())
    depth = 0
    for i in range(start, len(src)):
        if src[i] == "{":
            depth += 1
        elif src[i] == "}":
            depth -= 1
            if depth == 0:
                return src[start:i]
    raise SystemExit("unterminated function %s" % name)


def _array(body, name, n):
    m = re.search(r"static\s+double\s+%s\s*\[\s*%d\s*\]\s*=\s*\{([^}]*)\}" % (name, n), body)
    if not m:
        raise SystemExit("array %s[%d] not found" % (name, n))
    vals = [float(t) for t in m.group(1).replace("\n", " ").split(",") if t.strip()]
    if len(vals) != n:
        raise SystemExit("array %s: %d values, expected %d" % (name, len(vals), n))
    return np.asarray(vals, dtype="<f8")


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("JURASSIC_REF_DIR")
    if not ref:
        raise SystemExit("usage: make_continua.py <reference tree> (or set JURASSIC_REF_DIR)")
    src = open(os.path.join(ref, "src", "jurassic.c")).read()
    parts = [_array(_function_body(src, fn), arr, n) for fn, arr, n in ORDER]
    blob = np.concatenate(parts).tobytes()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "continua.bin")
    with open(out, "wb") as f:
        f.write(blob)
    print("wrote %s (%d bytes, sha256 %s)" % (out, len(blob), hashlib.sha256(blob).hexdigest()))


if __name__ == "__main__":
    main()
