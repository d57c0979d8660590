"""Extract the knot-vector golden vectors from the reference's pFUnit tests.

Reads ``tests/test_knot.pf`` of the IGA-ADS reference as text and writes
``knot_vectors.json`` beside this script.  Each record is one assertion of the
reference test:

* ``test_knot1`` (tests/test_knot.pf:1-74): ``FillOpenKnot(n, p)`` must equal U.
* ``test_knot2`` (tests/test_knot.pf:78-132): ``CountSpans(n, p, U) == n-p+1``.
* ``test_knot3`` (tests/test_knot.pf:135-215): ``PrepareKnot(n, p)`` gives
  ``nelem == n-p+1`` and, where the assertion is enabled, the vector U.  The
  n = -1 case has its vector assertion commented out in the reference ("FIX
  THIS"), which is recorded as ``"check_vector": false``.

Usage: python tests/golden/make_knot_vectors.py <path to the reference's tests/test_knot.pf>
"""
import json
import os
import re
import sys


def parse(text):
    records = []
    test = None
    n = p = None
    U = None
    for raw in text.splitlines():
        line = raw.strip()
        m = re.match(r"subroutine\s+(test_knot\d+)", line)
        if m:
            test = m.group(1)
            continue
        m = re.match(r"n\s*=\s*(-?\d+)$", line)
        if m:
            n = int(m.group(1))
            U = None
            continue
        m = re.match(r"p\s*=\s*(-?\d+)$", line)
        if m:
            p = int(m.group(1))
            continue
        m = re.match(r"U\s*=\s*\(/(.*)/\)", line)
        if m:
            U = [float(v) for v in m.group(1).split(",")]
            if test == "test_knot3":
                # the vector assertion follows on the next non-comment line, or is disabled
                records.append({"test": test, "n": n, "p": p, "U": U, "check_vector": None})
            continue
        if line.startswith("@assertEqual"):
            if test == "test_knot1":
                records.append({"test": test, "n": n, "p": p, "U": U, "check": "fill"})
            elif test == "test_knot2":
                records.append({"test": test, "n": n, "p": p, "U": U, "check": "count"})
            elif test == "test_knot3":
                if "nelem" in line:
                    records.append({"test": test, "n": n, "p": p, "check": "prepare_nelem"})
                elif "(U, res)" in line.replace(" ", "").replace("(U,res)", "(U, res)"):
                    for r in reversed(records):
                        if r["test"] == "test_knot3" and r.get("check_vector") is None and "U" in r:
                            r["check_vector"] = True
                            r["check"] = "prepare_vector"
                            break
            continue
        if line.startswith("!@assertEqual") and test == "test_knot3":
            for r in reversed(records):
                if r["test"] == "test_knot3" and r.get("check_vector") is None and "U" in r:
                    r["check_vector"] = False
                    r["check"] = "prepare_vector_disabled"
                    break
    return records


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_knot_vectors.py <path to the reference's tests/test_knot.pf>")
    src = sys.argv[1]
    with open(src) as f:
        records = parse(f.read())
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "knot_vectors.json")
    with open(out, "w") as f:
        json.dump({"source": "tests/test_knot.pf", "records": records}, f, indent=1)
    print(f"wrote {len(records)} records to {out}")


if __name__ == "__main__":
    main()
