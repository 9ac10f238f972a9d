"""Regenerate tests/golden/dragstr_cases.json from the reference's DRAGstr test resources.

Run in a checkout that has the reference mounted (it is not needed afterwards):

    python tests/golden/make_dragstr_golden.py /path/to/gatk

Inputs (paths inside the GATK repository):
  src/test/resources/org/broadinstitute/hellbender/tools/haplotypecaller/example.dragstr-params.txt
      the DRAGstr model the HaplotypeCaller integration tests run with (--dragstr-params-path,
      HaplotypeCallerIntegrationTest.java:296); its GOP and GCP tables, [period][repeat length], as DragstrParams
      reads them (one header row of repeat lengths, then a "GOP:", "GCP:" and "API:" block of one row per period)
  src/test/java/org/broadinstitute/hellbender/utils/pairhmm/DragstrReadSTRAnalyzerTest.java
      the empirical known-answer case of testCasesData (:58-66): a read and its most repeated period and repeat
      count per position, as hexadecimal digits

The generated tests/golden/dragstr_cases.json is what the tests read.  The two large generated case files the
analyzer test also reads are not part of the reference checkout (only their storage pointers are), so they are not
used.
"""
from __future__ import annotations

import json
import os
import re
import sys

PARAMS = "src/test/resources/org/broadinstitute/hellbender/tools/haplotypecaller/example.dragstr-params.txt"
STR_TEST = "src/test/java/org/broadinstitute/hellbender/utils/pairhmm/DragstrReadSTRAnalyzerTest.java"


def parse_params(text: str) -> dict:
    lines = [ln.strip() for ln in text.splitlines() if ln.strip()]
    repeats = [int(x) for x in lines[0].split()]
    blocks: dict[str, list[list[float]]] = {}
    name = None
    for ln in lines[1:]:
        if ln.endswith(":"):
            name = ln[:-1]
            blocks[name] = []
        else:
            blocks[name].append([float(x) for x in ln.split()])
    for k in ("GOP", "GCP", "API"):
        rows = blocks[k]
        assert rows and all(len(r) == len(repeats) for r in rows), k
    assert len(blocks["GOP"]) == len(blocks["GCP"])
    return {"max_period": len(blocks["GOP"]), "max_repeats": len(repeats), "gop": blocks["GOP"], "gcp": blocks["GCP"]}


def parse_empirical(text: str) -> dict:
    start = text.index("An empirical test case")
    lits = re.findall(r'"([^"]*)"', text[start:start + 4000])[:3]
    seq, periods, repeats = lits
    assert set(seq) <= set("ACGT") and len(periods.split()) == len(repeats.split())
    return {"read": seq, "periods": [int(x, 16) for x in periods.split()],
            "repeats": [int(x, 16) for x in repeats.split()]}


def main(root: str) -> None:
    with open(os.path.join(root, PARAMS)) as f:
        params = parse_params(f.read())
    with open(os.path.join(root, STR_TEST)) as f:
        emp = parse_empirical(f.read())
    out = {"source": {"params": PARAMS, "str_case": STR_TEST + ":58-66"}, "example_params": params,
           "str_empirical": emp}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dragstr_cases.json")
    with open(dst, "w") as f:
        json.dump(out, f)
        f.write("\n")
    print(f"wrote {dst}: tables {params['max_period']}x{params['max_repeats']}, read of {len(emp['read'])} bases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_dragstr_golden.py GATK_CHECKOUT  (the root of a broadinstitute/gatk source tree)")
    main(sys.argv[1])
