"""Regenerate tests/golden/sw_unit_cases.json from the reference's Smith-Waterman unit tests.

Run in a checkout that has the reference mounted (it is not needed afterwards):

    python tests/golden/make_sw_golden.py /path/to/gatk

Input (path inside the GATK repository):
  src/test/java/org/broadinstitute/hellbender/utils/smithwaterman/SmithWatermanAlignerAbstractUnitTest.java
      the known-answer cases every SmithWatermanAligner implementation runs (Java, native wrapper, Intel):
      makeComplexReadAlignedToRef :140-150, makeOddNoAlignment :152-167, testIndelsAtStartAndEnd :169-177,
      testDegenerateAlignmentWithIndelsAtBothEnds :179-187, getSubstringMatchTests :238-255,
      getSubstringMatchLong :266-281, and the sequences of testForIdenticalAlignmentsWithDifferingFlankLengths
      :189-236 (a property test: padded and unpadded alignments have the same indel elements).
  Parameter sets: SmithWatermanAlignmentConstants.java:30 (ORIGINAL_DEFAULT), :38 (STANDARD_NGS),
  :52 (NEW_SW_PARAMETERS).

The script reads the test source as text and pulls out its string literals and numbers; it checks the count
of what it found, so a changed test file fails loudly instead of producing a partial fixture.
"""
from __future__ import annotations

import json
import os
import re
import sys

TEST = "src/test/java/org/broadinstitute/hellbender/utils/smithwaterman/SmithWatermanAlignerAbstractUnitTest.java"
CONSTANTS = "src/main/java/org/broadinstitute/hellbender/utils/smithwaterman/SmithWatermanAlignmentConstants.java"


def _block(src: str, start_marker: str, end_marker: str) -> str:
    a = src.index(start_marker)
    return src[a:src.index(end_marker, a)]


def _strings(text: str):
    return re.findall(r'"([^"]*)"', text)


def main(argv):
    root = argv[1] if len(argv) > 1 else os.environ.get("GATK_REFERENCE", "")
    if not root:
        raise SystemExit("usage: make_sw_golden.py <gatk checkout>")
    src = open(os.path.join(root, TEST)).read()
    consts = open(os.path.join(root, CONSTANTS)).read()
    params = {}
    for name, vals in re.findall(r"SWParameters (\w+) = new SWParameters\(([^)]*)\)", consts):
        params[name] = [int(v) for v in vals.split(",")]
    assert {"ORIGINAL_DEFAULT", "STANDARD_NGS", "NEW_SW_PARAMETERS"} <= set(params), params
    cases = []

    b = _block(src, "makeComplexReadAlignedToRef", "@Test")
    m = re.search(r'\{"(\w+)", "(\w+)", (\d+), "(\w+)"\}', b)
    cases.append(dict(name="ComplexReadAlignedToRef", ref=m[1], alt=m[2], params=params["ORIGINAL_DEFAULT"],
                      strategy="SOFTCLIP", offset=int(m[3]), cigar=m[4]))

    b = _block(src, "makeOddNoAlignment", "@Test")
    ref1, read1 = _strings(b)[:2]
    rows = re.findall(r"new SWParameters\(([-\d, ]+)\), (\d+),\s+\"(\w+)\"", b)
    assert len(rows) == 2, rows
    for vals, off, cig in rows:
        cases.append(dict(name="OddNoAlignment", ref=ref1, alt=read1, params=[int(v) for v in vals.split(",")],
                          strategy="SOFTCLIP", offset=int(off), cigar=cig))

    b = _block(src, "testIndelsAtStartAndEnd", "@Test")
    match = _strings(b)[0]
    flank_ref, flank_read = _strings(b)[1], _strings(b)[2]
    exp_cigar = _strings(b)[3]
    off = int(re.search(r"expectedStart = (\d+)", b)[1])
    cases.append(dict(name="IndelsAtStartAndEnd", ref=flank_ref + match, alt=match + flank_read,
                      params=params["ORIGINAL_DEFAULT"], strategy="SOFTCLIP", offset=off, cigar=exp_cigar))

    b = _block(src, "testDegenerateAlignmentWithIndelsAtBothEnds", "@Test")
    s = _strings(b)
    ref, alt, cig = s[1], s[2], s[3]
    off = int(re.search(r"expectedStart = (\d+)", b)[1])
    cases.append(dict(name="DegenerateAlignmentWithIndelsAtBothEnds", ref=ref, alt=alt,
                      params=params["STANDARD_NGS"], strategy="SOFTCLIP", offset=off, cigar=cig))

    b = _block(src, "getSubstringMatchTests", "protected void assertAlignmentMatchesExpected")
    rows = re.findall(r"\{(\d+), \"(\w+)\", SWOverhangStrategy\.(\w+)\}", b)
    section = re.search(r'matchingSection = "(\w+)"', b)[1]
    prefix = re.search(r'reference = "(\w+)" \+ matchingSection', b)[1]
    assert len(rows) == 4, rows
    for off, cig, strat in rows:
        cases.append(dict(name="SubstringMatch", ref=prefix + section, alt=section, params=params["ORIGINAL_DEFAULT"],
                          strategy=strat, offset=int(off), cigar=cig))

    b = _block(src, "getSubstringMatchLong", "assertAlignmentMatchesExpected(reference, read, expectedStart, "
                                             "expectedCigar, ORIGINAL_DEFAULT, strategy);\n    }\n}")
    rows = re.findall(r"\{(\d+), \"(\w+)\", SWOverhangStrategy\.(\w+)\}", b)
    ref = re.search(r'reference = "(\w+)";', b)[1]
    read = re.search(r'read\s+= "(\w+)";', b)[1]
    assert len(rows) == 4, rows
    for off, cig, strat in rows:
        cases.append(dict(name="SubstringMatchLong", ref=ref, alt=read, params=params["ORIGINAL_DEFAULT"],
                          strategy=strat, offset=int(off), cigar=cig))

    b = _block(src, "testForIdenticalAlignmentsWithDifferingFlankLengths", "@DataProvider")
    seqs = {}
    for name in ("paddedRef", "paddedHap", "notPaddedRef", "notPaddedHap"):
        seqs[name] = re.search(name + r' = "([ACGT-]+)"', b)[1].replace("-", "")
    pad = re.search(r'SW_PAD = "(\w+)"', b)[1]
    flank = dict(pad=pad, params=params["NEW_SW_PARAMETERS"], strategy="SOFTCLIP", **seqs)

    out = dict(source=TEST, cases=cases, flank_test=flank)
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "sw_unit_cases.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(f"sw_unit_cases.json: {len(cases)} known-answer cases + the flank-length property test")


if __name__ == "__main__":
    main(sys.argv)
