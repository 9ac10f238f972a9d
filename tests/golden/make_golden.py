"""Regenerate the golden PairHMM fixtures in this folder from the reference's own test resources.

Run in a checkout that has the reference mounted (it is not needed afterwards):

    python tests/golden/make_golden.py /path/to/gatk

Inputs (paths inside the GATK repository):
  src/test/resources/org/broadinstitute/hellbender/tools/haplotypecaller/expected.Java.hmmresults.txt
      written by PairHMM.writeToResultsFileIfApplicable (PairHMM.java:376-385) during
      HaplotypeCallerIntegrationTest.testPairHMMResultsFile (LOGLESS_CACHING):
      hap read qual+33 ins+33 del+33 gcp+33 %e(log10 L), one pair per line.
  .../expected.AVX.hmmresults.txt  the same pairs through GKL's AVX FP32 kernel.
  src/test/resources/pairhmm-testdata.txt
      input of VectorPairHMMUnitTest (quals +33; base quals floored at 6, VectorPairHMMUnitTest.java:65,108-118).

Output: one TSV per input with columns hap, read, qual, ins, del, gcp (Phred values as
comma-separated integers, already decoded and, for the vector test data, floored exactly as
the reference test does) and the expected log10 likelihood as printed by the reference.
"""
from __future__ import annotations

import os
import sys

HC_DIR = "src/test/resources/org/broadinstitute/hellbender/tools/haplotypecaller"
SOURCES = {
    "hc_java_hmmresults.tsv": (f"{HC_DIR}/expected.Java.hmmresults.txt", 0),
    "hc_avx_hmmresults.tsv": (f"{HC_DIR}/expected.AVX.hmmresults.txt", 0),
    "vector_pairhmm_testdata.tsv": ("src/test/resources/pairhmm-testdata.txt", 6),
}


def decode(qs: str, floor: int) -> str:
    return ",".join(str(max(ord(ch) - 33, floor)) for ch in qs)


def convert(src: str, dst: str, base_qual_floor: int) -> int:
    n = 0
    with open(src) as fin, open(dst, "w") as fout:
        fout.write("#hap\tread\tqual\tins\tdel\tgcp\texpected_log10\n")
        for line in fin:
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            hap, read, q, ins, dele, gcp, exp = line.split()
            fout.write("\t".join([hap, read, decode(q, base_qual_floor), decode(ins, 0), decode(dele, 0),
                                  decode(gcp, 0), exp]) + "\n")
            n += 1
    return n


def main(argv):
    root = argv[1] if len(argv) > 1 else os.environ.get("GATK_REFERENCE", "")
    if not root:
        raise SystemExit("usage: make_golden.py <gatk checkout>")
    here = os.path.dirname(os.path.abspath(__file__))
    for dst, (src, floor) in SOURCES.items():
        n = convert(os.path.join(root, src), os.path.join(here, dst), floor)
        print(f"{dst}: {n} pairs")


if __name__ == "__main__":
    main(sys.argv)
