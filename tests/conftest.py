import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (compute capability 10.3) GPU")
    config.addinivalue_line("markers", "slow: long-running")


def load_golden(name):
    """Rows of a golden TSV (tests/golden/make_golden.py): hap, read, qual, ins, del, gcp, expected."""
    import numpy as np

    rows = []
    with open(os.path.join(GOLDEN, name)) as f:
        for line in f:
            if line.startswith("#"):
                continue
            h, r, q, i, d, g, e = line.rstrip("\n").split("\t")
            conv = lambda s: np.array([int(x) for x in s.split(",")], dtype=np.uint8)
            rows.append((h.encode(), r.encode(), conv(q), conv(i), conv(d), conv(g), e))
    return rows


@pytest.fixture(scope="session")
def engine():
    """A GPU engine (GPU tests only)."""
    from gatk_gb300.pairhmm import Engine

    e = Engine()
    yield e
    e.close()
