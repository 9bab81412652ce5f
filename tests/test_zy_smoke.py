"""The round-trip that the entry point's smoke() runs on cuda:0: every timed
kernel (FP32 Hogwild, FP32 and BF16 staged) against the oracle's epoch by the
factor check, the FP64 deterministic epoch bit-exact."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_smoke_runs_against_the_oracle():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as entry

    entry.smoke()
