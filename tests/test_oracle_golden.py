"""The oracle against its committed regression fixtures (tests/golden/oracle_regression.npz,
written by tests/golden/make_golden.py): a change to the oracle that alters the RGBA8 LUT, the
f64 DrainageSimulator run or the foam default cluster's steps fails here and needs a reason.
(These are not reference golden vectors; the reference ships none for this path.)"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_matches_its_regression_fixtures(orc):
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden

    want = np.load(os.path.join(HERE, "golden", "oracle_regression.npz"))
    got = make_golden.cases()
    assert sorted(got) == sorted(want.files)
    for k in want.files:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
