"""The oracle against its committed regression fixtures (tests/golden/oracle_regression.npz,
written by tests/golden/make_golden.py): a change to the oracle that alters the RGBA8 LUT, the
f64 DrainageSimulator run or the foam default cluster's steps fails here and needs a reason.
(These are not reference golden vectors; the reference ships none for this path.)

The oracle calls the C library's sin, cos, exp and pow, whose last bit differs between libm
versions and between x86_64 and aarch64, so only the integer arrays (connection lists) are
compared exactly. Float arrays are compared within a bound far below any change of the oracle's
arithmetic (1e-12 relative for f64, 1e-6 for f32) and the RGBA8 LUT, whose bytes truncate f32
values, may differ by one in at most 8 of its 65,536 bytes."""
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
        g, w = np.asarray(got[k]), want[k]
        assert g.shape == w.shape and g.dtype == w.dtype, k
        if w.dtype == np.uint8:
            d = np.abs(g.astype(int) - w.astype(int))
            assert d.max() <= 1 and np.count_nonzero(d) <= 8, k
        elif np.issubdtype(w.dtype, np.integer):
            np.testing.assert_array_equal(g, w, err_msg=k)
        else:
            rtol = 1e-12 if w.dtype == np.float64 else 1e-6
            scale = float(np.max(np.abs(w))) or 1.0
            assert float(np.max(np.abs(g.astype(np.float64) - w))) <= rtol * scale, k
