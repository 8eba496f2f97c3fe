"""The error measures the scale parity tests and the benchmark report (numpy only, no GPU)."""
import math

import numpy as np
import pytest


def test_rel_linf_and_masks():
    from soap_bubble_simulation_gb300 import parity

    ref = np.full((40, 16), 500e-9)
    got = ref.copy()
    got[20, 3] *= 1 + 1e-6
    assert abs(parity.rel_linf(got, ref) - 1e-6) < 1e-15
    ref2 = ref.copy()
    ref2[1] = 0.0  # a collapsed ring
    st = parity.stable_rows(ref2, ref)
    assert not st[1] and st[0] and st[2]
    sm = parity.stable_rows(ref2, ref, margin=3)
    assert not sm[:5].any() and sm[5:].all()
    assert parity.rel_linf(got, ref, np.zeros(40, bool)) == 0.0
    assert parity.rel_linf(np.full_like(ref, np.nan), ref) == float("inf")


def test_cfl_rows_at_2048():
    """D dt / R^2 (1/dtheta^2 + 1/(sin^2 dphi^2)) <= 1/2 fails on the first 24 rings of each pole
    at 2048 x 4096 with the reference defaults (D 1e-9, dt 1 ms, R 25 mm)."""
    from soap_bubble_simulation_gb300 import parity

    ok = parity.cfl_rows(2048, 4096)
    assert ok.sum() == 2048 - 2 * 25  # rings 1..24 and their pole rows, at each end
    assert not ok[:25].any() and ok[25] and not ok[-25:].any()
    theta = 25 * math.pi / 2047
    assert 1e-12 / 0.025 ** 2 * ((2047 / math.pi) ** 2 + (4096 / (2 * math.pi)) ** 2 / math.sin(theta) ** 2) <= 0.5
    assert parity.cfl_rows(128, 256).all()  # config 0 is stable everywhere


def test_report_keys():
    from soap_bubble_simulation_gb300 import parity

    a = np.ones((30, 8))
    r = parity.report(a, a, a)
    assert r["rel_linf"] == 0.0 and r["stable_rows"] == 30 and r["rows"] == 30
    assert set(r) >= {"rel_linf_cfl_rows", "rel_linf_stable_rows", "rel_linf_stable_rows_margin8", "rel_linf_sin_ge_0.2"}


def test_surrogate_training_kinds():
    """Config-1 fields and mirrored windows are periodic in phi without a jump at the seam (a film
    on a sphere has none); step windows keep the jump where their two ends meet."""
    from soap_bubble_simulation_gb300 import synthetic

    kinds = synthetic.SURROGATE_KINDS
    assert set(kinds) == {"c1", "mirror", "step"}
    for k, (h, c, visc, rad) in enumerate(synthetic.surrogate_trajectories(8)):
        seam = np.abs(h[:, 0].astype(np.float64) - h[:, -1]).max()
        inner = np.abs(np.diff(h.astype(np.float64), axis=1)).max()
        if kinds[k % len(kinds)] == "step":
            assert seam > 4 * inner, (k, seam, inner)
        else:
            assert seam <= inner + 1e-15, (k, seam, inner)
        assert h.shape == (256, 512) and 1e-4 <= visc <= 1e-2 and 0.0015 <= rad <= 0.04
    for h, *_ in synthetic.surrogate_trajectories(3, seed=5, kinds=("mirror",)):
        assert np.array_equal(h[:, :256], h[:, 256:][:, ::-1])
    with pytest.raises(ValueError):
        next(synthetic.surrogate_trajectories(1, kinds=("ring",)))
