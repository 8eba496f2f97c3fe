"""GPU parity of the spectral contraction (tensor cores, tcgen05) against the FP64 oracle.

Bars: the FP32 path within 1e-4 relative L-inf of the oracle (near grazing incidence the finesse F
reaches ~4e6 and the reflectance becomes a very steep function of phase, so f32 phase rounding
shows at the 1e-5 level); the BF16 tensor-core path within
1e-2 relative L-inf (BF16 keeps 8 significant bits of each reflectance and weight) and a mean
CIE76 colour difference below 0.5 (just noticeable is about 1-2.3).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def workload(n, seed=3, nl=81):
    from soap_bubble_simulation_gb300 import synthetic as S

    t, c, nf = S.spectral_points(n, seed=seed)
    if n >= 4:  # edges: thinnest, thickest, zero thickness; grazing and normal incidence
        t[:4] = [10.0, 1500.0, 777.7, 0.0]
        c[:4] = [0.0, 1.0, 1e-6, 0.5]
    wl = np.linspace(380.0, 780.0, nl) if nl != 81 else S.WAVELENGTHS_81
    return t, c, nf, wl, S.spectral_cmf(wl)


def rel_linf(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("nl", [81, 7, 50, 128])
def test_spectral_fp32_matches_oracle(sbs, orc, nl):
    t, c, nf, wl, cmf = workload(20000 + 77, nl=nl)
    got = sbs.spectral_rgb(t, c, nf, wl, cmf, mode="fp32")
    want = orc.spectral_rgb(t, c, nf, wl, cmf)
    assert rel_linf(got, want) <= 1e-4


@pytest.mark.parametrize("nl", [81, 7, 50, 128])
def test_spectral_tensor_cores_match_oracle(sbs, orc, nl):
    from soap_bubble_simulation_gb300 import synthetic as S

    t, c, nf, wl, cmf = workload(65536 + 77, seed=5, nl=nl)
    tc = sbs.spectral_rgb(t, c, nf, wl, cmf, mode="tc")
    fp = sbs.spectral_rgb(t, c, nf, wl, cmf, mode="fp32")
    want = orc.spectral_rgb(t, c, nf, wl, cmf)
    assert rel_linf(fp, want) <= 1e-4
    err = rel_linf(tc, want)
    assert err <= 1e-2, err
    de = S.delta_e76(tc, want, cmf.sum(axis=0))
    assert float(np.mean(de)) < 0.5, float(np.mean(de))


def test_spectral_small_and_ragged(sbs, orc):
    for n in (1, 5, 127, 129, 300):
        t, c, nf, wl, cmf = workload(n, seed=n)
        tc = sbs.spectral_rgb(t, c, nf, wl, cmf, mode="tc")
        want = orc.spectral_rgb(t, c, nf, wl, cmf)
        assert rel_linf(tc, want) <= 1e-2


def test_spectral_rejects_bad_arguments(sbs):
    t, c, nf, wl, cmf = workload(10)
    with pytest.raises(ValueError):
        sbs.spectral_rgb(t, c, nf, wl, cmf[:-1])
    wl129 = np.linspace(380, 780, 129)
    from soap_bubble_simulation_gb300 import synthetic as S

    with pytest.raises(sbs.SbsError, match="nl"):
        sbs.spectral_rgb(t, c, nf, wl129, S.spectral_cmf(wl129))


def test_spectral_very_thick_films(sbs, orc):
    """Points whose phase opd / lambda reaches 2^22 (films thicker than ~0.5 m) next to ordinary
    ones: the thin points keep their accuracy, and the thick ones give finite reflectances in
    [0, 1] weighted by the CMF (their f32 phase is coarser than a period, so no oracle comparison
    applies)."""
    t, c, nf, wl, cmf = workload(4096, seed=9)
    thick = np.arange(0, 4096, 7)
    t = t.copy()
    t[thick] = np.float32(2e9)
    thin = np.setdiff1d(np.arange(4096), thick)
    want = orc.spectral_rgb(t[thin], c[thin], nf[thin], wl, cmf)
    cap = cmf.clip(min=0).sum(axis=0)
    for mode, tol in (("fp32", 1e-4), ("tc", 1e-2)):
        got = sbs.spectral_rgb(t, c, nf, wl, cmf, mode=mode)
        assert rel_linf(got[thin], want) <= tol, mode
        g = got[thick]
        assert np.isfinite(g).all() and (g >= -1e-3).all() and (g <= cap * 1.01 + 1e-3).all(), mode
