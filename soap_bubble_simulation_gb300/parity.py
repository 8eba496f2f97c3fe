"""Error measures for comparing two thickness fields of the same grid (numpy only).

The relative L-inf error is max |a - b| / max |b| over the compared cells, b being the
reference run. At resolution 2048 the explicit scheme with the reference's dt (1 ms) is
unstable in phi next to the poles (the phi diffusion number D dt / (R sin(theta) dphi)^2 is far
above 1/2 on the first rings), so the polar rows of any run blow up and collapse to zero or to
the critical-thickness freeze, and two runs that differ in the last bit diverge there. On those
rows even a single step amplifies the f32 rounding of the Laplacian by the diffusion number
(~290 on ring 1 at 2048), so two correct f32 operation orders differ by ~1e-5 after one step.
Besides the unmasked figure, three masks are reported:

* CFL-stable rows: rows where the explicit step is stable, D dt / R^2 (1/dtheta^2 +
  1/(sin(theta)^2 dphi^2)) <= 1/2 (the pole rows count with their rings);
* stable rows: rows on which the reference run stayed finite and positive and inside twice the
  initial field's range (the rows the instability has not reached), reported also with a margin
  of 8 rows: the rows next to a collapsed one see its values through the theta stencil;
* sin(theta) >= 0.2: the fixed latitude band the learned surrogate's checks use (87 % of rows).
"""
from __future__ import annotations

import math

import numpy as np


def rel_linf(a, b, rows=None) -> float:
    """max |a - b| / max |b| over the rows selected by the boolean mask `rows` (all if None)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if rows is not None:
        a, b = a[rows], b[rows]
    if a.size == 0:
        return 0.0
    den = float(np.max(np.abs(b)))
    num = float(np.max(np.abs(a - b)))
    if not math.isfinite(num) or not math.isfinite(den) or den == 0.0:
        return float("inf")
    return num / den


def stable_rows(ref, initial, margin: int = 0) -> np.ndarray:
    """Rows of the reference field `ref` that are finite, positive and within twice the range of
    the initial field on every cell and, with margin > 0, have no row failing that within `margin`
    rows."""
    ref = np.asarray(ref, dtype=np.float64)
    init = np.asarray(initial, dtype=np.float64)
    lo, hi = 0.5 * float(np.min(init)), 2.0 * float(np.max(init))
    ok = (np.isfinite(ref) & (ref > 0.0) & (ref >= lo) & (ref <= hi)).all(axis=1)
    bad = ~ok
    grown = bad.copy()
    for s in range(1, margin + 1):
        grown[s:] |= bad[:-s]
        grown[:-s] |= bad[s:]
    return ~grown


def sin_rows(nt: int, min_sin: float = 0.2) -> np.ndarray:
    theta = np.arange(nt) * (math.pi / (nt - 1))
    return np.sin(theta) >= min_sin


def cfl_rows(nt: int, np_: int, diffusion: float = 1e-9, dt: float = 1e-3, radius: float = 0.025,
             sin_floor: float = 1e-10) -> np.ndarray:
    """Rows where one explicit step of the surface Laplacian is stable (see the module text)."""
    dth, dph = math.pi / (nt - 1), 2.0 * math.pi / np_
    s = np.abs(np.sin(np.arange(nt) * dth))
    s = np.maximum(s, sin_floor)
    num = diffusion * dt / radius ** 2 * (1.0 / dth ** 2 + 1.0 / (s * s * dph * dph))
    ok = num <= 0.5
    ok[0], ok[-1] = ok[1], ok[-2]
    return ok


def report(got, ref, initial, cfl=None) -> dict:
    """Unmasked and masked relative L-inf of `got` against `ref`, with the row counts. `cfl`:
    keyword arguments of cfl_rows (diffusion, dt, radius, sin_floor) for the CFL-stable mask."""
    nt, np_ = np.asarray(ref).shape
    st = stable_rows(ref, initial)
    sm = stable_rows(ref, initial, margin=8)
    sn = sin_rows(nt)
    cf = cfl_rows(nt, np_, **(cfl or {}))
    return {
        "rel_linf": rel_linf(got, ref),
        "rel_linf_cfl_rows": rel_linf(got, ref, cf),
        "rel_linf_stable_rows": rel_linf(got, ref, st),
        "rel_linf_stable_rows_margin8": rel_linf(got, ref, sm),
        "rel_linf_sin_ge_0.2": rel_linf(got, ref, sn),
        "cfl_rows": int(cf.sum()),
        "stable_rows": int(st.sum()),
        "rows": int(nt),
    }
