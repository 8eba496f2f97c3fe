"""Seeded synthetic inputs for the benchmark workloads (no datasets exist for this path).

All generators use numpy's PCG64 with fixed seeds, so every run and every
machine builds the same inputs:

* bubble_c0: one bubble, resolution 128 (128 x 256), h = 500 nm (1 + 0.05 U[-1,1]), seed 0.
* bubble_c1: resolution 2048 (2048 x 4096), h = 550 nm + 16 smooth modes
  a_k cos(m_k theta + psi_k) cos(n_k phi + chi_k), a_k ~ N(0, 60 nm), m_k in 1..8,
  n_k in 0..8, clamped to [100, 1000] nm; surfactant 0.5 + U[-0.1, 0.1].
* icosphere(5): the 10242 unit vertices of a subdivision-5 icosphere.
"""
from __future__ import annotations

import math

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def bubble_c0(resolution: int = 128, seed: int = 0, h0: float = 500e-9, noise: float = 0.05) -> np.ndarray:
    """Initial thickness [theta][phi] (metres, f64)."""
    g = rng(seed)
    nt, np_ = resolution, 2 * resolution
    return h0 * (1.0 + noise * g.uniform(-1.0, 1.0, size=(nt, np_)))


def smooth_modes(nt: int, np_: int, seed: int = 1, modes: int = 16, base: float = 550e-9, amp: float = 60e-9,
                 lo: float = 100e-9, hi: float = 1000e-9) -> np.ndarray:
    """Sum of separable cosine modes on the theta-phi grid (f64, metres)."""
    g = rng(seed)
    a = g.normal(0.0, amp, size=modes)
    m = g.integers(1, 9, size=modes)
    n = g.integers(0, 9, size=modes)
    psi = g.uniform(0.0, 2 * math.pi, size=modes)
    chi = g.uniform(0.0, 2 * math.pi, size=modes)
    theta = np.arange(nt) * (math.pi / (nt - 1))
    phi = np.arange(np_) * (2 * math.pi / np_)
    U = a[None, :] * np.cos(m[None, :] * theta[:, None] + psi[None, :])  # [nt, modes]
    V = np.cos(n[None, :] * phi[:, None] + chi[None, :])  # [np, modes]
    h = base + U @ V.T
    return np.clip(h, lo, hi)


def smooth_modes_window(full_nt: int, full_np: int, r0: int, c0: int, nt: int, np_: int, seed: int = 1,
                        **kw) -> np.ndarray:
    """Rows r0 .. r0+nt-1 and columns c0 .. c0+np_-1 (mod full_np) of smooth_modes(full_nt, full_np, seed)."""
    g = rng(seed)
    modes = kw.get("modes", 16)
    a = g.normal(0.0, kw.get("amp", 60e-9), size=modes)
    m = g.integers(1, 9, size=modes)
    n = g.integers(0, 9, size=modes)
    psi = g.uniform(0.0, 2 * math.pi, size=modes)
    chi = g.uniform(0.0, 2 * math.pi, size=modes)
    theta = (r0 + np.arange(nt)) * (math.pi / (full_nt - 1))
    phi = ((c0 + np.arange(np_)) % full_np) * (2 * math.pi / full_np)
    U = a[None, :] * np.cos(m[None, :] * theta[:, None] + psi[None, :])
    V = np.cos(n[None, :] * phi[:, None] + chi[None, :])
    h = kw.get("base", 550e-9) + U @ V.T
    return np.clip(h, kw.get("lo", 100e-9), kw.get("hi", 1000e-9))


SURROGATE_KINDS = ("c1", "step", "c1", "mirror")


def surrogate_trajectories(count: int = 512, seed: int = 21, resolution: int = 256, fine: int = 2048,
                           kinds: tuple[str, ...] = SURROGATE_KINDS):
    """Initial states of the surrogate's training trajectories on a resolution x 2 resolution grid.

    Trajectory k is of kind kinds[k % len(kinds)]:
    * "c1": a config-1 field at `resolution` (bubble_c1);
    * "mirror": a resolution x resolution window of a config-1 field at `fine`, followed by its
      mirror image in phi, so the film is continuous across the periodic phi seam; this shows the
      network the cell-scale content of a `fine` field - kinks where the clamp to [100, 1000] nm
      bites, nearly flat smooth modes;
    * "step": a resolution x 2 resolution window of a config-1 field at `fine`, whose two ends meet
      at the phi seam with a jump of up to a few hundred nm. No film on a sphere has such a step;
      it is the largest gradient in the data and teaches the network the response to a sharp
      feature. A network trained without it under-predicts the drainage at the clamp kinks of the
      2048 x 4096 field: in the 10,000-step checked rollout there 4-9 of 20 checks fail (largest
      check error 3e-3 - 1e-2), against none (largest 6e-5) with it. A 64-pass interval diffuses
      the step itself further than the network's 4-cell receptive field reaches, so held-out error
      is reported for step and continuous trajectories apart.
    Viscosity is log-uniform in [1e-4, 1e-2] Pa s and the diameter log-uniform in [3, 80] mm; the
    small end gives, at `resolution`, the per-cell diffusion numbers of 25-40 mm bubbles at `fine`.
    Yields (h f32, c f32, viscosity, radius)."""
    for kind in kinds:
        if kind not in ("c1", "mirror", "step"):
            raise ValueError(f"unknown trajectory kind {kind!r}")
    g = rng(seed)
    nt, np_ = resolution, 2 * resolution
    for k in range(count):
        kind = kinds[k % len(kinds)]
        visc = float(10 ** g.uniform(-4.0, -2.0))
        radius = float(0.5 * 10 ** g.uniform(math.log10(0.003), math.log10(0.08)))
        s = int(g.integers(0, 2**31 - 1))
        if kind == "c1":
            h = smooth_modes(nt, np_, seed=s).astype(np.float32)
        else:
            r0 = int(g.integers(0, fine - nt + 1))
            c0 = int(g.integers(0, 2 * fine))
            if kind == "mirror":
                w = smooth_modes_window(fine, 2 * fine, r0, c0, nt, np_ // 2, seed=s)
                h = np.concatenate([w, w[:, ::-1]], axis=1).astype(np.float32)
            else:
                h = smooth_modes_window(fine, 2 * fine, r0, c0, nt, np_, seed=s).astype(np.float32)
        c = surfactant_noise(nt, np_, seed=s + 1)
        yield h, c, visc, radius


def surfactant_noise(nt: int, np_: int, seed: int = 2, mean: float = 0.5, spread: float = 0.1) -> np.ndarray:
    g = rng(seed)
    return (mean + g.uniform(-spread, spread, size=(nt, np_))).astype(np.float32)


def bubble_c1(resolution: int = 2048, seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """(h f32 [nt][np] metres, surfactant f32 [nt][np])."""
    nt, np_ = resolution, 2 * resolution
    h = smooth_modes(nt, np_, seed=seed).astype(np.float32)
    c = surfactant_noise(nt, np_, seed=seed + 1)
    return h, c


def icosphere(subdivisions: int = 5) -> np.ndarray:
    """Unit vertices of an icosphere, [10 * 4^s + 2, 3] f64, deterministic order."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts, dtype=np.float64)


# --- spectral interference workload ---------------------------------------------------------
WAVELENGTHS_81 = np.arange(380.0, 781.0, 5.0)  # 380..780 nm, 5 nm step


def spectral_points(n: int = 8_388_608, seed: int = 3):
    """Surface points: thickness U[10, 1500] nm, cos(theta) U[0, 1], film index U[1.30, 1.40] (f32)."""
    g = rng(seed)
    t = g.uniform(10.0, 1500.0, n).astype(np.float32)
    c = g.uniform(0.0, 1.0, n).astype(np.float32)
    nf = g.uniform(1.30, 1.40, n).astype(np.float32)
    return t, c, nf


def spectral_cmf(wl: np.ndarray = WAVELENGTHS_81, seed: int = 4) -> np.ndarray:
    """[len(wl), 3] colour-matching matrix: per channel a sum of 2 or 3 Gaussian lobes with
    seeded amplitude U[0.2, 1.2], centre in the channel's band and width U[15, 60] nm."""
    g = rng(seed)
    bands = [(550.0, 700.0), (480.0, 600.0), (400.0, 500.0)]  # R, G, B
    out = np.zeros((wl.size, 3))
    for ch, (lo, hi) in enumerate(bands):
        for _ in range(int(g.integers(2, 4))):
            a, mu, s = g.uniform(0.2, 1.2), g.uniform(lo, hi), g.uniform(15.0, 60.0)
            out[:, ch] += a * np.exp(-0.5 * ((wl - mu) / s) ** 2)
    return out


def delta_e76(rgb_a: np.ndarray, rgb_b: np.ndarray, white: np.ndarray) -> np.ndarray:
    """CIE76 colour difference of two linear-RGB arrays [n, 3]: each channel is divided by the
    white response (the CMF column sums: a perfect reflector maps to 1), then linear sRGB -> XYZ
    (D65) -> CIELAB."""
    M = np.array([[0.4124564, 0.3575761, 0.1804375], [0.2126729, 0.7151522, 0.0721750],
                  [0.0193339, 0.1191920, 0.9503041]])
    wn = np.array([0.95047, 1.0, 1.08883])

    def lab(rgb):
        xyz = (np.asarray(rgb, np.float64) / white) @ M.T / wn
        d = 6.0 / 29.0
        f = np.where(xyz > d ** 3, np.cbrt(np.maximum(xyz, 0)), xyz / (3 * d * d) + 4.0 / 29.0)
        return np.stack([116 * f[:, 1] - 16, 500 * (f[:, 0] - f[:, 1]), 200 * (f[:, 1] - f[:, 2])], axis=1)

    return np.linalg.norm(lab(rgb_a) - lab(rgb_b), axis=1)


# --- batched foam workload ------------------------------------------------------------------
def foam_bubbles(n: int = 4096, seed: int = 6):
    """Diameters log-uniform in 2-80 mm; resolution = 32 * round(512 d / 80 mm / 32) clamped to
    [32, 512] (theta rows; phi = 2 x rows). Returns (resolution uint32 [n], radius metres f32 [n])."""
    g = rng(seed)
    d_mm = np.exp(g.uniform(np.log(2.0), np.log(80.0), n))
    res = np.clip(32 * np.round(512.0 * d_mm / 80.0 / 32.0), 32, 512).astype(np.uint32)
    return res, (d_mm * 1e-3 / 2.0).astype(np.float32)


def foam_fields(res: np.ndarray, seed: int = 7):
    """Per bubble: h = U[300, 800] nm x (1 + 0.05 U[-1, 1]) (f32, [res][2 res]); surfactant 0.5."""
    g = rng(seed)
    hs = []
    for r in res:
        base = g.uniform(300e-9, 800e-9)
        hs.append((base * (1.0 + 0.05 * g.uniform(-1.0, 1.0, size=(int(r), 2 * int(r))))).astype(np.float32))
    return hs
