"""The exact FP32 prefilter of the neighbour search (hcc_search.cu, `Prefilter`), emulated on the CPU with numpy's
correctly rounded float32 operations (the device uses the _rn intrinsics): on adversarial pairs (offsets within 0.1 %
of the radius, coordinates up to 1e3, periodic wraps near half a period, 1-D to 3-D) every pair it decides must get
the FP64 test's answer (r^2 <= R^2 with the FP64 wrap), and on a realistic cloud it must leave only a small share of
the pairs to FP64."""
import numpy as np
import pytest

U = 2.0 ** -24


def _round_down(x):
    f = np.float32(x)
    return np.nextafter(f, np.float32(-np.inf)) if float(f) > x else f


def _round_up(x):
    f = np.float32(x)
    return np.nextafter(f, np.float32(np.inf)) if float(f) < x else f


def _prefilter(pi, pj, L, R_sq, P, D):
    """+1 inside, -1 outside, 0 undecided, per pair (rows of pi, pj: float64 positions)."""
    Lmax = float(max(L)) if len(L) else 0.0
    delta = 16.0 * U * (P + Lmax)
    R = np.sqrt(R_sq)
    rho = 2.0 * (2.0 * np.sqrt(D) * delta / R + 3.0 * D * delta * delta / R_sq + D * U)
    if not rho < 0.05:
        return np.zeros(pi.shape[0], dtype=int)
    lo, hi = _round_down(R_sq * (1.0 - rho)), _round_up(R_sq / (1.0 - rho))
    pi32, pj32 = pi.astype(np.float32), pj.astype(np.float32)
    L32 = np.array(L, dtype=np.float32)
    invL32 = np.array([np.float32(1.0 / v) if v > 0 else np.float32(0.0) for v in L], dtype=np.float32)
    s = np.zeros(pi.shape[0], dtype=np.float32)
    amb = np.zeros(pi.shape[0], dtype=bool)
    for d in range(D):
        dx = pj32[:, d] - pi32[:, d]
        q = dx * invL32[d]
        r = np.rint(q)
        amb |= np.abs(np.abs(q - r) - np.float32(0.5)) < np.float32(0.01)
        dd = dx - L32[d] * r
        s = dd * dd if d == 0 else s + dd * dd
    out = np.where(s < lo, 1, np.where(s > hi, -1, 0))
    out[amb] = 0
    return out


def _fp64_inside(pi, pj, L, R_sq, D):
    s = np.zeros(pi.shape[0])
    for d in range(D):
        dx = pj[:, d] - pi[:, d]
        inv = 1.0 / L[d] if L[d] > 0 else 0.0
        dist = dx - L[d] * np.rint(dx * inv)
        s = dist * dist if d == 0 else s + dist * dist
    return s <= R_sq


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("scale,periodic", [(1.0, False), (1.0, True), (1e3, False), (1e3, True), (0.01, True)])
def test_decided_pairs_agree_with_fp64(D, scale, periodic):
    rng = np.random.default_rng(7 + D)
    n = 400_000
    L = [scale if periodic else 0.0] * D
    R = 0.0125 * scale
    pi = rng.uniform(0.0, scale, (n, D))
    # offsets concentrated at the radius (within 0.1 %), some far, some across the periodic seam
    dirs = rng.normal(size=(n, D))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rad = R * np.where(rng.random(n) < 0.8, 1.0 + rng.uniform(-1e-3, 1e-3, n), rng.uniform(0.0, 3.5, n))
    pj = pi + dirs * rad[:, None]
    if periodic:
        pj = np.where(rng.random((n, D)) < 0.3, pj - scale * np.round(pj / scale), pj)
        seam = rng.random(n) < 0.05                          # pairs half a period apart
        pj[seam, 0] = pi[seam, 0] + 0.5 * scale * (1.0 + rng.uniform(-1e-6, 1e-6, seam.sum()))
    P = float(np.abs(np.concatenate([pi, pj])).max())
    dec = _prefilter(pi, pj, L, R * R, P, D)
    inside = _fp64_inside(pi, pj, L, R * R, D)
    assert np.all(inside[dec == 1]), "a pair proved inside is outside in FP64"
    assert not np.any(inside[dec == -1]), "a pair proved outside is inside in FP64"
    assert (dec != 0).mean() > 0.3          # most of these pairs sit inside the band on purpose


def test_realistic_cloud_leaves_few_pairs_to_fp64():
    rng = np.random.default_rng(3)
    h, D = 1.0 / 200, 3
    R = 2.5 * h
    pi = rng.uniform(0.0, 1.0, (200_000, D))
    pj = pi + rng.uniform(-3.0 * R, 3.0 * R, pi.shape)      # the candidates of a 3 x 3 x 3 window of cells
    P = float(np.abs(np.concatenate([pi, pj])).max())
    dec = _prefilter(pi, pj, [0.0] * D, R * R, P, D)
    inside = _fp64_inside(pi, pj, [0.0] * D, R * R, D)
    assert np.all(inside[dec == 1]) and not np.any(inside[dec == -1])
    assert (dec == 0).mean() < 1e-3
