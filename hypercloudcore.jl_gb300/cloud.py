"""Point clouds for the explicit right-hand-side path.

Host-side set-up that the reference runs once per grid (out of the kernels' scope): the rectangular geometry
with its ghost canvas, the jittered lattice, the narrow ghost band, the boundary tags and the Morton numbering.
It restates

  * ``get_rectangular_domain`` (src/Grid/Domains.jl:46-97) — interior test and face tags,
  * ``ComputationalDomain`` (src/Grid/Domains.jl:159-191) — ghost layers and canvas,
  * ``get_points`` (src/Grid/Domains.jl:220-287) — lattice, wall snapping, jitter, periodic wrap, ghost band,
  * the Morton reorder (src/Grid/Reordering.jl:55-102) — the particle numbering the neighbour lists follow,

with a counter-based splitmix64 generator in place of Julia's MersenneTwister (the reference's stream is not
reproduced; both sides of every comparison get the same positions from here).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_EPS64 = np.finfo(np.float64).eps


def splitmix64_uniform(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Uniform doubles in [0, 1) from a counter-based splitmix64 stream: value k uses counter seed + (k+1)·φ."""
    k = np.arange(offset, offset + count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (k + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _wall_index(w: float, canvas_min: float, dx: float) -> int:
    """Lattice index of a wall, or -1 (src/Grid/Domains.jl:202-207)."""
    r = (w - canvas_min) / dx
    k = int(np.rint(r))
    tol = (2 * (np.spacing(abs(w)) + np.spacing(abs(canvas_min))) + _EPS64 * abs(w - canvas_min)) / dx \
        + 4 * _EPS64 * abs(r)
    return k if abs(r - k) <= min(0.25, tol) else -1


def _julia_mod(x: np.ndarray, y: float) -> np.ndarray:
    r = np.fmod(x, y)
    return np.where(r == 0, np.copysign(r, y), np.where((r > 0) != (y > 0), r + y, r))


def rect_tags(pos: np.ndarray, mins, maxs, periodic) -> np.ndarray:
    """Face tags 2d-1 / 2d of the box (farthest outside wins, lower tag on ties); 0 inside
    (src/Grid/Domains.jl:59-94)."""
    n, D = pos.shape
    inside = np.ones(n, dtype=bool)
    for d in range(D):
        inside &= (pos[:, d] >= mins[d]) & (pos[:, d] <= maxs[d])
    best_tag = np.zeros(n, dtype=np.int32)
    best_out = np.zeros(n, dtype=np.float64)
    for d in range(D):
        if periodic[d]:
            continue
        o_lo = mins[d] - pos[:, d]
        o_hi = pos[:, d] - maxs[d]
        sel = o_lo > best_out
        best_tag = np.where(sel, 2 * d + 1, best_tag)
        best_out = np.where(sel, o_lo, best_out)
        sel = o_hi > best_out
        best_tag = np.where(sel, 2 * d + 2, best_tag)
        best_out = np.where(sel, o_hi, best_out)
    # points outside only a periodic axis: nearest face plane (cannot occur after the periodic wrap)
    missing = (~inside) & (best_tag == 0)
    if missing.any():
        bd = np.full(n, np.inf)
        bt = np.ones(n, dtype=np.int32)
        for d in range(D):
            if periodic[d]:
                continue
            dl = np.abs(pos[:, d] - mins[d])
            dh = np.abs(pos[:, d] - maxs[d])
            s = dl < bd
            bt = np.where(s, 2 * d + 1, bt); bd = np.where(s, dl, bd)
            s = dh < bd
            bt = np.where(s, 2 * d + 2, bt); bd = np.where(s, dh, bd)
        best_tag = np.where(missing, bt, best_tag)
    return np.where(inside, 0, best_tag).astype(np.int32)


def _expand_bits_2d(w: np.ndarray) -> np.ndarray:
    w = w & np.uint32(0x0000FFFF)
    w = (w | (w << np.uint32(8))) & np.uint32(0x00FF00FF)
    w = (w | (w << np.uint32(4))) & np.uint32(0x0F0F0F0F)
    w = (w | (w << np.uint32(2))) & np.uint32(0x33333333)
    w = (w | (w << np.uint32(1))) & np.uint32(0x55555555)
    return w


def _expand_bits_3d(w: np.ndarray) -> np.ndarray:
    w = w & np.uint32(0x000003FF)
    w = (w | (w << np.uint32(16))) & np.uint32(0xFF0000FF)
    w = (w | (w << np.uint32(8))) & np.uint32(0x0300F00F)
    w = (w | (w << np.uint32(4))) & np.uint32(0x030C30C3)
    w = (w | (w << np.uint32(2))) & np.uint32(0x09249249)
    return w


def morton_permutation(pos: np.ndarray, box_min, box_max) -> np.ndarray:
    """Morton (Z-order) permutation of the particles (src/Grid/Reordering.jl:55-102): keys of 16 bits per
    axis in 2-D, 10 in 3-D, ((x - min) / extent) * top floored and clamped; 1-D sorts by x. Stable sort
    (the reference's QuickSort is unstable; the clouds here have no key ties)."""
    n, D = pos.shape
    if D == 1:
        return np.argsort(pos[:, 0], kind="stable")
    top = 65535 if D == 2 else 1023
    keys = []
    for d in range(D):
        ext = box_max[d] - box_min[d]
        v = np.floor((pos[:, d] - box_min[d]) / ext * float(top))
        keys.append(np.clip(v, 0, top).astype(np.uint32))
    if D == 2:
        code = _expand_bits_2d(keys[0]) | (_expand_bits_2d(keys[1]) << np.uint32(1))
    else:
        code = _expand_bits_3d(keys[0]) | (_expand_bits_3d(keys[1]) << np.uint32(1)) | \
            (_expand_bits_3d(keys[2]) << np.uint32(2))
    return np.argsort(code, kind="stable")


@dataclass
class Cloud:
    """A particle cloud in the reference's numbering, plus the canvas the cell list spans."""
    pos: np.ndarray                 # (N, D) float64
    is_boundary: np.ndarray         # (N,) uint8
    tags: np.ndarray                # (N,) int32
    volumes: np.ndarray             # (N,) float64
    dx: tuple
    radius: float
    domain_min: tuple
    domain_max: tuple
    canvas_min: tuple
    canvas_max: tuple
    periodic: tuple
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    @property
    def dim(self) -> int:
        return int(self.pos.shape[1])

    @property
    def n_interior(self) -> int:
        return int((self.is_boundary == 0).sum())


def rectangular_cloud(mins, maxs, dx, radius: float, *, periodic=False, jitter=None, seed: int = 42,
                      reorder: bool = True) -> Cloud:
    """ParticleGrid(get_rectangular_domain(T, mins, maxs; is_periodic), dx, ExponentialWeightFunction(α, radius), M;
    randomness = jitter) point set (src/Grid/ParticleGrids.jl:221-279, src/Grid/Domains.jl:159-287).

    `jitter` is the per-axis amplitude of the uniform offset (the reference's `randomness`)."""
    mins = tuple(float(v) for v in mins)
    maxs = tuple(float(v) for v in maxs)
    D = len(mins)
    dxs = tuple(float(v) for v in (dx if isinstance(dx, (tuple, list)) else (dx,) * D))
    per = tuple(bool(v) for v in (periodic if isinstance(periodic, (tuple, list)) else (periodic,) * D))
    rnd = tuple(float(v) for v in (jitter if isinstance(jitter, (tuple, list)) else
                                   ((jitter or 0.0),) * D))
    max_dx = max(dxs)
    range_factor = radius / max_dx
    n_ghost = []
    for d in range(D):
        if dxs[d] == max_dx:
            n_ghost.append(math.ceil(range_factor))
        else:
            n_ghost.append(math.ceil(range_factor * (max_dx / dxs[d]) * (1 - 4 * _EPS64)))
    cmin = tuple(mins[d] if per[d] else mins[d] - n_ghost[d] * dxs[d] for d in range(D))
    cmax = tuple(maxs[d] if per[d] else maxs[d] + n_ghost[d] * dxs[d] for d in range(D))
    L = tuple(maxs[d] - mins[d] for d in range(D))
    ns = []
    for d in range(D):
        n = max(1, int(np.rint((cmax[d] - cmin[d]) / dxs[d])))
        ns.append(n if per[d] else n + 1)
    wall_lo = [(-1 if per[d] else _wall_index(mins[d], cmin[d], dxs[d])) for d in range(D)]
    wall_hi = [(-1 if per[d] else _wall_index(maxs[d], cmin[d], dxs[d])) for d in range(D)]
    total = int(np.prod(ns))
    # CartesianIndices order: axis 0 fastest
    lin = np.arange(total, dtype=np.int64)
    idx = []
    r = lin.copy()
    for d in range(D):
        idx.append(r % ns[d])
        r //= ns[d]
    u = splitmix64_uniform(seed, total * D).reshape(total, D) if any(v != 0.0 for v in rnd) else None
    pos = np.empty((total, D), dtype=np.float64)
    for d in range(D):
        j = idx[d]
        x = cmin[d] + j.astype(np.float64) * dxs[d]
        x = np.where(j == wall_lo[d], mins[d], np.where(j == wall_hi[d], maxs[d], x))
        if u is not None:
            x = x + rnd[d] * (u[:, d] * 2 - 1)
        if per[d]:
            y = mins[d] + _julia_mod(x - mins[d], L[d])
            x = np.where(y >= mins[d] + L[d], mins[d], y)
        pos[:, d] = x
    inside = np.ones(total, dtype=bool)
    for d in range(D):
        inside &= (pos[:, d] >= mins[d]) & (pos[:, d] <= maxs[d])
    inner = pos[inside]
    cand = pos[~inside]
    cutoff_sq = (range_factor * max_dx + max_dx) ** 2
    if len(inner) and len(cand):
        from scipy.spatial import cKDTree
        tree = cKDTree(inner)
        _, nearest = tree.query(cand, k=1)
        d2 = ((cand - inner[nearest]) ** 2).sum(axis=1)
        ghosts = cand[d2 <= cutoff_sq]
    else:
        ghosts = cand[:0]
    pos = np.concatenate([inner, ghosts], axis=0)
    tags = rect_tags(pos, mins, maxs, per)
    is_b = (tags != 0).astype(np.uint8)
    vol = np.full(pos.shape[0], float(np.prod(dxs)))
    if reorder and pos.shape[0] > 1:
        perm = morton_permutation(pos, cmin, cmax)
        pos, tags, is_b, vol = pos[perm], tags[perm], is_b[perm], vol[perm]
    return Cloud(pos=np.ascontiguousarray(pos), is_boundary=np.ascontiguousarray(is_b),
                 tags=np.ascontiguousarray(tags), volumes=vol, dx=dxs, radius=float(radius),
                 domain_min=mins, domain_max=maxs, canvas_min=cmin, canvas_max=cmax, periodic=per,
                 meta={"lattice": tuple(ns), "seed": seed, "jitter": rnd})
