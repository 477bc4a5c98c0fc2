"""GPU parity at the benchmark workloads' full sizes (the clouds the throughput figures are quoted on).

- 2-D Euler quadrant at h = 1e-3 (1.0M interior, 1.01M particles): FP64 neighbour lists, divergence weights, CFL
  step and three SSP-RK3 steps (states, orders, MOOD flags) bit for bit against the oracle; the FP32 bulk path after
  the same steps within 1e-5 relative L1 per component of the oracle.
- 3-D Euler blast at h = 1/100 (1.0M interior, K ~ 66): the same for two steps.
- 3-D Euler blast at h = 1/200 (8.0M interior, 8.85M particles, ~5.9e8 slots): the neighbour count of every particle,
  and the full lists (indices in order, weights, distances) of 10,000 seeded particles plus the extremes of the count,
  bit for bit against the oracle's own search.
These exercise what small clouds do not: 64-bit slot offsets, thousands of bins in the scan, worklists with
hundreds of MOOD tiles spread over many blocks.
"""
import sys

import numpy as np
import pytest

from conftest import blast_ic, quadrant_ic

pytestmark = pytest.mark.gpu


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def _cloud(hcc, D, h):
    # the benchmark's clouds: unit box, R = 2.5h, jitter +-0.25h, seed 42
    return hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, jitter=0.25 * h, seed=42)


def _cfg(hcc, cloud, h, precision):
    D = cloud.dim
    return hcc.make_config(hcc.Euler(D), cloud, scheme=hcc.MUSCL(2, 2),
                           mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h ** D)),
                           bc_map={t: hcc.BC_OUTFLOW for t in range(1, 2 * D + 1)}, precision=precision)


def _ready(ctx, cloud, U):
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.upload_state(U)


def _full_size_steps(hcc, oracle, D, h, steps):
    abi = sys.modules["hcc_gb300._abi"]
    cloud = _cloud(hcc, D, h)
    U0 = quadrant_ic(cloud) if D == 2 else blast_ic(cloud)
    oracle.OracleContext.set_threads(0)
    o = oracle.OracleContext(_cfg(hcc, cloud, h, "fp64"), abi)
    g = hcc.Context(_cfg(hcc, cloud, h, "fp64"))
    for c in (g, o):
        _ready(c, cloud, U0)
    cg, ig, wg, dg = g.neighbours()
    co, io, wo, do = o.neighbours()
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(ig, io)
    assert _bits_equal(wg, wo) and _bits_equal(dg, do)
    tot = int(co.sum())
    del ig, io, wg, wo, dg, do
    dwg, okrg, okdg = g.geometry(tot)
    dwo, okro, okdo = o.geometry(tot)
    np.testing.assert_array_equal(okrg, okro)
    np.testing.assert_array_equal(okdg, okdo)
    assert _bits_equal(dwg, dwo)
    del dwg, dwo
    dt = o.time_step()
    assert g.time_step() == dt
    dt = 0.4 * dt
    f = hcc.Context(_cfg(hcc, cloud, h, "fp32"))
    _ready(f, cloud, U0)
    for k in range(steps):
        for c in (g, o, f):
            c.step(k * dt, dt)
        uo = o.download_state()
        assert _bits_equal(g.download_state(), uo), f"step {k}"
        np.testing.assert_array_equal(g.orders(), o.orders())
        np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())
    assert o.counters()["mood_flagged"] > 0                     # MOOD acted on this cloud
    assert g.counters()["mood_iterations"] == o.counters()["mood_iterations"]
    uf = f.download_state()
    inner = cloud.is_boundary == 0
    for m in range(U0.shape[1]):
        scale = np.abs(uo[inner, m]).sum() + np.abs(uo[inner, 0]).sum() * 1e-3   # momenta start at zero
        assert np.abs(uf[inner, m] - uo[inner, m]).sum() <= 1e-5 * scale, m
    for c in (g, o, f):
        c.close()


def test_quadrant_1M_fp64_steps_bit_exact(hcc, oracle, cuda_lib):
    _full_size_steps(hcc, oracle, 2, 1e-3, steps=3)


def test_blast_3d_1M_fp64_steps_bit_exact(hcc, oracle, cuda_lib):
    _full_size_steps(hcc, oracle, 3, 1.0 / 100, steps=2)


def test_blast_3d_8M_neighbour_counts_and_sampled_lists(hcc, oracle, cuda_lib):
    abi = sys.modules["hcc_gb300._abi"]
    h = 1.0 / 200
    cloud = _cloud(hcc, 3, h)
    assert cloud.n > 8_000_000
    g = hcc.Context(_cfg(hcc, cloud, h, "fp32"))
    g.upload_cloud(cloud)
    g.build_neighbours()
    cg = g.neighbour_counts()
    oracle.OracleContext.set_threads(0)
    o = oracle.OracleContext(_cfg(hcc, cloud, h, "fp64"), abi)
    o.upload_cloud(cloud)
    co = o.neighbour_counts()
    np.testing.assert_array_equal(cg, co)
    assert g.counters()["total_neighbours"] == int(co.sum())
    rng = np.random.default_rng(2026)
    ids = np.unique(np.concatenate([rng.choice(cloud.n, 10_000, replace=False),
                                    [int(np.argmax(co)), int(np.argmin(co)), 0, cloud.n - 1],
                                    np.nonzero(cloud.is_boundary)[0][:50]]))
    mx = int(co[ids].max())
    c1, i1, w1, d1 = g.neighbours_of(ids, mx)
    c2, i2, w2, d2 = o.neighbours_of(ids, mx)
    np.testing.assert_array_equal(c1, c2)
    np.testing.assert_array_equal(i1, i2)                     # same neighbours in the same order
    assert _bits_equal(w1, w2) and _bits_equal(d1, d2)
    g.close()
    o.close()
