"""GPU: batched ensembles (hcc_upload_batch) — many independent clouds advanced by one context.

The union the library builds is checked against the oracle run on the same union (bit for bit: lists, states,
MOOD flags), no particle may have a neighbour in another cloud, per-cloud total mass is the per-cloud sum, and each
cloud's solution equals its stand-alone run up to summation order (the cell list of the union bins differently).
"""
import sys

import numpy as np
import pytest

from conftest import quadrant_ic

pytestmark = pytest.mark.gpu

OUTFLOW = {t: 2 for t in range(1, 5)}


def _clouds(hcc, h, sizes):
    return [hcc.rectangular_cloud((0.0, 0.0), (n * h, n * h), h, 2.5 * h, jitter=0.25 * h, seed=11 + k)
            for k, n in enumerate(sizes)]


def _local_quadrant(cloud, L):
    c = type(cloud)(cloud.pos / L, cloud.is_boundary, cloud.tags, cloud.volumes, cloud.dx, cloud.radius,
                    cloud.domain_min, cloud.domain_max, cloud.canvas_min, cloud.canvas_max, cloud.periodic)
    return quadrant_ic(c)


def test_batch_union_matches_the_oracle_and_stays_independent(hcc, oracle, cuda_lib):
    abi = sys.modules["hcc_gb300._abi"]
    h = 1 / 64
    sizes = (24, 40, 16)
    clouds = _clouds(hcc, h, sizes)
    cfg = hcc.make_config(hcc.Euler(2, 1.4), clouds[0], scheme=hcc.MUSCL(2, 2),
                          mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), bc_map=OUTFLOW)
    g = hcc.Context(cfg)
    union = g.upload_batch(clouds)
    g.build_neighbours()
    g.prepare_geometry()
    offs = union.meta["offsets"]
    cloud_of = np.repeat(np.arange(len(clouds)), np.diff(offs))
    # no neighbour in another cloud
    counts, idx, _, _ = g.neighbours()
    owner = np.repeat(np.arange(union.n), counts)
    assert np.array_equal(cloud_of[owner], cloud_of[idx])
    # the oracle on the same union
    o = oracle.OracleContext(hcc.make_config(hcc.Euler(2, 1.4), union, scheme=hcc.MUSCL(2, 2),
                                             mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), bc_map=OUTFLOW), abi)
    o.upload_cloud(union)
    o.build_neighbours()
    o.prepare_geometry()
    co, io, _, _ = o.neighbours()
    np.testing.assert_array_equal(counts, co)
    np.testing.assert_array_equal(idx, io)
    U0 = np.concatenate([_local_quadrant(c, n * h) for c, n in zip(clouds, sizes)])
    g.upload_state(U0)
    o.upload_state(U0)
    dt = 0.3 * o.time_step()
    assert g.time_step() == o.time_step()
    for k in range(3):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
    Ug, Uo = g.download_state(), o.download_state()
    assert np.array_equal(Ug.view(np.uint64), Uo.view(np.uint64))
    np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())
    assert o.mood_flags().sum() > 0
    # per-cloud mass
    mass = g.batch_total_mass()
    for b in range(len(clouds)):
        sl = slice(offs[b], offs[b + 1])
        want = (Uo[sl] * union.volumes[sl, None]).sum(axis=0)
        np.testing.assert_allclose(mass[b], want, rtol=1e-12)
    # each cloud alone, same dt: equal up to summation order
    for b, (c, n) in enumerate(zip(clouds, sizes)):
        cfg1 = hcc.make_config(hcc.Euler(2, 1.4), c, scheme=hcc.MUSCL(2, 2),
                               mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), bc_map=OUTFLOW)
        g1 = hcc.Context(cfg1)
        g1.upload_cloud(c)
        g1.build_neighbours()
        g1.prepare_geometry()
        g1.upload_state(_local_quadrant(c, n * h))
        for k in range(3):
            g1.step(k * dt, dt)
        U1 = g1.download_state()
        sl = slice(offs[b], offs[b + 1])
        inner = c.is_boundary == 0
        rel = np.abs(U1[inner] - Ug[sl][inner]).sum() / np.abs(U1[inner]).sum()
        assert rel < 1e-9, (b, rel)


def test_bgk_batch_matches_the_oracle(hcc, oracle, cuda_lib):
    """A BGK batch (16 ring velocities, IMEX ARS(2,2,2), clouds started at the Maxwellian of their densities):
    states and MOOD flags of the union bit for bit against the oracle, FP64."""
    abi = sys.modules["hcc_gb300._abi"]
    h = 1 / 48
    clouds = _clouds(hcc, h, (20, 12))
    ring = [(float(np.cos(2 * np.pi * q / 16)), float(np.sin(2 * np.pi * q / 16))) for q in range(16)]
    pde = hcc.KineticRelaxation(ring, epsilon=1e-4, macro_velocity=(1.0, 0.5))
    kw = dict(scheme=hcc.MUSCL(2, 2), mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), tableau="IMEX_ARS222",
              bc_map=OUTFLOW)
    g = hcc.Context(hcc.make_config(pde, clouds[0], **kw))
    union = g.upload_batch(clouds)
    g.build_neighbours()
    g.prepare_geometry()
    o = oracle.OracleContext(hcc.make_config(pde, union, **kw), abi)
    o.upload_cloud(union)
    o.build_neighbours()
    o.prepare_geometry()
    rho = 1.0 + 0.2 * np.sin(7.0 * union.pos[:, 0]) * np.cos(5.0 * union.pos[:, 1])
    U0 = pde.maxwellian(rho)
    g.upload_state(U0)
    o.upload_state(U0)
    dt = 0.4 * o.time_step()
    assert g.time_step() == o.time_step()
    for k in range(3):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
    assert np.array_equal(g.download_state().view(np.uint64), o.download_state().view(np.uint64))
    np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())


def test_batch_rejects_periodic_and_bad_offsets(hcc, cuda_lib):
    h = 1 / 32
    per = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True)
    g = hcc.Context(hcc.make_config(hcc.LinearAdvection(((1.0,), (1.0,))), per))
    with pytest.raises(hcc.HCCError):
        g.upload_batch([per, per])


def _scaled_quadrant(c, L, s):
    """The local quadrant state with every velocity scaled by sqrt(s) and the pressure by s: all wave speeds scale
    by sqrt(s), so the clouds of a batch get different CFL steps."""
    U = _local_quadrant(c, L)
    q = np.sqrt(s)
    return np.column_stack([U[:, 0], U[:, 1] * q, U[:, 2] * q, U[:, 3] * s])


def test_batch_steps_each_cloud_with_its_own_dt(hcc, cuda_lib):
    """One dt per cloud (the reference steps every ParticleGrid with its own get_time_step, ParticleGrids.jl:386-415):
    the per-cloud CFL steps equal each cloud's stand-alone step and their minimum the batch's; a batch step with
    those dts equals every cloud's stand-alone run at its own dt up to summation order; the step graph and the
    host-driven step agree bit for bit."""
    h = 1 / 64
    sizes = (24, 40, 16)
    scales = (1.0, 4.0, 9.0)
    clouds = _clouds(hcc, h, sizes)
    kw = dict(scheme=hcc.MUSCL(2, 2), mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), bc_map=OUTFLOW)
    ctxs = []
    for graphs in (True, False):
        g = hcc.Context(hcc.make_config(hcc.Euler(2, 1.4), clouds[0], **kw))
        union = g.upload_batch(clouds)
        g.build_neighbours()
        g.prepare_geometry()
        g.set_step_graphs(graphs)
        g.upload_state(np.concatenate([_scaled_quadrant(c, n * h, s) for c, n, s in zip(clouds, sizes, scales)]))
        ctxs.append(g)
    g = ctxs[0]
    offs = union.meta["offsets"]
    dts = g.batch_time_steps()
    assert len(set(dts.tolist())) == 3 and dts.min() == g.time_step()
    assert dts[0] > dts[1] > dts[2]
    steps = 0.3 * dts
    for k in range(3):
        for c in ctxs:
            c.step_batch(k * 0.0, steps)
    Ug = ctxs[0].download_state()
    assert np.array_equal(Ug.view(np.uint64), ctxs[1].download_state().view(np.uint64))
    np.testing.assert_array_equal(ctxs[0].mood_flags(), ctxs[1].mood_flags())
    for b, (c, n, s) in enumerate(zip(clouds, sizes, scales)):
        g1 = hcc.Context(hcc.make_config(hcc.Euler(2, 1.4), c, **kw))
        g1.upload_cloud(c)
        g1.build_neighbours()
        g1.prepare_geometry()
        g1.upload_state(_scaled_quadrant(c, n * h, s))
        assert abs(g1.time_step() - dts[b]) <= 1e-12 * dts[b]
        for k in range(3):
            g1.step(0.0, steps[b])
        U1 = g1.download_state()
        sl = slice(offs[b], offs[b + 1])
        inner = c.is_boundary == 0
        rel = np.abs(U1[inner] - Ug[sl][inner]).sum() / np.abs(U1[inner]).sum()
        assert rel < 1e-9, (b, rel)
    # a single-dt step afterwards still works (the graphs switch back)
    g.step(0.0, float(steps.min()))
    assert np.all(np.isfinite(g.download_state()))
