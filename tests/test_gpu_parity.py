"""GPU parity: the CUDA library against the CPU oracle on the same seeded clouds and states.

FP64 plain path: neighbour lists (indices, order, weights, distances), divergence weights, right-hand sides, states,
orders, MOOD flags and CFL steps are compared bit for bit (both sides evaluate the same operation sequence without
contraction). FP32 bulk path: states within the stated tolerance of the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import c1_cloud, gaussian_ic, quadrant_ic, blast_ic

pytestmark = pytest.mark.gpu

ADV_BC = {1: 1, 3: 1, 2: 2, 4: 2}      # left/bottom inflow -> FixedDirichlet, right/top -> OutflowBC
OUTFLOW = {t: 2 for t in range(1, 7)}


def _pair(hcc, oracle, cfg, cloud):
    abi = __import__("sys").modules["hcc_gb300._abi"]
    g = hcc.Context(cfg)
    o = oracle.OracleContext(cfg, abi)
    for c in (g, o):
        c.upload_cloud(cloud)
        c.build_neighbours()
        c.prepare_geometry()
    return g, o


def _assert_same_lists(g, o):
    cg, ig, wg, dg = g.neighbours()
    co, io, wo, do = o.neighbours()
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(ig, io)          # same neighbours in the same order
    assert np.array_equal(wg.view(np.uint64), wo.view(np.uint64))
    assert np.array_equal(dg.view(np.uint64), do.view(np.uint64))
    return co, io


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


@pytest.mark.parametrize("D,periodic", [(1, True), (2, False), (2, True), (3, False)])
def test_neighbour_lists_bit_exact(hcc, oracle, cuda_lib, D, periodic):
    h = {1: 0.01, 2: 0.02, 3: 0.05}[D]
    cloud = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, periodic=periodic, jitter=0.25 * h, seed=7)
    pde = hcc.LinearAdvection(tuple((1.0,) for _ in range(D)))
    cfg = hcc.make_config(pde, cloud, scheme=hcc.MUSCL(2, 2))
    g, o = _pair(hcc, oracle, cfg, cloud)
    counts, idx = _assert_same_lists(g, o)
    assert counts.sum() > 0 and idx.min() >= 0
    tot = int(counts.sum())
    dwg, okrg, okdg = g.geometry(tot)
    dwo, okro, okdo = o.geometry(tot)
    np.testing.assert_array_equal(okrg, okro)
    np.testing.assert_array_equal(okdg, okdo)
    assert _bits_equal(dwg, dwo)


def test_advection_rhs_and_steps_bit_exact(hcc, oracle, cuda_lib):
    cloud = c1_cloud(hcc)
    pde = hcc.LinearAdvection(((1.0,), (1.0,)))
    h = 0.01
    mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h))
    cfg = hcc.make_config(pde, cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=ADV_BC)
    g, o = _pair(hcc, oracle, cfg, cloud)
    U0 = gaussian_ic(cloud)
    g.upload_state(U0)
    o.upload_state(U0)
    assert _bits_equal(g.compute_rhs(), o.compute_rhs())
    dtg, dto = g.time_step(), o.time_step()
    assert dtg == dto and np.isfinite(dtg)
    dt = 0.5 * dto
    t = 0.0
    flagged = 0
    for _ in range(6):
        g.step(t, dt)
        o.step(t, dt)
        t += dt
        assert _bits_equal(g.download_state(), o.download_state())
        np.testing.assert_array_equal(g.orders(), o.orders())
        np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())
        flagged += int(o.mood_flags().sum())
    assert flagged > 0                            # MOOD acted in this window
    assert g.counters()["inadmissible"] == o.counters()["inadmissible"]
    np.testing.assert_allclose(g.total_mass(), o.total_mass(), rtol=1e-12)


@pytest.mark.parametrize("order", [2, 3])
def test_euler2d_quadrant_steps_bit_exact(hcc, oracle, cuda_lib, order):
    h = 0.02
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=3)
    mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h))
    cfg = hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(order, 0), mood=mood, bc_map=OUTFLOW)
    g, o = _pair(hcc, oracle, cfg, cloud)
    U0 = quadrant_ic(cloud)
    g.upload_state(U0)
    o.upload_state(U0)
    dt = 0.4 * o.time_step()
    assert g.time_step() == o.time_step()
    for k in range(4):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
        assert _bits_equal(g.download_state(), o.download_state()), f"step {k}"
        np.testing.assert_array_equal(g.orders(), o.orders())
        np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())
    assert o.counters()["mood_flagged"] > 0


def test_euler3d_blast_steps_bit_exact(hcc, oracle, cuda_lib):
    h = 1.0 / 16
    cloud = hcc.rectangular_cloud((0.0,) * 3, (1.0,) * 3, h, 2.5 * h, jitter=0.25 * h, seed=11)
    mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h ** 3))
    cfg = hcc.make_config(hcc.Euler(3), cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=OUTFLOW)
    g, o = _pair(hcc, oracle, cfg, cloud)
    U0 = blast_ic(cloud)
    g.upload_state(U0)
    o.upload_state(U0)
    dt = 0.4 * o.time_step()
    for k in range(2):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
        assert _bits_equal(g.download_state(), o.download_state())
        np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())


def test_bgk_imex_steps_bit_exact(hcc, oracle, cuda_lib):
    h = 0.04
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True, jitter=0.2 * h, seed=5)
    ang = 2 * np.pi * np.arange(16) / 16
    speeds = tuple((float(np.cos(a)), float(np.sin(a))) for a in ang)
    pde = hcc.KineticRelaxation(speeds, epsilon=1e-4, macro_velocity=(1.0, 0.5))
    cfg = hcc.make_config(pde, cloud, scheme=hcc.MUSCL(2, 2), mood=hcc.MOOD(hcc.EPD1, hcc.MOODPAD()),
                          tableau="IMEX_ARS222")
    g, o = _pair(hcc, oracle, cfg, cloud)
    x, y = cloud.pos[:, 0], cloud.pos[:, 1]
    rho = 1.0 + 0.3 * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
    U0 = np.repeat(rho[:, None] / 16.0, 16, axis=1)
    g.upload_state(U0)
    o.upload_state(U0)
    dt = 0.3 * o.time_step()
    for k in range(3):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
        assert _bits_equal(g.download_state(), o.download_state())


def test_fp32_bulk_within_tolerance(hcc, oracle, cuda_lib):
    """FP32 bulk path vs the FP64 oracle after 5 steps of the quadrant problem: L1 density error below 1e-4
    relative (FP32 round-off; MOOD decisions may differ where a candidate sits within round-off of a bound)."""
    h = 0.02
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=3)
    mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h))
    cfg64 = hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=OUTFLOW)
    cfg32 = hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=OUTFLOW, precision="fp32")
    abi = __import__("sys").modules["hcc_gb300._abi"]
    o = oracle.OracleContext(cfg64, abi)
    g = hcc.Context(cfg32)
    for c in (g, o):
        c.upload_cloud(cloud)
        c.build_neighbours()
        c.prepare_geometry()
    U0 = quadrant_ic(cloud)
    o.upload_state(U0)
    g.upload_state(U0.astype(np.float32))
    dt = 0.4 * o.time_step()
    for k in range(5):
        o.step(k * dt, dt)
        g.step(k * dt, dt)
    Uo, Ug = o.download_state(), g.download_state()
    interior = cloud.is_boundary == 0
    l1 = np.abs(Ug[interior, 0] - Uo[interior, 0]).sum() / np.abs(Uo[interior, 0]).sum()
    assert l1 < 1e-4, l1


@pytest.mark.parametrize("order,limiter", [(3, "vk_hard"), (2, "bj_soft"), (3, "bj_hard")])
def test_limited_muscl_steps_bit_exact(hcc, oracle, cuda_lib, order, limiter):
    """MUSCL with Barth-Jespersen / Venkatakrishnan limiting (Limiter.jl:120-143) + MOOD: states, orders, flags."""
    h = 0.02
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=13)
    mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h))
    cfg = hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(order, 0, limiter), mood=mood, bc_map=OUTFLOW)
    g, o = _pair(hcc, oracle, cfg, cloud)
    U0 = quadrant_ic(cloud)
    g.upload_state(U0)
    o.upload_state(U0)
    dt = 0.4 * o.time_step()
    for k in range(3):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
        assert _bits_equal(g.download_state(), o.download_state()), f"step {k}"
        np.testing.assert_array_equal(g.orders(), o.orders())
        np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())


def test_published_benchmark_case_bit_exact(hcc, oracle, cuda_lib):
    """The reference benchmark's scheme (benchmark/step.jl:56-74): periodic lattice, advection speeds (1, 0.5),
    MUSCL3 + VK(:hard) + MOOD(EPD1, MOODu1(1e-6)), SSP-RK3, dt = 0.3 x the CFL step; a 64^2 cloud."""
    n = 64
    h = 1.0 / n
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True)
    cfg = hcc.make_config(hcc.LinearAdvection(((1.0,), (0.5,))), cloud, scheme=hcc.MUSCL(3, 0, "vk_hard"),
                          mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-6)))
    g, o = _pair(hcc, oracle, cfg, cloud)
    U0 = np.exp(-((cloud.pos - 0.5) ** 2).sum(axis=1) / 0.02)[:, None]
    g.upload_state(U0)
    o.upload_state(U0)
    dt = 0.3 * o.time_step()
    assert g.time_step() == o.time_step()
    for k in range(4):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
    assert _bits_equal(g.download_state(), o.download_state())
    np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())


@pytest.mark.parametrize("D,order", [(1, 2), (2, 2), (2, 3), (3, 2)])
def test_weno_steps_bit_exact(hcc, oracle, cuda_lib, D, order):
    """Scalar meshless WENO (WENO.jl:55-165) with MOOD u1: RHS, CFL (assembled Taylor fit) and states."""
    h = {1: 0.02, 2: 0.04, 3: 0.1}[D]
    cloud = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, periodic=True, jitter=0.2 * h, seed=17)
    vel = tuple(((1.0, 0.5, -0.3)[d],) for d in range(D))
    cfg = hcc.make_config(hcc.LinearAdvection(vel), cloud, scheme=hcc.WENO(order),
                          mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h ** D)))
    g, o = _pair(hcc, oracle, cfg, cloud)
    r2 = ((cloud.pos - 0.5) ** 2).sum(axis=1)
    U0 = np.where(r2 < 0.04, 1.0, 0.0)[:, None] + 0.1 * np.exp(-r2 / 0.02)[:, None]
    g.upload_state(U0)
    o.upload_state(U0)
    assert _bits_equal(g.compute_rhs(), o.compute_rhs())
    assert g.time_step() == o.time_step()
    dt = 0.3 * o.time_step()
    for k in range(3):
        g.step(k * dt, dt)
        o.step(k * dt, dt)
        assert _bits_equal(g.download_state(), o.download_state()), f"step {k}"
        np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())
