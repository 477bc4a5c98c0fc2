"""Tile-staged FP32 full passes (neighbours staged in shared memory per 128-particle tile, slot offsets and weights
recomputed from quantised positions and per-particle FP32 fit rows) against the stream-fed FP32 passes and the FP64
oracle.

Both FP32 forms round the same FP64 geometry to FP32. On a smooth state each right-hand side is within the FP32 path's
stated 1e-4 relative L1 per component of the FP64 oracle's, the tile form no further from it than twice the stream
form's distance (the divergence of flux differences amplifies FP32 rounding by about 1/(K h), so the two FP32 forms
themselves differ by a few 1e-5); after steps the states agree with each other and with the oracle to 1e-5 relative L1.
The tile path is taken only where the context and the cloud qualify.
"""
import sys

import numpy as np
import pytest

from conftest import blast_ic, quadrant_ic

pytestmark = pytest.mark.gpu

OUTFLOW = {t: 2 for t in range(1, 7)}


def _rel_l1(a, b, sel):
    out = []
    for m in range(a.shape[1]):
        den = np.abs(b[sel, m]).sum() + np.abs(b[sel, 0]).sum() * 1e-3
        out.append(np.abs(a[sel, m] - b[sel, m]).sum() / den)
    return max(out)


def _system(hcc, kind, h, seed=3, periodic=False):
    D = 3 if kind == "euler3d" else 2
    cloud = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, jitter=0.25 * h, seed=seed, periodic=periodic)
    mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h ** D))
    bc = {} if periodic else OUTFLOW
    if kind == "euler2d":
        cfg = lambda prec: hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=bc,
                                           precision=prec)
        U = quadrant_ic(cloud)
    elif kind == "euler3d":
        cfg = lambda prec: hcc.make_config(hcc.Euler(3), cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=bc,
                                           precision=prec)
        U = blast_ic(cloud)
    elif kind == "advection":
        pde = hcc.LinearAdvection(((1.0,), (0.5,)))
        cfg = lambda prec: hcc.make_config(pde, cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=bc, precision=prec)
        U = np.exp(-((cloud.pos - 0.4) ** 2).sum(axis=1) / 0.01)[:, None].copy()
    else:
        ring = tuple((float(np.cos(2 * np.pi * q / 16)), float(np.sin(2 * np.pi * q / 16))) for q in range(16))
        pde = hcc.KineticRelaxation(ring, epsilon=1e-4, macro_velocity=(1.0, 0.5))
        cfg = lambda prec: hcc.make_config(pde, cloud, scheme=hcc.MUSCL(2, 2), mood=mood, tableau="IMEX_ARS222",
                                           bc_map=bc, precision=prec)
        x = cloud.pos
        U = pde.maxwellian(1.0 + 0.2 * np.sin(2 * np.pi * x[:, 0]) * np.cos(2 * np.pi * x[:, 1]))
    return cloud, cfg, np.ascontiguousarray(U, dtype=np.float64)


def _smooth(kind, cloud, U):
    """A smooth state of the system (the unlimited full-order right-hand side of a discontinuous Euler state has
    negative-pressure reconstructions, NaN in either form)."""
    if not kind.startswith("euler"):
        return U
    x = cloud.pos
    D = x.shape[1]
    rho = 1.0 + 0.2 * np.prod(np.sin(2 * np.pi * x), axis=1)
    vel = np.array([0.3, -0.2, 0.1][:D])
    p = 1.0 + 0.1 * np.cos(2 * np.pi * x[:, 0])
    E = p / 0.4 + 0.5 * rho * (vel ** 2).sum()
    return np.ascontiguousarray(np.column_stack([rho] + [rho * v for v in vel] + [E]))


def _ctx(hcc, cfg, cloud, U, tiles=True):
    g = hcc.Context(cfg)
    g.upload_cloud(cloud)
    g.build_neighbours()
    g.prepare_geometry()
    g.set_tile_staging(tiles)
    g.upload_state(U)
    return g


@pytest.mark.parametrize("kind,h", [("euler2d", 0.01), ("euler3d", 1.0 / 24), ("advection", 0.01), ("bgk", 0.02)])
def test_tile_passes_match_stream_passes_and_oracle(hcc, oracle, cuda_lib, kind, h):
    abi = sys.modules["hcc_gb300._abi"]
    cloud, cfg, U0 = _system(hcc, kind, h)
    t = _ctx(hcc, cfg("fp32"), cloud, U0, tiles=True)
    s = _ctx(hcc, cfg("fp32"), cloud, U0, tiles=False)
    info = t.tile_staging()
    assert info["active"] and info["largest_union"] > 0
    assert not s.tile_staging()["active"]
    inner = cloud.is_boundary == 0
    o = oracle.OracleContext(cfg("fp64"), abi)
    o.upload_cloud(cloud)
    o.build_neighbours()
    o.prepare_geometry()
    Us = _smooth(kind, cloud, U0)
    for c in (t, s, o):
        c.upload_state(Us)
    kt, ks, ko = t.compute_rhs(), s.compute_rhs(), o.compute_rhs()
    assert np.all(np.isfinite(kt[inner]))
    et, es = _rel_l1(kt, ko, inner), _rel_l1(ks, ko, inner)
    assert et < 1e-4 and et <= 2.0 * es + 1e-7, (et, es)
    for c in (t, s, o):
        c.upload_state(U0)
    dt = 0.4 * o.time_step()
    for k in range(3):
        for c in (t, s, o):
            c.step(k * dt, dt)
    ut, us, uo = t.download_state(), s.download_state(), o.download_state()
    assert np.all(np.isfinite(ut))
    assert _rel_l1(ut, us, inner) < 1e-5
    assert _rel_l1(ut, uo, inner) < 1e-5
    for c in (t, s, o):
        c.close()


def test_tile_step_graph_matches_host_driven_tile_step(hcc, cuda_lib):
    """The captured step graph and the host-driven step run the same tile kernels: bit-identical results."""
    cloud, cfg, U0 = _system(hcc, "euler2d", 0.01)
    a = _ctx(hcc, cfg("fp32"), cloud, U0)
    b = _ctx(hcc, cfg("fp32"), cloud, U0)
    b.set_step_graphs(False)
    dt = 0.4 * a.time_step()
    for k in range(3):
        a.step(k * dt, dt)
        b.step(k * dt, dt)
    assert np.array_equal(a.download_state(dtype=np.float32), b.download_state(dtype=np.float32))
    np.testing.assert_array_equal(a.mood_flags(), b.mood_flags())


def test_tile_staging_defaults(hcc, cuda_lib):
    """On by default for 3-D FP32 contexts (where it measured faster), off for 2-D ones (where it measured slower)."""
    for kind, h, on in (("euler3d", 1.0 / 16, True), ("euler2d", 0.02, False)):
        cloud, cfg, U0 = _system(hcc, kind, h)
        g = hcc.Context(cfg("fp32"))
        g.upload_cloud(cloud)
        g.build_neighbours()
        g.prepare_geometry()
        assert g.tile_staging()["active"] == on
        g.close()


def test_tile_staging_only_where_it_applies(hcc, cuda_lib):
    cloud, cfg, U0 = _system(hcc, "euler2d", 0.02)
    g = _ctx(hcc, cfg("fp64"), cloud, U0)
    assert not g.tile_staging()["active"]                     # FP64 keeps the stream-fed (bit-exact) passes
    h = 0.02
    c3 = hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(3, 0), precision="fp32", bc_map=OUTFLOW)
    g3 = _ctx(hcc, c3, cloud, U0)
    assert not g3.tile_staging()["active"]                    # MUSCL3: degree-2 reconstruction
    ce = hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(2, 2), precision="fp32", bc_map=OUTFLOW,
                         mood=hcc.MOOD(hcc.EPD2, hcc.MOODu1(1e-4 * h * h)))
    assert not _ctx(hcc, ce, cloud, U0).tile_staging()["active"]
    # a small periodic box: a tile's union spans too much of the period for consistent minimum-image offsets
    small, cfgs, Us = _system(hcc, "advection", 0.05, periodic=True)
    assert not _ctx(hcc, cfgs("fp32"), small, Us).tile_staging()["active"]
    # (on larger periodic boxes the Morton curve's jumps still give some tiles a union wider than half the period)
    # a moving grid reads the slot streams
    cl, cfgm, Um = _system(hcc, "euler2d", 0.02)
    gm = _ctx(hcc, cfgm("fp32"), cl, Um)
    assert gm.tile_staging()["active"]
    gm.set_mover(hcc.mover("lagrangian"))
    assert not gm.tile_staging()["active"]


@pytest.mark.parametrize("kind,h", [("euler2d", 0.01), ("euler3d", 1.0 / 24), ("bgk", 0.02)])
def test_tile_cfl_matches_stream_cfl_and_oracle(hcc, oracle, cuda_lib, kind, h):
    """The tile-staged CFL step (speeds per union entry, weights from the fit rows) against the stream-fed FP32 one
    and the FP64 oracle's: the same formula on FP32 weights rounded by two routes, within 1e-5 relative."""
    abi = sys.modules["hcc_gb300._abi"]
    cloud, cfg, U0 = _system(hcc, kind, h)
    t = _ctx(hcc, cfg("fp32"), cloud, U0, tiles=True)
    s = _ctx(hcc, cfg("fp32"), cloud, U0, tiles=False)
    assert t.tile_staging()["active"]
    o = oracle.OracleContext(cfg("fp64"), abi)
    o.upload_cloud(cloud)
    o.build_neighbours()
    o.prepare_geometry()
    o.upload_state(U0)
    dt_t, dt_s, dt_o = t.time_step(), s.time_step(), o.time_step()
    assert np.isfinite(dt_t) and dt_t > 0
    assert abs(dt_t - dt_s) <= 1e-5 * dt_s, (dt_t, dt_s)
    assert abs(dt_t - dt_o) <= 1e-5 * dt_o, (dt_t, dt_o)
    dt = 0.4 * dt_o                                           # after steps (new states, lowered orders)
    for k in range(2):
        for c in (t, s, o):
            c.step(k * dt, dt)
    dt_t, dt_s, dt_o = t.time_step(), s.time_step(), o.time_step()
    assert abs(dt_t - dt_s) <= 1e-5 * dt_s and abs(dt_t - dt_o) <= 1e-5 * dt_o, (dt_t, dt_s, dt_o)
    for c in (t, s, o):
        c.close()
