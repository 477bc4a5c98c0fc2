"""GPU: launch shapes (hcc_set_tuning) and the autotuner (hcc_autotune).

The shapes change no result: states, orders and MOOD flags after several steps are bit-identical across flux /
gather block sizes and worklist / decision grids (FP64 and FP32, MUSCL with MOOD, WENO). The autotuner returns a
valid configuration, leaves the state and counters as they were, and the next step equals the step of an untuned
context bit for bit.
"""
import numpy as np
import pytest

from conftest import gaussian_ic, quadrant_ic

pytestmark = pytest.mark.gpu

OUTFLOW = {t: 2 for t in range(1, 5)}
ODD = dict(flux_block=64, gather_block=96, list_blocks_per_sm=2, drop_blocks_per_sm=1)


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


def _euler_ctx(hcc, precision, h=1 / 96):
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=5)
    cfg = hcc.make_config(hcc.Euler(2, 1.4), cl, scheme=hcc.MUSCL(2, 2),
                          mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), bc_map=OUTFLOW, precision=precision)
    g = hcc.Context(cfg)
    g.upload_cloud(cl)
    g.build_neighbours()
    g.prepare_geometry()
    U0 = quadrant_ic(cl)
    return g, (U0.astype(np.float32) if precision == "fp32" else U0)


def _run(g, U0, dt, steps):
    g.upload_state(U0)
    for k in range(steps):
        g.step(k * dt, dt)
    return g.download_state(), g.orders(), g.mood_flags()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("graphs", [True, False])
def test_launch_shapes_do_not_change_results(hcc, cuda_lib, precision, graphs):
    g, U0 = _euler_ctx(hcc, precision)
    g.set_step_graphs(graphs)
    g.upload_state(U0)
    dt = 0.4 * g.time_step()
    assert g.tuning() == dict(flux_block=128, gather_block=128, list_blocks_per_sm=8, drop_blocks_per_sm=2)
    U1, o1, f1 = _run(g, U0, dt, 4)
    assert f1.sum() > 0
    g.set_tuning(**ODD)
    assert g.tuning() == ODD
    U2, o2, f2 = _run(g, U0, dt, 4)
    assert np.array_equal(_bits(U1), _bits(U2))
    np.testing.assert_array_equal(o1, o2)
    np.testing.assert_array_equal(f1, f2)
    g.set_tuning(flux_block=32, gather_block=32, list_blocks_per_sm=32, drop_blocks_per_sm=32)
    U3, _, f3 = _run(g, U0, dt, 4)
    assert np.array_equal(_bits(U1), _bits(U3))
    np.testing.assert_array_equal(f1, f3)


def test_weno_full_pass_shapes(hcc, cuda_lib):
    h = 1 / 80
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 3.5 * h, jitter=0.25 * h, seed=9, periodic=True)
    cfg = hcc.make_config(hcc.LinearAdvection(((1.0,), (0.5,))), cl, scheme=hcc.WENO(2),
                          mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)))
    g = hcc.Context(cfg)
    g.upload_cloud(cl)
    g.build_neighbours()
    g.prepare_geometry()
    U0 = gaussian_ic(cl)
    g.upload_state(U0)
    dt = 0.4 * g.time_step()
    U1, _, _ = _run(g, U0, dt, 3)
    g.set_tuning(flux_block=96)
    U2, _, _ = _run(g, U0, dt, 3)
    assert np.array_equal(_bits(U1), _bits(U2))


def test_set_tuning_rejects_out_of_range(hcc, cuda_lib):
    g, _ = _euler_ctx(hcc, "fp64", h=1 / 32)
    for bad in (dict(flux_block=100), dict(flux_block=256), dict(gather_block=0), dict(list_blocks_per_sm=0),
                dict(drop_blocks_per_sm=33)):
        with pytest.raises(hcc.HCCError):
            g.set_tuning(**bad)
    assert g.tuning()["flux_block"] == 128


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_autotune_restores_the_state_and_keeps_results(hcc, cuda_lib, precision):
    g, U0 = _euler_ctx(hcc, precision)
    g.upload_state(U0)
    dt = 0.4 * g.time_step()
    g.step(0.0, dt)                       # a state that is not the upload, and a last step to restore
    Ua, oa, fa = g.download_state(), g.orders(), g.mood_flags()
    c0 = g.counters()
    rep = g.autotune(dt, steps=2)
    assert rep["candidates"] >= 9 and rep["steps"] == 2
    assert rep["best_ms"] > 0 and rep["best_ms"] <= rep["default_ms"]
    assert g.tuning() == rep["best"]
    assert np.array_equal(_bits(g.download_state()), _bits(Ua))
    np.testing.assert_array_equal(g.orders(), oa)
    np.testing.assert_array_equal(g.mood_flags(), fa)
    c1 = g.counters()
    assert c1["steps"] == c0["steps"] and c1["kernel_launches_total"] == c0["kernel_launches_total"]
    g.step(dt, dt)
    # an untuned context over the same two steps
    h, _ = _euler_ctx(hcc, precision)
    h.upload_state(U0)
    h.step(0.0, dt)
    h.step(dt, dt)
    assert np.array_equal(_bits(g.download_state()), _bits(h.download_state()))
    np.testing.assert_array_equal(g.mood_flags(), h.mood_flags())


def test_autotune_refuses_a_moving_grid(hcc, cuda_lib):
    g, U0 = _euler_ctx(hcc, "fp64", h=1 / 32)
    g.upload_state(U0)
    g.set_mover(hcc.mover("lagrangian"))
    with pytest.raises(hcc.HCCError):
        g.autotune(1e-4, steps=1)


def test_autotune_with_the_predictor_keeps_the_next_steps(hcc, cuda_lib):
    """With the shipped predictor attached the tuner also puts back the rough-tile marks that steer the next
    step's feature pass: three steps after tuning equal three steps of an untuned context bit for bit."""
    import sys
    L = sys.modules["hcc_gb300.learned"]
    pred = hcc.TroubledPointPredictor(capacity=16)
    pred.load(L.default_weights_path())
    h = 1 / 128
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=42)
    U0 = L.voronoi_state(cl.pos, 77).astype(np.float32)

    def ctx():
        cfg = hcc.make_config(hcc.Euler(2, 1.4), cl, scheme=hcc.MUSCL(2, 2),
                              mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), bc_map=OUTFLOW, precision="fp32")
        g = hcc.Context(cfg)
        g.upload_cloud(cl)
        g.build_neighbours()
        g.prepare_geometry()
        g.set_predictor(pred, 0.7)
        g.upload_state(U0)
        return g

    g, r = ctx(), ctx()
    dt = 0.4 * g.time_step()
    for c in (g, r):
        c.step(0.0, dt)                  # leaves rough-tile marks behind
    g.autotune(dt, steps=2)
    g.set_tuning(**ODD)                  # and other shapes than the reference context's
    pg = pr = 0
    for k in range(3):
        g.step((k + 1) * dt, dt)
        r.step((k + 1) * dt, dt)
        pg += g.counters()["predicted"]
        pr += r.counters()["predicted"]
    assert pr > 0 and pg == pr
    assert np.array_equal(_bits(g.download_state()), _bits(r.download_state()))
    np.testing.assert_array_equal(g.mood_flags(), r.mood_flags())
