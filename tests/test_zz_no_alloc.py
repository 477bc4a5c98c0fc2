"""hcc_cfl_time_step_noalloc: the CFL step of caller-owned device arrays, computed without any device allocation.

It serves callers that cannot allocate GPU memory when they need a time step (device memory reserved up front and
frozen, or routed through the caller's own pool with cudaMalloc/cudaFree forbidden in the time loop). The tests
hand it device arrays that the test itself owns and compare its result with hcc_time_step, the entry point that
uses the context's own scratch: two calls in a row (a large cloud, then a smaller one, so the second call runs over
scratch words the first one left behind), every physics shape family it instantiates (2-D and 3-D Euler, scalar
advection, the 16-velocity kinetic model), the default stream and a caller-created stream. Both entry points
evaluate the same FP64 arithmetic: the results must be equal. A warm call must leave the device's free memory
unchanged.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import blast_ic, quadrant_ic

pytestmark = pytest.mark.gpu


def _slot_major(counts, idx, dw, n, D):
    npad = ((n + 31) // 32) * 32
    kmax = int(counts.max())
    nidx = np.zeros((kmax, npad), dtype=np.int32)
    dws = np.zeros((kmax, D, npad), dtype=np.float64)
    start = np.concatenate([[0], np.cumsum(counts)])
    for i in range(n):
        c = counts[i]
        nidx[:c, i] = idx[start[i]:start[i + 1]]
        dws[:c, :, i] = dw[start[i]:start[i + 1]]
    return npad, nidx, dws


def _system(hcc, kind, cloud, h):
    D = cloud.dim
    mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h ** D))
    outflow = {t: hcc.BC_OUTFLOW for t in range(1, 2 * D + 1)}
    x = cloud.pos
    if kind == "euler":
        cfg = hcc.make_config(hcc.Euler(D), cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=outflow)
        U = quadrant_ic(cloud) if D == 2 else blast_ic(cloud)
    elif kind == "advection":
        pde = hcc.LinearAdvection(tuple((v,) for v in (1.0, -0.5, 0.25)[:D]))
        cfg = hcc.make_config(pde, cloud, scheme=hcc.MUSCL(2, 2), mood=mood, bc_map=outflow)
        U = np.exp(-((x - 0.4) ** 2).sum(axis=1) / 0.01)[:, None].copy()
    else:
        ring = tuple((float(np.cos(2 * np.pi * q / 16)), float(np.sin(2 * np.pi * q / 16))) for q in range(16))
        pde = hcc.KineticRelaxation(ring, epsilon=1e-4, macro_velocity=(1.0, 0.5))
        cfg = hcc.make_config(pde, cloud, scheme=hcc.MUSCL(2, 2), mood=mood, tableau="IMEX_ARS222",
                              bc_map=outflow)
        rho = 1.0 + 0.2 * np.sin(2 * np.pi * x[:, 0]) * np.cos(2 * np.pi * x[:, 1])
        U = pde.maxwellian(rho)
    return cfg, np.ascontiguousarray(U, dtype=np.float64)


def _case(hcc, kind, D, h, seed):
    import torch
    cloud = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, jitter=0.25 * h, seed=seed)
    cfg, U = _system(hcc, kind, cloud, h)
    ctx = hcc.Context(cfg)
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.upload_state(U)
    dt_ref = ctx.time_step()                               # the existing entry point
    counts, idx, _, _ = ctx.neighbours()
    dw, _, _ = ctx.geometry(int(counts.sum()))
    npad, nidx, dws = _slot_major(counts, idx, dw, cloud.n, D)
    dev = {                                                 # caller-owned device arrays
        "counts": torch.from_numpy(np.ascontiguousarray(counts)).cuda(),
        "nidx": torch.from_numpy(np.ascontiguousarray(nidx)).cuda(),
        "dw": torch.from_numpy(np.ascontiguousarray(dws)).cuda(),
        "bnd": torch.from_numpy(np.ascontiguousarray(cloud.is_boundary)).cuda(),
        "U": torch.from_numpy(U).cuda(),
    }
    torch.cuda.synchronize()
    ctx.close()
    return cfg, cloud.n, npad, dev, dt_ref


def _noalloc(lib, cfg, n, npad, dev, stream=None):
    dt = C.c_double(-1.0)
    st = lib.hcc_cfl_time_step_noalloc(C.byref(cfg), n, npad, dev["counts"].data_ptr(), dev["nidx"].data_ptr(),
                                       dev["dw"].data_ptr(), dev["bnd"].data_ptr(), dev["U"].data_ptr(), stream,
                                       C.byref(dt))
    return st, dt.value


def test_noalloc_time_step_matches_the_context_entry_point(hcc, cuda_lib):
    pytest.importorskip("torch")
    big = _case(hcc, "euler", 2, 0.01, seed=3)
    small = _case(hcc, "euler", 2, 0.025, seed=4)
    for cfg, n, npad, dev, dt_ref in (big, small):        # two calls in a row
        st, dt = _noalloc(cuda_lib, cfg, n, npad, dev)
        assert st == 0
        assert np.isfinite(dt) and dt == dt_ref


@pytest.mark.parametrize("kind,D,h", [("euler", 3, 1.0 / 14), ("advection", 2, 0.02), ("advection", 3, 1.0 / 14),
                                      ("bgk", 2, 0.03)])
def test_noalloc_every_shape_family_on_a_caller_stream(hcc, cuda_lib, kind, D, h):
    torch = pytest.importorskip("torch")
    cfg, n, npad, dev, dt_ref = _case(hcc, kind, D, h, seed=9)
    stream = torch.cuda.Stream()
    for s in (None, C.c_void_p(stream.cuda_stream)):      # default stream, then the caller's own stream
        st, dt = _noalloc(cuda_lib, cfg, n, npad, dev, s)
        assert st == 0
        assert np.isfinite(dt) and dt == dt_ref


def test_noalloc_warm_call_allocates_nothing(hcc, cuda_lib):
    torch = pytest.importorskip("torch")
    cfg, n, npad, dev, dt_ref = _case(hcc, "euler", 2, 0.02, seed=5)
    st, _ = _noalloc(cuda_lib, cfg, n, npad, dev)          # the first call on this device loads the module
    assert st == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        st, dt = _noalloc(cuda_lib, cfg, n, npad, dev)
        assert st == 0 and dt == dt_ref
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_scratch(hcc, cuda_lib):
    cfg = hcc.config_defaults()
    cfg.dim, cfg.n_vars, cfg.pde = 2, 4, 1
    too_many = hcc._abi.HCC_NOALLOC_MAX_PARTICLES + 1
    dt = C.c_double(0.0)
    dummy = C.c_void_p(1)          # never dereferenced: the size check comes first
    st = cuda_lib.hcc_cfl_time_step_noalloc(C.byref(cfg), too_many, too_many, dummy, dummy, dummy, dummy, dummy, None,
                                            C.byref(dt))
    assert st == hcc._abi.HCC_ERR_CAPACITY
