"""hcc_cfl_time_step_noalloc: the CFL step of caller-owned device arrays, computed without any device allocation.

It serves callers that cannot allocate GPU memory when they need a time step (device memory reserved up front and
frozen, or routed through the caller's own pool with cudaMalloc/cudaFree forbidden in the time loop). The test
hands it device arrays that the test itself owns and compares its result with hcc_time_step, the entry point that
uses the context's own scratch, on two calls in a row (a large cloud, then a smaller one, so the second call runs
over scratch words the first one left behind). Both evaluate the same FP64 arithmetic: the results must be equal.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import quadrant_ic

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


def _case(hcc, h, seed):
    import torch
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=seed)
    cfg = hcc.make_config(hcc.Euler(2), cloud, scheme=hcc.MUSCL(2, 2),
                          mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)),
                          bc_map={t: hcc.BC_OUTFLOW for t in (1, 2, 3, 4)})
    ctx = hcc.Context(cfg)
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    U = quadrant_ic(cloud)
    ctx.upload_state(U)
    dt_ref = ctx.time_step()                               # the existing entry point
    counts, idx, _, _ = ctx.neighbours()
    dw, _, _ = ctx.geometry(int(counts.sum()))
    npad, nidx, dws = _slot_major(counts, idx, dw, cloud.n, 2)
    dev = {                                                 # caller-owned device arrays
        "counts": torch.from_numpy(np.ascontiguousarray(counts)).cuda(),
        "nidx": torch.from_numpy(np.ascontiguousarray(nidx)).cuda(),
        "dw": torch.from_numpy(np.ascontiguousarray(dws)).cuda(),
        "bnd": torch.from_numpy(np.ascontiguousarray(cloud.is_boundary)).cuda(),
        "U": torch.from_numpy(np.ascontiguousarray(U)).cuda(),
    }
    torch.cuda.synchronize()
    ctx.close()
    return cfg, cloud.n, npad, dev, dt_ref


def _noalloc(lib, cfg, n, npad, dev):
    dt = C.c_double(-1.0)
    st = lib.hcc_cfl_time_step_noalloc(C.byref(cfg), n, npad, dev["counts"].data_ptr(), dev["nidx"].data_ptr(),
                                       dev["dw"].data_ptr(), dev["bnd"].data_ptr(), dev["U"].data_ptr(), None,
                                       C.byref(dt))
    return st, dt.value


def test_noalloc_time_step_matches_the_context_entry_point(hcc, cuda_lib):
    pytest.importorskip("torch")
    big = _case(hcc, 0.01, seed=3)
    small = _case(hcc, 0.025, seed=4)
    for cfg, n, npad, dev, dt_ref in (big, small):        # two calls in a row
        st, dt = _noalloc(cuda_lib, cfg, n, npad, dev)
        assert st == 0
        assert np.isfinite(dt) and dt == dt_ref


def test_noalloc_rejects_sizes_beyond_its_scratch(hcc, cuda_lib):
    cfg = hcc.config_defaults()
    cfg.dim, cfg.n_vars, cfg.pde = 2, 4, 1
    too_many = hcc._abi.HCC_NOALLOC_MAX_PARTICLES + 1
    dt = C.c_double(0.0)
    dummy = C.c_void_p(1)          # never dereferenced: the size check comes first
    st = cuda_lib.hcc_cfl_time_step_noalloc(C.byref(cfg), too_many, too_many, dummy, dummy, dummy, dummy, dummy, None,
                                            C.byref(dt))
    assert st == hcc._abi.HCC_ERR_CAPACITY
