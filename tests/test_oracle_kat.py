"""The oracle against the reference's own known-answer tests (test/unit_core.jl, test/unit_schemes.jl).

The reference ships no golden-vector files and cannot run here (Julia); these analytic, structural and cross-path
checks are what pins the CPU restatement to it. Each test names the reference test it ports.
"""
import math
import sys

import numpy as np
import pytest


@pytest.fixture(scope="module")
def abi(hcc):
    return sys.modules["hcc_gb300._abi"]


@pytest.fixture(scope="module")
def olib(oracle, abi):
    return oracle.load(abi)


def make(hcc, oracle, abi, cloud, pde, **kw):
    cfg = hcc.make_config(pde, cloud, **kw)
    o = oracle.OracleContext(cfg, abi)
    o.upload_cloud(cloud)
    o.build_neighbours()
    return o


def lattice_1d(hcc, N, rng=2.5):
    """make_pg_1d (test/runtests.jl:37-43): uniform periodic grid on [-1, 1] with N particles."""
    dx = 2.0 / N
    return hcc.rectangular_cloud((-1.0,), (1.0,), dx, rng * dx, periodic=True)


# ----------------------------------------------------------------------------------------------- basis tables
def test_basis_order_and_counts(olib):
    """_generate_exponents: index 1 is x, 2 is y, 3 is z; within a degree sorted by (-max, reverse)."""
    import ctypes as C
    ex = (C.c_int32 * 60)()
    B = olib.orc_basis_exponents(2, 2, ex)
    assert B == 5
    assert [tuple(ex[2 * k:2 * k + 2]) for k in range(B)] == [(1, 0), (0, 1), (2, 0), (0, 2), (1, 1)]
    B = olib.orc_basis_exponents(3, 2, ex)
    assert [tuple(ex[3 * k:3 * k + 3]) for k in range(B)] == [
        (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]
    for D in (1, 2, 3):
        for q in range(0, 5):
            assert olib.orc_basis_count(D, q) == (math.comb(D + q, q) - 1 if q > 0 else 0)


def test_divergence_degree_rules(olib):
    """unit_core.jl:401-419: _div_idx and _divergence_index."""
    assert olib.orc_div_idx(2, 1) == 2 and olib.orc_div_idx(2, 2) == 2
    assert olib.orc_div_idx(2, 3) == 4 and olib.orc_div_idx(2, 4) == 4
    assert olib.orc_div_idx(2, 5) == 6 and olib.orc_div_idx(3, 5) == 5
    assert olib.orc_divergence_index(0, 1, 3, 4) == 3
    assert olib.orc_divergence_index(0, 1, 3, 6) == 4
    assert olib.orc_divergence_index(3, 1, 1, 6) == 4
    assert olib.orc_divergence_index(0, 1, 4, 3) == 3


def test_ssp_coefficients(olib, abi):
    """unit_schemes.jl:203-213."""
    T = abi.TABLEAUS
    assert abs(olib.orc_ssp_coefficient(T["RK1_Euler"]) - 1) < 1e-9
    assert abs(olib.orc_ssp_coefficient(T["RK2_SSP"]) - 1) < 1e-9
    assert abs(olib.orc_ssp_coefficient(T["RK2_Ralston"]) - 0.5) < 1e-9
    assert abs(olib.orc_ssp_coefficient(T["RK3_SSP"]) - 1) < 1e-9
    assert abs(olib.orc_ssp_coefficient(T["RK4_SSP"]) - 1.50818004918983) < 1e-8
    assert olib.orc_ssp_coefficient(T["RK4_Classical"]) == 0
    assert olib.orc_ssp_coefficient(T["IMEX_ARS222"]) == 0


# ----------------------------------------------------------------------------------------------- grids / search
@pytest.mark.parametrize("D", [1, 2])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_jittered_periodic_grid_has_no_boundary(hcc, D, seed):
    """unit_core.jl:319-329: N = 20^D, no boundary particles, positions in [0, 1)."""
    cl = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, 0.05, 0.125, periodic=True, jitter=0.01, seed=seed)
    assert cl.n == 20 ** D and cl.is_boundary.sum() == 0
    assert np.all((cl.pos >= 0) & (cl.pos < 1))


@pytest.mark.parametrize("R", [0.45, 0.6])
def test_small_periodic_domains_do_not_duplicate(hcc, oracle, abi, R):
    """unit_core.jl:331-341: two and one coarse bins; no duplicates, no self, counts = brute force."""
    cl = hcc.rectangular_cloud((0.0,), (1.0,), 0.1, R, periodic=True)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)))
    counts, idx, _, _ = o.neighbours()
    x = o.positions()[:, 0]
    start = np.concatenate([[0], np.cumsum(counts)])
    for i in range(cl.n):
        lst = idx[start[i]:start[i + 1]]
        assert len(set(lst)) == len(lst) and i not in lst
        dd = x - x[i]
        brute = sum(1 for j in range(cl.n) if j != i and abs(dd[j] - np.round(dd[j])) <= R + 1e-12)
        assert counts[i] == brute


@pytest.mark.parametrize("D,periodic", [(2, False), (2, True), (3, False)])
def test_neighbour_lists_match_brute_force(hcc, oracle, abi, D, periodic):
    """Fixed-radius lists: every pair with r^2 <= R^2 (wrapped when periodic), j != i, in window order with
    descending indices within a bin (NeighborLogic.jl:153-167, :288-329)."""
    h = 0.1 if D == 2 else 0.2
    cl = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, periodic=periodic, jitter=0.25 * h, seed=9)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(tuple((1.0,) for _ in range(D))))
    counts, idx, w, dist = o.neighbours()
    pos = o.positions()
    L = np.array([1.0 if periodic else 0.0] * D)
    invL = np.array([1.0 if periodic else 0.0] * D)
    start = np.concatenate([[0], np.cumsum(counts)])
    R2 = (2.5 * h) ** 2
    for i in range(cl.n):
        d = pos - pos[i]
        d = d - L * np.round(d * invL)
        r2 = (d ** 2).sum(axis=1)
        expect = set(np.nonzero(r2 <= R2)[0]) - {i}
        got = idx[start[i]:start[i + 1]]
        assert set(got) == expect
        np.testing.assert_array_equal(dist[start[i]:start[i + 1]], d[got])
        y = (d[got] ** 2).sum(axis=1) / R2
        np.testing.assert_allclose(w[start[i]:start[i + 1]],
                                   1 / (1 + y * (1 + y * (0.5 + y * (1 / 6 + y / 24)))), rtol=1e-14)


@pytest.mark.parametrize("D,periodic", [(2, True), (3, False)])
def test_selected_lists_and_counts_equal_the_full_search(hcc, oracle, abi, D, periodic):
    """The oracle's per-particle lists (used on clouds too large to list whole) and its count pass equal the rows and
    counts of the full search (NeighborLogic.jl:288-329)."""
    h = 0.05 if D == 2 else 0.1
    cl = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, periodic=periodic, jitter=0.25 * h, seed=4)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(tuple((1.0,) for _ in range(D))))
    counts, idx, w, dist = o.neighbours()
    np.testing.assert_array_equal(o.neighbour_counts(), counts)
    start = np.concatenate([[0], np.cumsum(counts)])
    ids = np.random.default_rng(1).choice(cl.n, 50, replace=False)
    mx = int(counts.max())
    c2, i2, w2, d2 = o.neighbours_of(ids, mx)
    for q, i in enumerate(ids):
        c = counts[i]
        assert c2[q] == c
        np.testing.assert_array_equal(i2[q, :c], idx[start[i]:start[i + 1]])
        assert np.array_equal(w2[q, :c], w[start[i]:start[i + 1]])
        assert np.array_equal(d2[q, :c], dist[start[i]:start[i + 1]])
    with pytest.raises(Exception):
        o.neighbours_of(ids, int(counts[ids].max()) - 1)   # a row shorter than a count is refused


def test_morton_numbering_is_z_order(hcc):
    """Reordering.jl:55-102: the permutation sorts by interleaved 16-bit keys (2-D)."""
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), 0.05, 0.125, jitter=0.01, seed=4)
    kx = np.clip(np.floor((cl.pos[:, 0] - cl.canvas_min[0]) / (cl.canvas_max[0] - cl.canvas_min[0]) * 65535), 0, 65535)
    ky = np.clip(np.floor((cl.pos[:, 1] - cl.canvas_min[1]) / (cl.canvas_max[1] - cl.canvas_min[1]) * 65535), 0, 65535)

    def spread(v):
        out = 0
        for b in range(16):
            out |= ((int(v) >> b) & 1) << (2 * b)
        return out

    codes = [spread(a) | (spread(b) << 1) for a, b in zip(kx, ky)]
    assert all(codes[i] <= codes[i + 1] for i in range(len(codes) - 1))


def test_rectangle_tags_and_ghost_band(hcc):
    """Domains.jl:59-94, :268-270: face tags of the box, ghosts only within R + dx of an interior point."""
    h = 0.05
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=2)
    inner = cl.pos[cl.is_boundary == 0]
    ghosts = cl.pos[cl.is_boundary == 1]
    assert set(np.unique(cl.tags[cl.is_boundary == 1])) == {1, 2, 3, 4}
    x, y = ghosts[:, 0], ghosts[:, 1]
    t = cl.tags[cl.is_boundary == 1]
    assert np.all(x[t == 1] < 0) and np.all(x[t == 2] > 1) and np.all(y[t == 3] < 0) and np.all(y[t == 4] > 1)
    from scipy.spatial import cKDTree
    dmin, _ = cKDTree(inner).query(ghosts)
    assert np.all(dmin <= 2.5 * h + h + 1e-12)


# ----------------------------------------------------------------------------------------------- MLS
def test_mls_divergence_exact_for_linear_flux(hcc, oracle, abi, olib):
    """unit_core.jl:361-380: ΔF = ((1.5dx, -0.5dx + 2dy), (2dy, 3dy - dx)) -> divergence (3.5, 2.5), degrees 1..3."""
    import ctypes as C
    dx = 1 / 20
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), dx, 2.5 * dx, periodic=True)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0, 1.0), (1.0, 1.0))))
    counts, idx, w, dist = o.neighbours()
    start = np.concatenate([[0], np.cumsum(counts)])
    for i in (0, cl.n // 2):
        d = np.ascontiguousarray(dist[start[i]:start[i + 1]])
        wt = np.ascontiguousarray(w[start[i]:start[i + 1]])
        dF = np.stack([1.5 * d[:, 0], -0.5 * d[:, 0] + 2 * d[:, 1], 2.0 * d[:, 1], 3.0 * d[:, 1] - d[:, 0]], axis=1)
        dF = np.ascontiguousarray(dF)
        for q in (1, 2, 3):
            out = np.zeros(2)
            ok = olib.orc_mls_divergence(2, 2, q, len(wt), d.ctypes.data_as(C.POINTER(C.c_double)),
                                         wt.ctypes.data_as(C.POINTER(C.c_double)),
                                         dF.ctypes.data_as(C.POINTER(C.c_double)), dx,
                                         out.ctypes.data_as(C.POINTER(C.c_double)))
            assert ok
            np.testing.assert_allclose(out, [3.5, 2.5], atol=1e-8)


def test_constant_flux_has_zero_divergence(hcc, oracle, abi, olib):
    """unit_core.jl:392-400: the intercept fit gives zero divergence of a constant flux on any stencil."""
    import ctypes as C
    dx = 1 / 24
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), dx, 2.5 * dx, periodic=True, jitter=0.2 * dx, seed=3)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0, 1.0), (1.0, 1.0))))
    counts, idx, w, dist = o.neighbours()
    start = np.concatenate([[0], np.cumsum(counts)])
    for i in (0, cl.n // 2, cl.n - 1):
        d = np.ascontiguousarray(dist[start[i]:start[i + 1]])
        wt = np.ascontiguousarray(w[start[i]:start[i + 1]])
        dF = np.ascontiguousarray(np.tile([1.0, -2.0, 0.5, 3.0], (len(wt), 1)))
        for q in (1, 2, 3):
            out = np.zeros(2)
            olib.orc_mls_divergence(2, 2, q, len(wt), d.ctypes.data_as(C.POINTER(C.c_double)),
                                    wt.ctypes.data_as(C.POINTER(C.c_double)), dF.ctypes.data_as(C.POINTER(C.c_double)),
                                    dx, out.ctypes.data_as(C.POINTER(C.c_double)))
            assert np.abs(out).max() < 1e-9


def _basis(olib, D, q, x):
    import ctypes as C
    ex = (C.c_int32 * 64)()
    B = olib.orc_basis_exponents(D, q, ex)
    e = np.array(ex[:B * D]).reshape(B, D)
    fac = np.array([np.prod([math.factorial(int(t)) for t in row]) for row in e], dtype=float)
    return np.prod(x[None, :] ** e, axis=1) / fac


def test_conditional_regularisation(olib):
    """unit_core.jl:443-463: healthy stencils keep the plain factorisation; collinear ones get the retry and
    still the right x-derivative (within 100 sqrt(eps))."""
    import ctypes as C
    dists = np.array([[0.37 * np.cos(k), 0.37 * np.sin(k) + 0.1 * k] for k in range(1, 13)])
    wts = np.exp(-(dists ** 2).sum(axis=1))
    Nm = sum(w * np.outer(_basis(olib, 2, 2, d), _basis(olib, 2, 2, d)) for w, d in zip(wts, dists))
    Nm = np.ascontiguousarray(Nm)
    U = np.zeros_like(Nm)
    plain = C.c_int32()
    ok = olib.orc_cholesky_moment(5, Nm.ctypes.data_as(C.POINTER(C.c_double)), U.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.byref(plain))
    assert ok and plain.value == 1
    np.testing.assert_allclose(U.T @ U, Nm, rtol=1e-12, atol=1e-14)
    xd = np.array([[0.3 * k, 0.0] for k in range(-4, 5) if k != 0])
    xw = np.ones(len(xd))
    Nx = np.ascontiguousarray(sum(w * np.outer(_basis(olib, 2, 2, d), _basis(olib, 2, 2, d)) for w, d in zip(xw, xd)))
    ok = olib.orc_cholesky_moment(5, Nx.ctypes.data_as(C.POINTER(C.c_double)), U.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.byref(plain))
    assert ok and plain.value == 0
    f = np.ascontiguousarray((2 * xd[:, 0] + xd[:, 0] ** 2)[:, None])
    out = np.zeros(5)
    ok = olib.orc_mls_solve(2, 1, 2, len(xd), np.ascontiguousarray(xd).ctypes.data_as(C.POINTER(C.c_double)),
                            xw.ctypes.data_as(C.POINTER(C.c_double)), f.ctypes.data_as(C.POINTER(C.c_double)), 1.0,
                            out.ctypes.data_as(C.POINTER(C.c_double)))
    assert ok and np.all(np.isfinite(out))
    assert abs(out[0] - 2) < 100 * np.sqrt(np.finfo(float).eps) and abs(out[1]) < 100 * np.sqrt(np.finfo(float).eps)


def test_divergence_weights_are_face_vectors(hcc, oracle, abi):
    """dweights of the intercept fit (MUSCL.jl:197-223, unit_schemes.jl:429-460): Σ_j c_ij = 0 and
    Σ_j c_ij x_ij^T = I (the fit reproduces constants and linear functions)."""
    dx = 1 / 16
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), dx, 2.5 * dx, periodic=True, jitter=0.25 * dx, seed=5)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,), (1.0,))), scheme=hcc.MUSCL(3, 0))
    o.prepare_geometry()
    counts, idx, w, dist = o.neighbours()
    dw, okr, okd = o.geometry(len(idx))
    start = np.concatenate([[0], np.cumsum(counts)])
    assert okd.all()
    for i in range(0, cl.n, 7):
        c = dw[start[i]:start[i + 1]]
        x = dist[start[i]:start[i + 1]]
        np.testing.assert_allclose(c.sum(axis=0), 0, atol=1e-9 / dx)
        np.testing.assert_allclose(c.T @ x, np.eye(2), atol=1e-9)


def test_cached_fit_equals_direct_solve(hcc, oracle, abi, olib):
    """unit_core.jl:463-495: the cached inverse moment (apply_weights) equals the direct solve within 1e-9."""
    import ctypes as C
    dx = 1 / 24
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), dx, 2.5 * dx, periodic=True, jitter=0.2 * dx, seed=3)
    pde = hcc.LinearAdvection(((1.0, 0.5), (0.7, -0.3)))
    for order in (2, 3):
        o = make(hcc, oracle, abi, cl, pde, scheme=hcc.MUSCL(order, 0))
        x, y = cl.pos[:, 0], cl.pos[:, 1]
        U = np.stack([np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y), np.exp(-((x - .5) ** 2 + (y - .5) ** 2) / .05)], 1)
        o.upload_state(U)
        o.compute_rhs()
        g = o.gradients()
        counts, idx, w, dist = o.neighbours()
        start = np.concatenate([[0], np.cumsum(counts)])
        pos = o.positions()
        for i in (0, cl.n // 3, cl.n - 1):
            sl = slice(start[i], start[i + 1])
            df = np.ascontiguousarray(U[idx[sl]] - U[i])
            d = np.ascontiguousarray(dist[sl])
            wt = np.ascontiguousarray(w[sl])
            B = g.shape[1]
            out = np.zeros(B * 2)
            assert olib.orc_mls_solve(2, 2, order - 1, len(wt), d.ctypes.data_as(C.POINTER(C.c_double)),
                                      wt.ctypes.data_as(C.POINTER(C.c_double)), df.ctypes.data_as(C.POINTER(C.c_double)),
                                      dx, out.ctypes.data_as(C.POINTER(C.c_double)))
            np.testing.assert_allclose(g[i].ravel(), out, atol=1e-9 * max(1, np.abs(out).max()))
        assert pos.shape == (cl.n, 2)


# ----------------------------------------------------------------------------------------------- MOOD
@pytest.fixture(scope="module")
def mood_grid(hcc, oracle, abi):
    cl = lattice_1d(hcc, 40)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0),
             mood=hcc.MOOD(hcc.EPD1, hcc.OnlyMOOD()))
    return cl, o


def test_uniform_1d_grid_has_four_neighbours(mood_grid):
    """unit_core.jl:675-686: N = 40 (no duplicated seam point), R = 2.5dx -> ±1, ±2."""
    cl, o = mood_grid
    counts, _, _, _ = o.neighbours()
    assert cl.n == 40 and np.all(counts == 4)


def test_interface_orders(hcc, oracle, abi):
    """unit_core.jl:688-697: EPD0 (3,1); EPD1 (1,1) on the edge, (3,3) off it; EPD2 (1,1) through N(i)."""
    cl = lattice_1d(hcc, 40)
    x = cl.pos[:, 0]
    order_of_x = np.argsort(x)
    i = order_of_x[9]
    j = order_of_x[11]
    k = order_of_x[7]
    res = {}
    for name, strat in (("EPD0", hcc.EPD0), ("EPD1", hcc.EPD1), ("EPD2", hcc.EPD2)):
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0),
                 mood=hcc.MOOD(strat, hcc.OnlyMOOD()))
        orders = np.full(cl.n, 3, dtype=np.int32)
        orders[j] = 1
        o.set_orders(orders)
        res[name] = (o.interface_orders(i, j), o.interface_orders(i, k))
    assert res["EPD0"][0] == (3, 1)
    assert res["EPD1"][0] == (1, 1) and res["EPD1"][1] == (3, 3)
    assert res["EPD2"][1] == (1, 1)


def test_mask_expansion(mood_grid):
    """unit_core.jl:707-714: one hop adds the 4 neighbours, two hops 8."""
    cl, o = mood_grid
    mask = np.zeros(cl.n, dtype=np.uint8)
    mask[7] = 1
    assert o.expand_mask(mask, 1).sum() == 1 + 4
    assert o.expand_mask(mask, 2).sum() == 1 + 8


def test_detect_and_drop_terminates_at_order_one(hcc, oracle, abi):
    """unit_core.jl:748-764: OnlyMOOD 3 -> 2 -> 1, then nothing changes; an empty dirty mask checks nobody."""
    cl = lattice_1d(hcc, 40)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0),
             mood=hcc.MOOD(hcc.EPD1, hcc.OnlyMOOD()))
    U = np.zeros((cl.n, 1))
    o.set_orders(np.full(cl.n, 3))
    assert o.detect_and_drop(U, U, full=True) and np.all(o.orders() == 2)
    assert not o.detect_and_drop(U, U, full=False, dirty=np.zeros(cl.n, np.uint8))
    assert o.detect_and_drop(U, U, full=False, dirty=np.ones(cl.n, np.uint8)) and np.all(o.orders() == 1)
    assert not o.detect_and_drop(U, U, full=True) and np.all(o.orders() == 1)


def test_detect_and_drop_flags_inadmissible_candidates(hcc, oracle, abi):
    """unit_core.jl:766-779: a NaN candidate passes the DMP but fails PAD, only with the equation."""
    cl = lattice_1d(hcc, 40)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0),
             mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(0.0)))
    U = np.exp(-cl.pos[:, :1] ** 2 / 0.1)
    cand = U.copy()
    q = 5
    cand[q] = np.nan
    o.set_orders(np.full(cl.n, 3))
    assert not o.detect_and_drop(U, cand, full=True, with_eq=False)
    o.set_orders(np.full(cl.n, 3))
    assert o.detect_and_drop(U, cand, full=True, with_eq=True)
    orders = o.orders()
    assert orders[q] == 2 and (orders == 2).sum() == 1


# ----------------------------------------------------------------------------------------------- CFL
def test_cfl_equals_host_formula(hcc, oracle, abi):
    """unit_schemes.jl:496-510: get_time_step with cached weights equals the host sum (rtol 1e-12); Inf for zero
    speeds."""
    h = 0.05
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=8)
    o = make(hcc, oracle, abi, cl, hcc.Euler(2), scheme=hcc.MUSCL(2, 2))
    o.prepare_geometry()
    rng = np.random.default_rng(0)
    rho = 1 + 0.5 * rng.random(cl.n)
    u = rng.standard_normal((cl.n, 2)) * 0.3
    p = 1 + rng.random(cl.n)
    U = np.column_stack([rho, rho * u[:, 0], rho * u[:, 1], p / 0.4 + 0.5 * rho * (u ** 2).sum(1)])
    o.upload_state(U)
    counts, idx, w, dist = o.neighbours()
    dw, _, _ = o.geometry(len(idx))
    c = np.sqrt(1.4 * p / rho)
    lam = np.abs(u) + c[:, None]
    start = np.concatenate([[0], np.cumsum(counts)])
    best = np.inf
    for i in range(cl.n):
        if cl.is_boundary[i]:
            continue
        sl = slice(start[i], start[i + 1])
        s = (np.abs(dw[sl]) * np.maximum(lam[i][None, :], lam[idx[sl]])).sum()
        if s > np.finfo(float).tiny:
            best = min(best, 0.5 / s)
    assert o.time_step() == pytest.approx(best, rel=1e-12)
    o0 = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((0.0,), (0.0,))), scheme=hcc.MUSCL(2, 2))
    o0.upload_state(np.ones((cl.n, 1)))
    assert o0.time_step() == np.inf


# ----------------------------------------------------------------------------------------------- schemes
@pytest.mark.parametrize("drop", [False, True])
def test_streamed_equals_buffered(hcc, oracle, abi, drop):
    """unit_schemes.jl:398-427: streamed divergence = buffered fit within 1e-11 * scale (also with dropped orders)."""
    dx = 1 / 24
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), dx, 3.5 * dx, periodic=True, jitter=0.2 * dx, seed=21)
    pde = hcc.LinearAdvection(((1.0, 0.5), (0.7, -0.3)))
    x, y = cl.pos[:, 0], cl.pos[:, 1]
    U = np.stack([np.exp(-((x - .5) ** 2 + (y - .5) ** 2) / .05), np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)], 1)
    orders = np.full(cl.n, 3, dtype=np.int32)
    if drop:
        orders[np.abs(x - 0.5) < 0.1] = 2
    K = {}
    for streamed in (False, True):
        o = make(hcc, oracle, abi, cl, pde, scheme=hcc.MUSCL(3, 0))
        o.set_streamed(streamed)
        o.upload_state(U)
        K[streamed] = o.compute_rhs_orders(orders)
    scale = np.abs(K[False]).max()
    assert np.abs(K[False] - K[True]).max() < 1e-11 * scale


# ----------------------------------------------------------------------------------------------- boundary conditions
def _bc_grid(hcc, oracle, abi, bc_map):
    N = 60
    dx = 2.0 / N
    cl = hcc.rectangular_cloud((-1.0,), (1.0,), dx, 2.5 * dx)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0), bc_map=bc_map)
    x = cl.pos[:, 0]
    o.upload_state(x[:, None].copy())
    return cl, o, x


def test_dirichlet_restores_the_initial_state(hcc, oracle, abi):
    """unit_core.jl:525-533."""
    cl, o, x = _bc_grid(hcc, oracle, abi, {1: hcc.BC_DIRICHLET, 2: hcc.BC_DIRICHLET})
    buf = o.apply_bcs(np.full((cl.n, 1), 99.0))
    g = cl.is_boundary == 1
    assert g.any() and np.all(buf[g, 0] == x[g]) and np.all(buf[~g, 0] == 99.0)


def test_outflow_copies_the_nearest_resolved_donor(hcc, oracle, abi):
    """unit_core.jl:535-555: zero gradient, the outermost interior value."""
    cl, o, x = _bc_grid(hcc, oracle, abi, {1: hcc.BC_OUTFLOW, 2: hcc.BC_OUTFLOW})
    buf = o.apply_bcs(x[:, None].copy())
    inner = cl.is_boundary == 0
    lo, hi = x[inner].min(), x[inner].max()
    for i in np.nonzero(~inner)[0]:
        assert buf[i, 0] == (lo if x[i] < 0 else hi)


def test_dirichlet_left_outflow_right(hcc, oracle, abi):
    """unit_core.jl:557-573 (the Sod-tube map)."""
    cl, o, x = _bc_grid(hcc, oracle, abi, {1: hcc.BC_DIRICHLET, 2: hcc.BC_OUTFLOW})
    start = np.full((cl.n, 1), 99.0)
    inner = cl.is_boundary == 0
    start[inner, 0] = x[inner]
    buf = o.apply_bcs(start)
    hi = x[inner].max()
    for i in np.nonzero(~inner)[0]:
        assert buf[i, 0] == (x[i] if x[i] < 0 else hi)


# ----------------------------------------------------------------------------------------------- time stepper
def test_only_mood_drives_every_particle_to_order_one(hcc, oracle, abi):
    """unit_core.jl:930-936 (MUSCL of the highest order built here, RK2_SSP)."""
    cl = lattice_1d(hcc, 60)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0),
             mood=hcc.MOOD(hcc.EPD1, hcc.OnlyMOOD()), tableau="RK2_SSP")
    o.upload_state(np.exp(-cl.pos[:, :1] ** 2 / 0.02))
    o.step(0.0, 0.4 * 2 / 60)
    assert np.all(o.orders() == 1) and np.all(o.mood_flags() == 1)


@pytest.mark.parametrize("tab,mood", [("RK3_SSP", "none"), ("RK3_SSP", "u1"), ("IMEX_PRSSP3", "u1"),
                                      ("RK4_SSP", "u1"), ("RK2_Ralston", "pad")])
def test_steppers_run_and_stay_finite(hcc, oracle, abi, tab, mood):
    """unit_core.jl:905-928: explicit, IMEX and MOOD fixed points run, stay finite, keep the mass within 1e-2."""
    cl = lattice_1d(hcc, 60)
    crit = {"none": hcc.NoMOOD(), "u1": hcc.MOODu1(1e-4 * 2 / 60), "pad": hcc.MOODPAD()}[mood]
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0),
             mood=hcc.MOOD(hcc.EPD1, crit), tableau=tab)
    U0 = np.exp(-cl.pos[:, :1] ** 2 / 0.02)
    o.upload_state(U0)
    dt = 0.4 * 2 / 60
    for k in range(5):
        o.step(k * dt, dt)
    U = o.download_state()
    assert np.all(np.isfinite(U))
    assert abs(U.sum() - U0.sum()) <= 1e-2 * abs(U0.sum())
    assert np.all((o.orders() >= 1) & (o.orders() <= 3))


def test_maxwellian_initialisation_is_the_relaxation_fixed_point(hcc, oracle, abi):
    """set_initial_conditions! (test/kinetic_source.jl:110-131): the kinetic state built from macro moments u
    carries u as its moment, and a uniform one is left unchanged by an IMEX step of the oracle."""
    ring = [(math.cos(2 * math.pi * q / 16), math.sin(2 * math.pi * q / 16)) for q in range(16)]
    pde = hcc.KineticRelaxation(ring, epsilon=1e-4, macro_velocity=(1.0, 0.5))
    u = np.linspace(0.5, 1.5, 7)
    f = pde.maxwellian(u)
    np.testing.assert_allclose(f.sum(axis=1), u, rtol=1e-13)
    np.testing.assert_allclose(pde.maxwellian(f.sum(axis=1)), f, rtol=1e-12)
    h = 1 / 16
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=1, periodic=True)
    o = make(hcc, oracle, abi, cl, pde, scheme=hcc.MUSCL(2, 2),
             mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), tableau="IMEX_ARS222")
    o.prepare_geometry()
    U0 = pde.maxwellian(np.full(cl.n, 0.8))
    o.upload_state(U0)
    o.step(0.0, 0.4 * o.time_step())
    np.testing.assert_allclose(o.download_state(), U0, rtol=0, atol=1e-12)
    assert o.mood_flags().sum() == 0


def test_first_order_muscl_advances(hcc, oracle, abi):
    """unit_core.jl:938-945 (first half): MUSCL order 1 with forward Euler moves the solution."""
    cl = lattice_1d(hcc, 60)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(1, 0), tableau="RK1_Euler")
    U0 = np.exp(-cl.pos[:, :1] ** 2 / 0.02)
    o.upload_state(U0)
    o.step(0.0, 0.4 * 2 / 60)
    assert np.abs(o.download_state() - U0).max() > 1e-4


def test_advection_converges_to_the_analytic_solution(hcc, oracle, abi):
    """Linear advection against the characteristic solution (analytic_closure, test/PDEs/linear_advection.jl:61-128):
    MUSCL2 on a periodic cloud, error ratio between h and h/2 above 2.5 (second order: 4)."""
    errs = []
    for n in (40, 80):
        h = 1.0 / n
        cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True, jitter=0.1 * h, seed=3)
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,), (0.5,))), scheme=hcc.MUSCL(2, 2))
        f = lambda x, y: np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
        o.upload_state(f(cl.pos[:, 0], cl.pos[:, 1])[:, None])
        T = 0.1
        dt = 0.25 * o.time_step()
        steps = int(np.ceil(T / dt))
        dt = T / steps
        for k in range(steps):
            o.step(k * dt, dt)
        pos = o.positions()
        ex = f(pos[:, 0] - T, pos[:, 1] - 0.5 * T)
        errs.append(np.abs(o.download_state()[:, 0] - ex).mean())
    assert errs[0] / errs[1] > 2.5, errs


# ----------------------------------------------------------------------------------------------- limiters
def _box(x):
    return np.where(np.abs(x) < 0.3, 1.0, 0.0)


def test_limited_runs_are_scale_invariant_and_bounded(hcc, oracle, abi):
    """unit_schemes.jl:519-542: MUSCL3 + VK(:hard), a box scaled by 2^-50 gives bitwise scaled results, and the
    limited scheme stays within [0, 1]."""
    cl = lattice_1d(hcc, 60)

    def run(a):
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0, "vk_hard"),
                 tableau="RK2_SSP")
        o.upload_state(a * _box(cl.pos[:, :1]))
        dt = 0.4 * 2 / 60
        for k in range(10):
            o.step(k * dt, dt)
        return o.download_state()[:, 0]

    u1 = run(1.0)
    us = run(2.0 ** -50)
    assert np.array_equal(us, 2.0 ** -50 * u1)
    assert u1.min() >= -1e-12 and u1.max() <= 1 + 1e-12


@pytest.mark.parametrize("limiter", ["bj_soft", "vk_hard", "none"])
def test_limited_reconstructions_stay_in_local_bounds(hcc, oracle, abi, olib, limiter):
    """unit_schemes.jl:607-639: the midpoint reconstructions of limited MUSCL3 lie within the neighbourhood's
    [min, max] (<= 1e-12) for steps, kinks, peaks and ramps; unlimited, the box overshoots by more than 0.1."""
    cl = lattice_1d(hcc, 60)
    ics = [lambda x: 0.5 * (1 + np.tanh(x / 0.04)), _box, np.abs, lambda x: np.exp(-x ** 2 / 0.002),
           lambda x: np.where(x < 0, 0.0, np.where(x < 0.2, 5 * x, 0.5))]
    worst_box = None
    for n_ic, ic in enumerate(ics):
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0, limiter))
        U = ic(cl.pos[:, 0])[:, None]
        o.upload_state(U)
        o.compute_rhs()
        g = o.gradients()
        counts, idx, w, dist = o.neighbours()
        start = np.concatenate([[0], np.cumsum(counts)])
        worst = 0.0
        for i in range(cl.n):
            sl = slice(start[i], start[i + 1])
            vals = np.concatenate([U[idx[sl], 0], [U[i, 0]]])
            lo, hi = vals.min(), vals.max()
            for k in range(start[i], start[i + 1]):
                x = 0.5 * dist[k, 0]
                r = U[i, 0] + g[i, 0, 0] * x + g[i, 1, 0] * (0.5 * x * x)
                worst = max(worst, r - hi, lo - r)
        if limiter == "none":
            if n_ic == 1:
                worst_box = worst
        else:
            assert worst <= 1e-12, (n_ic, worst)
    if limiter == "none":
        assert worst_box > 0.1


# ----------------------------------------------------------------------------------------------- WENO
def test_weno_is_scale_invariant(hcc, oracle, abi):
    """unit_schemes.jl:519-542 (WENO2): a box scaled by 2^-50 gives bitwise scaled results."""
    cl = lattice_1d(hcc, 60)

    def run(a):
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.WENO(2), tableau="RK2_SSP")
        o.upload_state(a * _box(cl.pos[:, :1]))
        dt = 0.4 * 2 / 60
        for k in range(10):
            o.step(k * dt, dt)
        return o.download_state()[:, 0]

    u1 = run(1.0)
    us = run(2.0 ** -50)
    assert np.array_equal(us, 2.0 ** -50 * u1)
    assert np.all(np.isfinite(u1))


def test_weno_converges_on_smooth_advection(hcc, oracle, abi):
    """WENO2 (degree-2 fits) on a periodic 2-D cloud: the error against the characteristic solution falls by more
    than 2.5 when h halves."""
    errs = []
    for n in (24, 48):
        h = 1.0 / n
        cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True, jitter=0.1 * h, seed=5)
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,), (0.5,))), scheme=hcc.WENO(2))
        f = lambda x, y: np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
        o.upload_state(f(cl.pos[:, 0], cl.pos[:, 1])[:, None])
        T = 0.1
        dt = 0.2 * o.time_step()
        steps = int(np.ceil(T / dt))
        dt = T / steps
        for k in range(steps):
            o.step(k * dt, dt)
        pos = o.positions()
        errs.append(np.abs(o.download_state()[:, 0] - f(pos[:, 0] - T, pos[:, 1] - 0.5 * T)).mean())
    assert errs[0] / errs[1] > 2.5, errs


def test_weno_cfl_uses_the_assembled_fit(hcc, oracle, abi):
    """get_time_step without cached weights (_cfl_body!, ParticleGrids.jl:427-436): finite and positive, and the
    lattice value (1/D) / (Σ|c| λ) is reproduced by numpy from the same degree-2 fit."""
    cl = lattice_1d(hcc, 40)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((2.0,),)), scheme=hcc.WENO(2))
    o.upload_state(np.zeros((cl.n, 1)))
    dt = o.time_step()
    counts, idx, w, dist = o.neighbours()
    d = dist[:4, 0] / (2 / 40)
    P = np.stack([d, 0.5 * d * d], axis=1)
    Nm = (w[:4, None, None] * P[:, :, None] * P[:, None, :]).sum(0)
    c = np.abs((np.linalg.inv(Nm)[0] @ P.T) * w[:4] / (2 / 40))
    assert dt == pytest.approx(1.0 / (c.sum() * 2.0), rel=1e-12)


class _U2Lattice:
    """unit_core.jl:781-878: a 2-D periodic 20 x 20 lattice with hand-set states (M = 2) and curvature coefficients
    (the degree-2 terms D+1, D+2 of the cached reconstruction of MUSCL order 3); the criterion on its own."""

    def __init__(self, hcc, oracle, abi, crit):
        n = 20
        self.dx = dx = 1.0 / n
        self.cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), dx, 2.5 * dx, periodic=True)
        self.o = make(hcc, oracle, abi, self.cl, hcc.LinearAdvection(((1.0, 1.0), (0.0, 0.0))),
                      scheme=hcc.MUSCL(3, 2), mood=hcc.MOOD(hcc.EPD2, crit))
        self.N = self.cl.n
        counts, idx, _, _ = self.o.neighbours()
        self.start = np.concatenate([[0], np.cumsum(counts)])
        self.idx = idx
        self.orders = np.full(self.N, 3, dtype=np.int32)

    def nearest(self, c):
        return int(np.argmin(((self.cl.pos - np.asarray(c)) ** 2).sum(axis=1)))

    def set_fields(self, f1, d1, f2, d2):
        x = self.cl.pos
        self.U = np.stack([f1(x), f2(x)], axis=1)
        self.G = np.zeros((self.N, 5, 2))
        c1, c2 = d1(x), d2(x)
        self.G[:, 2, 0], self.G[:, 2, 1] = c1[0], c2[0]
        self.G[:, 3, 0], self.G[:, 3, 1] = c1[1], c2[1]

    def local_extrema(self, p, m):
        v = self.U[np.concatenate([[p], self.idx[self.start[p]:self.start[p + 1]]]), m]
        return v.min(), v.max()

    def flags(self, p, cand):
        return self.o.criterion_flags(p, self.U, self.G, self.orders, np.asarray(cand, dtype=np.float64))


@pytest.mark.parametrize("plateau", [0.0, 1e-3])
def test_mood_u2_smooth_minimum_next_to_an_inflection_line(hcc, oracle, abi, plateau):
    """unit_core.jl:815-833: an undershoot of a smooth minimum is accepted (one-signed, comparable curvature); the
    same undershoot of a component at its inflection line is rejected; below order 3 the plain DMP applies."""
    d = 1e-8
    L = _U2Lattice(hcc, oracle, abi, hcc.MOODu2(d, plateau=plateau))
    w, c0 = 0.1, (0.5, 0.5)
    gauss = lambda x: np.exp(-((x[:, 0] - c0[0]) ** 2 + (x[:, 1] - c0[1]) ** 2) / w)
    f1 = lambda x: 1 - 0.5 * gauss(x)
    d1 = lambda x: (-0.5 * gauss(x) * (4 * (x[:, 0] - c0[0]) ** 2 / w ** 2 - 2 / w),
                    -0.5 * gauss(x) * (4 * (x[:, 1] - c0[1]) ** 2 / w ** 2 - 2 / w))
    f2 = lambda x: np.sin(2 * np.pi * x[:, 0])
    d2 = lambda x: (-(2 * np.pi) ** 2 * np.sin(2 * np.pi * x[:, 0]), np.zeros(len(x)))
    L.set_fields(f1, d1, f2, d2)
    p = L.nearest(c0)
    lo1, _ = L.local_extrema(p, 0)
    cand = (lo1 - 10 * d, L.U[p, 1])
    assert not L.flags(p, cand)
    lo2, _ = L.local_extrema(p, 1)
    assert L.flags(p, (L.U[p, 0], lo2 - 10 * d))
    L.orders[p] = 2
    assert L.flags(p, cand)


def test_mood_u2_plateau(hcc, oracle, abi):
    """unit_core.jl:835-853: a ripple of amplitude 1e-6 (curvature changing sign) overshot by 5 delta is flagged
    without the plateau test and accepted with it (local range 2e-6 < 1e-3 x global range 0.5), also below order 3."""
    d = 1e-8
    c0, q = (0.5, 0.5), (0.1, 0.1)
    narrow = lambda x: np.exp(-((x[:, 0] - c0[0]) ** 2 + (x[:, 1] - c0[1]) ** 2) / 0.01)
    ripple = lambda x: 1e-6 * np.sin(20 * np.pi * x[:, 0] + 0.7)
    g1 = lambda x: 1 - 0.5 * narrow(x) + ripple(x)
    dg1 = lambda x: (-1e-6 * (20 * np.pi) ** 2 * np.sin(20 * np.pi * x[:, 0] + 0.7), np.zeros(len(x)))
    zero = lambda x: np.zeros(len(x))
    for plateau, expect in ((0.0, True), (1e-3, False)):
        L = _U2Lattice(hcc, oracle, abi, hcc.MOODu2(d, plateau=plateau))
        L.set_fields(g1, dg1, zero, lambda x: (zero(x), zero(x)))
        p = L.nearest(q)
        lo, hi = L.local_extrema(p, 0)
        assert hi - lo < 1e-5
        assert L.flags(p, (hi + 5 * d, 0.0)) == expect
        if plateau > 0:
            L.orders[p] = 1
            assert not L.flags(p, (hi + 5 * d, 0.0))


def test_mood_u2_jump_is_flagged(hcc, oracle, abi):
    """unit_core.jl:855-875: a jump with Gibbs-like curvature is flagged with or without the plateau test; at the
    corner of a jump (zero curvature next to it) only the magnitude test among the nearest neighbours sees it."""
    d = 1e-8
    dx = 1.0 / 20
    step = lambda x: np.where(x[:, 0] < 0.5, 0.0, 1.0)
    dstep = lambda x: (np.where(np.abs(x[:, 0] - 0.5) < 2.5 * dx, np.where(x[:, 0] < 0.5, 1 / dx ** 2, -1 / dx ** 2), 0.0),
                       np.zeros(len(x)))
    zero = lambda x: np.zeros(len(x))
    for crit in (dict(plateau=0.0), dict(), dict(plateau=1e-2)):
        L = _U2Lattice(hcc, oracle, abi, hcc.MOODu2(d, **crit))
        L.set_fields(step, dstep, zero, lambda x: (zero(x), zero(x)))
        p = L.nearest((0.5 - dx / 2, 0.5))
        _, hi = L.local_extrema(p, 0)
        assert L.flags(p, (hi + 1e-3, 0.0)), crit
    corner = lambda x: (np.where((0.5 <= x[:, 0]) & (x[:, 0] < 0.5 + dx / 2), -1 / dx ** 2, 0.0), np.zeros(len(x)))
    for ratio, expect in ((0.5, True), (0.0, False)):
        L = _U2Lattice(hcc, oracle, abi, hcc.MOODu2(d, ratio=ratio))
        L.set_fields(step, corner, zero, lambda x: (zero(x), zero(x)))
        p = L.nearest((0.5 + dx, 0.5))
        _, hi = L.local_extrema(p, 0)
        assert L.flags(p, (hi + 1e-3, 0.0)) == expect


def test_strict_epd0_forcing_uses_the_snapshot(hcc, oracle, abi):
    """unit_core.jl:719-746: StrictEPD0 lowers the neighbours of a dropped particle to its order from the
    post-decrement snapshot (one hop, no cascade); a neighbour that dropped itself is forced from the snapshot; the
    EPD strategies never force."""
    cl = lattice_1d(hcc, 40)
    U = np.zeros((cl.n, 1))
    for strategy, forces in ((hcc.STRICT_EPD0, True), (hcc.EPD2, False)):
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.MUSCL(3, 0),
                 mood=hcc.MOOD(strategy, hcc.OnlyMOOD()))
        counts, idx, _, _ = o.neighbours()
        start = np.concatenate([[0], np.cumsum(counts)])
        p = 20
        nbs = idx[start[p]:start[p + 1]]
        orders = np.full(cl.n, 3)
        orders[p] = 2                                    # p drops to 1 in this pass
        o.set_orders(orders)
        dirty = np.zeros(cl.n, np.uint8)
        dirty[p] = 1
        assert o.detect_and_drop(U, U, full=False, dirty=dirty)
        got = o.orders()
        assert got[p] == 1
        if forces:
            assert all(got[j] == 1 for j in nbs)
            assert got[(p + 3) % cl.n] == 3             # two hops away: untouched
        else:
            assert all(got[j] == 3 for j in nbs)
        if forces:
            # a neighbour that dropped itself (3 -> 2) is forced down to 1 from the snapshot
            q = nbs[0]
            orders = np.full(cl.n, 3)
            orders[p] = 2
            o.set_orders(orders)
            dirty[q] = 1
            assert o.detect_and_drop(U, U, full=False, dirty=dirty)
            got = o.orders()
            assert got[q] == 1 and got[p] == 1


# ----------------------------------------------------------------------------------------------- CentralDivergence
def test_central_divergence_exact_for_a_linear_flux(hcc, oracle, abi, olib):
    """unit_schemes.jl:356-373 (CentralDivergence on a jittered periodic 1-D cloud, R = 2.5 dx, F = u = x): the
    divergence is 1 away from the periodic seam, for every degree the order allows (orders 1-3 here), and the
    streamed per-slot form equals the direct fit of the same degree (orc_mls_divergence) to 1e-12."""
    dx = 2 / 40
    cl = hcc.rectangular_cloud((-1.0,), (1.0,), dx, 2.5 * dx, periodic=True, jitter=0.2 * dx, seed=1)
    inner = np.abs(cl.pos[:, 0]) < 0.7
    for order in (1, 2, 3):
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.CentralDivergence(order))
        o.prepare_geometry()
        o.upload_state(cl.pos[:, :1].copy())
        K = o.compute_rhs()[:, 0]
        assert np.max(np.abs(K[inner] + 1.0)) < 1e-10, order
    # streamed vs direct, degree 2 on a sine
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.CentralDivergence(2))
    o.prepare_geometry()
    u = np.sin(np.pi * cl.pos[:, 0])
    o.upload_state(u[:, None].copy())
    K = o.compute_rhs()[:, 0]
    counts, idx, w, dist = o.neighbours()
    start = np.concatenate([[0], np.cumsum(counts)])
    import ctypes as C
    for i in range(0, cl.n, 7):
        s0, s1 = start[i], start[i + 1]
        dists = np.ascontiguousarray(dist[s0:s1])
        ww = np.ascontiguousarray(w[s0:s1])
        dF = np.ascontiguousarray((u[idx[s0:s1]] - u[i])[:, None])
        out = np.zeros(1)
        dp = C.POINTER(C.c_double)
        ok = olib.orc_mls_divergence(1, 1, 2, s1 - s0, dists.ctypes.data_as(dp), ww.ctypes.data_as(dp),
                                     dF.ctypes.data_as(dp), dx, out.ctypes.data_as(dp))
        assert ok == 1
        assert abs(-K[i] - out[0]) <= 1e-12 * (1.0 + abs(out[0]))


def test_central_order_reach_and_cfl_degree(hcc, oracle, abi):
    """unit_core.jl:704-706: CentralDivergence has order reach 0 (MOOD recomputes only the changed particles) and
    divergence degree = its order (the CFL uses the assembled fit of that degree: degree 2 for Central2 equals
    WENO2's time step on the same cloud)."""
    cl = lattice_1d(hcc, 40)
    oc = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((2.0,),)), scheme=hcc.CentralDivergence(2))
    ow = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((2.0,),)), scheme=hcc.WENO(2))
    for o in (oc, ow):
        o.upload_state(np.zeros((cl.n, 1)))
    assert oc.time_step() == ow.time_step()
    # a single dropped particle recomputes only itself: OnlyMOOD drops everyone once per iteration, and with reach
    # 0 the fixed point still ends at order 1 everywhere
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.CentralDivergence(2),
             mood=hcc.MOOD(hcc.EPD1, hcc.OnlyMOOD()), tableau="RK2_SSP")
    o.upload_state(np.exp(-cl.pos[:, :1] ** 2 / 0.02))
    o.step(0.0, 0.01)
    assert np.all(o.orders()[cl.is_boundary == 0] == 1)


def test_central_converges_on_smooth_advection(hcc, oracle, abi):
    """Central2 (degree-2 divergence fit, RK3) on a periodic 2-D cloud: second-order convergence of a sine wave."""
    errs = []
    for n in (24, 48):
        h = 1.0 / n
        cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True, jitter=0.1 * h, seed=5)
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,), (0.5,))), scheme=hcc.CentralDivergence(2))
        f = lambda x, y: np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
        o.upload_state(f(cl.pos[:, 0], cl.pos[:, 1])[:, None])
        T = 0.1
        dt = 0.2 * o.time_step()
        steps = int(np.ceil(T / dt))
        dt = T / steps
        for k in range(steps):
            o.step(k * dt, dt)
        pos = o.positions()
        errs.append(np.abs(o.download_state()[:, 0] - f(pos[:, 0] - T, pos[:, 1] - 0.5 * T)).mean())
    assert errs[0] / errs[1] > 3.0, errs


# ----------------------------------------------------------------------------------------------- UpwindDivergence
@pytest.mark.parametrize("alg", ["Classic", "Tiwari", "Praveen"])
def test_2d_upwind_algorithms_converge_at_first_order(hcc, oracle, abi, alg):
    """pipeline_tests.jl:255-275: on the periodic [-1, 1]^2 cloud (50^2 and 100^2), advection with v = (1, 1) of a
    Gaussian to t = 0.1 with SSP-RK2 at CFL 0.4: the finer run is more accurate and the convergence order lies in
    (0.5, 1.5) for :Classic (first-order MUSCL), :Tiwari and :Praveen."""
    errs = []
    for n in (50, 100):
        h = 2.0 / n
        cl = hcc.rectangular_cloud((-1.0, -1.0), (1.0, 1.0), h, 2.5 * h, periodic=True)
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,), (1.0,))), scheme=hcc.Upwind(algorithm=alg),
                 tableau="RK2_SSP")
        f = lambda x, y: np.exp(-(x * x + y * y) / 0.1)
        o.upload_state(f(cl.pos[:, 0], cl.pos[:, 1])[:, None])
        T = 0.1
        dt = 0.4 * o.time_step()
        steps = int(np.ceil(T / dt))
        dt = T / steps
        for k in range(steps):
            o.step(k * dt, dt)
        x = cl.pos[:, 0] - T
        y = cl.pos[:, 1] - T
        x = x - 2.0 * np.round(x / 2.0)
        y = y - 2.0 * np.round(y / 2.0)
        ex = f(x, y)
        errs.append(np.sqrt(((o.download_state()[:, 0] - ex) ** 2).sum() / (ex ** 2).sum()))
    eoc = math.log(errs[0] / errs[1], 2)
    assert errs[1] < errs[0] and 0.5 < eoc < 1.5, (errs, eoc)


def test_tiwari_is_exact_for_a_linear_field(hcc, oracle, abi):
    """Tiwari: every axis with an upwind stencil fits a linear field exactly, so K = -(v . grad u) away from the
    periodic seam; Praveen is first order and only consistent (K -> -(v . grad u) as the cloud refines)."""
    h = 1 / 20
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True, jitter=0.2 * h, seed=2)
    inner = (np.abs(cl.pos - 0.5) < 0.3).all(axis=1)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,), (-0.5,))), scheme=hcc.Upwind(algorithm="Tiwari"))
    o.prepare_geometry()
    o.upload_state((2.0 * cl.pos[:, 0] + 3.0 * cl.pos[:, 1])[:, None].copy())
    K = o.compute_rhs()[:, 0]
    assert np.max(np.abs(K[inner] - (-(1.0 * 2.0 - 0.5 * 3.0)))) < 1e-10


def test_upwind_configuration_rules(hcc, oracle, abi):
    """Upwind.jl:70-86: :Tiwari / :Praveen are scalar and first order, :Praveen two-dimensional."""
    cl = lattice_1d(hcc, 20)
    with pytest.raises(Exception):
        make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=hcc.Upwind(algorithm="Praveen"))
    bad = hcc.Upwind(algorithm="Tiwari")
    bad.order = 2
    with pytest.raises(Exception):
        make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)), scheme=bad)


# ----------------------------------------------------------------------------------------------- moment correction
@pytest.mark.parametrize("D,jit,flux", [(1, 0.2, "aligned"), (1, 0.4, "rusanov"), (2, 0.2, "aligned"),
                                        (2, 0.4, "aligned"), (2, 0.2, "rusanov")])
def test_moment_correction_makes_first_order_consistent(hcc, oracle, abi, D, jit, flux):
    """unit_schemes.jl:127-168: the first-order scheme's response a_ij to a unit state at neighbour j has the first
    moment sum_j a_ij x_ij = -a (the advection velocity) only with the moment correction (< 1e-10; O(1e-2) off
    without it on a jittered periodic cloud); with AlignedRusanovFlux the coefficients stay non-negative."""
    n = 60 if D == 1 else 16
    dx = 1.0 / n
    cl = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, dx, 2.5 * dx, periodic=True, jitter=jit * dx, seed=4)
    a = (1.0,) if D == 1 else (1.0, -0.6)
    pde = hcc.LinearAdvection(tuple((v,) for v in a))

    def errors(moment):
        o = make(hcc, oracle, abi, cl, pde, scheme=hcc.MUSCL(1, 0, "none", flux, moment), tableau="RK2_SSP")
        o.prepare_geometry()
        counts, idx, _, dist = o.neighbours()
        start = np.concatenate([[0], np.cumsum(counts)])
        A = np.zeros((cl.n, cl.n))
        for j in range(cl.n):
            e = np.zeros((cl.n, 1))
            e[j] = 1.0
            o.upload_state(e)
            A[:, j] = o.compute_rhs()[:, 0]
        errs, amin = [], np.inf
        for i in range(0, cl.n, 1 if D == 1 else 3):
            sl = slice(start[i], start[i + 1])
            aij = A[i, idx[sl]]
            v = (aij[:, None] * dist[sl]).sum(axis=0)
            errs.append(np.max(np.abs(v + np.array(a))))
            amin = min(amin, aij.min())
        return max(errs), amin

    e0, _ = errors(False)
    e1, amin = errors(True)
    assert e0 > 1e-2
    assert e1 < 1e-10
    if flux == "aligned":
        assert amin >= -1e-12


def test_moment_correction_is_ignored_above_order_one(hcc, oracle, abi):
    """unit_schemes.jl:186-196: second-order MUSCL with moment_correction gives bitwise the same right-hand side."""
    cl = lattice_1d(hcc, 30)
    u = np.sin(np.pi * cl.pos[:, :1])
    out = []
    for moment in (True, False):
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,),)),
                 scheme=hcc.MUSCL(2, 0, "none", "aligned", moment))
        o.prepare_geometry()
        o.upload_state(u.copy())
        out.append(o.compute_rhs())
    assert np.array_equal(out[0], out[1])


# ----------------------------------------------------------------------------------------------- ShepardVolumes
def test_shepard_volumes_exact_on_a_uniform_periodic_lattice(hcc, oracle, abi):
    """Volumes.jl:36-50: ShepardVolumes is exact (V_i = dx^D) on a uniform periodic lattice, for any sweeps."""
    for D, n in ((1, 40), (2, 20)):
        h = 1.0 / n
        cl = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, periodic=True)
        o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(tuple((1.0,) for _ in range(D))))
        for sweeps in (0, 1, 3):
            o.update_volumes(sweeps)
            np.testing.assert_allclose(o.volumes(), h ** D, rtol=1e-13)


def test_shepard_volumes_partition_the_box(hcc, oracle, abi):
    """On a jittered bounded box: positive volumes summing to the box volume, the same for every sweep count, and
    close to dx^D inside (the partition-of-unity sweeps smooth the kernel-density estimate)."""
    h = 1 / 24
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.3 * h, seed=8)
    o = make(hcc, oracle, abi, cl, hcc.LinearAdvection(((1.0,), (1.0,))))
    inner = (np.abs(cl.pos - 0.5) < 0.35).all(axis=1)
    for sweeps in (0, 1, 2):
        o.update_volumes(sweeps)
        V = o.volumes()
        assert np.all(V >= 0.0)
        assert V.sum() == pytest.approx(1.0, rel=1e-13)
        assert np.abs(V[inner] / h ** 2 - 1.0).max() < 0.5


# ----------------------------------------------------------------------------------------------- WENO for systems
def _weno_oracle(hcc, oracle, abi, cloud, pde, order=2, **kw):
    o = oracle.OracleContext(hcc.make_config(pde, cloud, scheme=hcc.WENO(order), **kw), abi)
    o.upload_cloud(cloud)
    o.build_neighbours()
    o.prepare_geometry()
    return o


@pytest.mark.parametrize("order", [1, 2])
def test_weno_system_reduces_to_the_scalar_scheme(hcc, oracle, abi, order):
    """Component-wise WENO of a two-component advection system: each component's right-hand side equals the scalar
    WENO scheme's (WENO.jl:55-165) for that component and its velocity, bit for bit."""
    h = 0.05
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True, jitter=0.2 * h, seed=3)
    x, y = cl.pos[:, 0], cl.pos[:, 1]
    u0 = np.where((x - 0.5) ** 2 + (y - 0.5) ** 2 < 0.05, 1.0, 0.1) + 0.05 * np.sin(2 * np.pi * x)
    u1 = np.exp(-((x - 0.3) ** 2 + (y - 0.6) ** 2) / 0.02)
    vel = ((1.0, -0.4), (0.5, 0.7))                    # c[d][m]
    sys_ = _weno_oracle(hcc, oracle, abi, cl, hcc.LinearAdvection(vel), order)
    sys_.upload_state(np.stack([u0, u1], axis=1))
    K = sys_.compute_rhs()
    for m, u in enumerate((u0, u1)):
        sc = _weno_oracle(hcc, oracle, abi, cl, hcc.LinearAdvection(((vel[0][m],), (vel[1][m],))), order)
        sc.upload_state(u[:, None].copy())
        assert np.array_equal(K[:, m].view(np.uint64), sc.compute_rhs()[:, 0].view(np.uint64)), m


def test_weno_euler_converges_on_a_smooth_wave(hcc, oracle, abi):
    """Euler WENO (local Lax-Friedrichs splitting, component-wise fits): a density wave carried by a uniform flow at
    uniform pressure converges to the exact solution at second order (errors ratio >= 2.8 for halved spacing; measured
    1.06e-2 -> 2.26e-3 mean absolute density error at h = 1/16 -> 1/32)."""
    errs = []
    for h in (1.0 / 16, 1.0 / 32):
        cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True, jitter=0.1 * h, seed=5)
        x, y = cl.pos[:, 0], cl.pos[:, 1]
        u, v, p = 1.0, 0.5, 1.0
        rho = 1.0 + 0.2 * np.sin(2 * np.pi * (x + y))
        U0 = np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)], axis=1)
        o = _weno_oracle(hcc, oracle, abi, cl, hcc.Euler(2), 2, mood=hcc.MOOD(hcc.EPD1, hcc.MOODPAD()))
        o.upload_state(U0)
        t_end = 0.1
        n = int(np.ceil(t_end / (0.3 * o.time_step())))
        dt = t_end / n
        for k in range(n):
            o.step(k * dt, dt)
        exact = 1.0 + 0.2 * np.sin(2 * np.pi * ((x - u * t_end) + (y - v * t_end)))
        errs.append(np.abs(o.download_state()[:, 0] - exact).mean())
        o.close()
    assert errs[1] < errs[0] / 2.8, errs
