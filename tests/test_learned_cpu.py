"""CPU checks of the learned troubled-point predictor's oracle and host side (no GPU).

The numpy restatement of the network (oracle/mlp.py) is pinned by finite differences of its FP64 form; its BF16
rounding by known values; the C++ stencil features (oracle/hcc_oracle.cpp) by fields with known answers.
"""
import ctypes as C
import importlib.util
import sys

import numpy as np
import pytest

from conftest import ROOT


def _mlp_oracle():
    if "hcc_oracle_mlp" in sys.modules:
        return sys.modules["hcc_oracle_mlp"]
    spec = importlib.util.spec_from_file_location("hcc_oracle_mlp", ROOT / "oracle" / "mlp.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["hcc_oracle_mlp"] = mod
    spec.loader.exec_module(mod)
    return mod


def test_bf16_rounding_known_values():
    m = _mlp_oracle()
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125 + 2.0 ** -8, 3.14159, -2.5e-3, 0.0, -0.0, 65504.0,
                  np.inf, 2.0 ** -133], dtype=np.float32)
    want = np.array([1.0, 1.0, 1.0078125, 1.015625, 3.140625, -0.00250244140625, 0.0, -0.0, 65536.0, np.inf,
                     2.0 ** -133], dtype=np.float32)
    np.testing.assert_array_equal(m.bf16(x), want)   # ties to even: 1 + 2^-8 -> 1, 1 + 2^-7 + 2^-8 -> 1 + 2^-6
    assert np.isnan(m.bf16(np.array([np.nan], dtype=np.float32)))[0]


def test_oracle_gradient_matches_finite_differences():
    m = _mlp_oracle()
    rng = np.random.default_rng(0)
    p = rng.normal(0.0, 0.3, m.NPARAMS)
    norm = np.concatenate([rng.normal(0.0, 0.1, 24), rng.uniform(0.5, 2.0, 24)]).astype(np.float32)
    X = rng.normal(0.0, 1.0, (40, 24)).astype(np.float32)
    y = rng.random(40) < 0.3
    _, g = m.loss_grad(p, norm, X, y, 2.0, exact=True)
    idx = [0, 5, m.OFF_B1, m.OFF_W2, m.OFF_W2 + 100, 4000, m.OFF_B2, m.OFF_W3 + 3, m.OFF_B3, 100]
    for k in idx:
        e = 1e-6
        a, b = p.copy(), p.copy()
        a[k] += e
        b[k] -= e
        fd = (m.loss_grad(a, norm, X, y, 2.0, exact=True)[0] - m.loss_grad(b, norm, X, y, 2.0, exact=True)[0]) / (2 * e)
        assert abs(fd - g[k]) <= 1e-6 * (1.0 + abs(g[k])), (k, fd, g[k])


def test_rounded_network_stays_close_to_exact():
    """The BF16 rounding points perturb logits by O(2^-8) relative, not more."""
    m = _mlp_oracle()
    rng = np.random.default_rng(1)
    p = rng.normal(0.0, 0.3, m.NPARAMS)
    norm = np.concatenate([np.zeros(24), np.ones(24)]).astype(np.float32)
    X = rng.normal(0.0, 1.0, (200, 24)).astype(np.float32)
    a, _ = m.forward(p, norm, X, exact=True)
    b, _ = m.forward(p, norm, X)
    assert np.max(np.abs(a - b)) < 0.05 * (1.0 + np.max(np.abs(a)))


def _oracle_ctx(hcc, oracle, cfg, cloud):
    abi = sys.modules["hcc_gb300._abi"]
    o = oracle.OracleContext(cfg, abi)
    o.upload_cloud(cloud)
    o.build_neighbours()
    o.prepare_geometry()
    return o


def test_oracle_features_known_answers(hcc, oracle):
    h = 1 / 32
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=3)
    cfg = hcc.make_config(hcc.LinearAdvection(((1.0,), (1.0,))), cloud, scheme=hcc.MUSCL(2, 2))
    o = _oracle_ctx(hcc, oracle, cfg, cloud)
    # constant field: every feature is zero
    o.upload_state(np.full((cloud.n, 1), 2.5))
    assert not np.any(o.features())
    # linear field u = 3 + x - 2 y: the least-squares residual vanishes and |grad u| h / range matches the stencil
    x, y = cloud.pos[:, 0], cloud.pos[:, 1]
    u = 3.0 + x - 2.0 * y
    o.upload_state(u[:, None].copy())
    F = o.features()
    counts, idx, _, _ = o.neighbours()
    start = np.concatenate([[0], np.cumsum(counts)])
    for i in range(0, cloud.n, 37):
        nb = idx[start[i]:start[i + 1]]
        vals = np.concatenate([[u[i]], u[nb]]).astype(np.float32)
        r = float(vals.max() - vals.min())
        assert F[i, 0] == pytest.approx(r / (abs(vals.max()) + abs(vals.min())), rel=1e-5)
        assert abs(F[i, 3]) < 1e-3                                  # residual of an exact linear fit
        assert F[i, 4] == pytest.approx(min(8.0, np.sqrt(5.0) * h / r), rel=1e-3)
        # the four quantities of a scalar system are the same component
        np.testing.assert_array_equal(F[i, 0:6], F[i, 18:24])


def test_oracle_features_of_a_jump(hcc, oracle):
    """A density jump: particles whose stencil straddles it have a large relative range and residual."""
    h = 1 / 32
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=3)
    cfg = hcc.make_config(hcc.Euler(2, 1.4), cloud, scheme=hcc.MUSCL(2, 2), bc_map={t: 2 for t in range(1, 5)})
    o = _oracle_ctx(hcc, oracle, cfg, cloud)
    x = cloud.pos[:, 0]
    rho = np.where(x < 0.5, 1.0, 0.125)
    p = np.where(x < 0.5, 1.0, 0.1)
    U = np.stack([rho, 0 * rho, 0 * rho, p / 0.4], axis=1)
    o.upload_state(U)
    F = o.features()
    near = np.abs(x - 0.5) < 0.5 * h
    far = np.abs(x - 0.5) > 4 * h
    assert np.all(F[near, 0] > 0.7)                     # (1 - 0.125) / 1.125
    assert np.all(F[near, 3] > 0.05)
    assert not np.any(F[far])


def test_mlp_create_rejects_bad_configs_without_a_gpu(hcc, cuda_lib):
    abi = sys.modules["hcc_gb300._abi"]
    lib = cuda_lib
    for field, value in [("lr", 0.0), ("neg_keep", 1.5), ("beta1", 1.0), ("pos_weight", -1.0), ("capacity", -5)]:
        cfg = abi.HccMlpConfig(capacity=16, neg_keep=0.1, seed=1, lr=1e-3, beta1=0.9, beta2=0.999, adam_eps=1e-8,
                               pos_weight=1.0)
        setattr(cfg, field, value)
        h = C.c_void_p()
        assert lib.hcc_mlp_create(C.byref(cfg), C.byref(h)) == abi.HCC_ERR_INVALID
        assert not h.value
