"""Shared fixtures: the package (loaded from its directory), the oracle (the checker) and cloud builders."""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def load_package():
    if "hcc_gb300" in sys.modules:
        return sys.modules["hcc_gb300"]
    pkg_dir = ROOT / "hypercloudcore.jl_gb300"
    spec = importlib.util.spec_from_file_location("hcc_gb300", pkg_dir / "__init__.py",
                                                  submodule_search_locations=[str(pkg_dir)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["hcc_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    if "hcc_oracle_py" in sys.modules:
        return sys.modules["hcc_oracle_py"]
    spec = importlib.util.spec_from_file_location("hcc_oracle_py", ROOT / "oracle" / "oracle.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["hcc_oracle_py"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


@pytest.fixture(scope="session")
def hcc():
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    return load_oracle()


@pytest.fixture(scope="session")
def cuda_lib(hcc):
    """The built CUDA library (build first if needed; nvcc cross-compiles without a GPU)."""
    sys.path.insert(0, str(ROOT / "hypercloudcore.jl_gb300"))
    import build as _build  # noqa: E402
    sys.path.pop(0)
    _build.build()
    return hcc.load_library()


def c1_cloud(hcc, h=0.01, seed=42):
    """Advection parity cloud: [0,1]^2, spacing h, jitter ±0.25h, R = 2.5h."""
    return hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=seed)


def gaussian_ic(cloud, x0=0.3, y0=0.3, w=0.005):
    x, y = cloud.pos[:, 0], cloud.pos[:, 1]
    return np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / w)[:, None].copy()


def quadrant_ic(cloud, gamma=1.4):
    """Four-quadrant Riemann problem split at (0.5, 0.5), conservative variables."""
    x, y = cloud.pos[:, 0], cloud.pos[:, 1]
    vals = {  # (rho, u, v, p)
        "NE": (1.5, 0.0, 0.0, 1.5), "NW": (0.5323, 1.206, 0.0, 0.3),
        "SW": (0.138, 1.206, 1.206, 0.029), "SE": (0.5323, 0.0, 1.206, 0.3)}
    rho = np.empty(cloud.n); u = np.empty(cloud.n); v = np.empty(cloud.n); p = np.empty(cloud.n)
    for key, (r0, u0, v0, p0) in vals.items():
        sel = ((x >= 0.5) if key[1] == "E" else (x < 0.5)) & ((y >= 0.5) if key[0] == "N" else (y < 0.5))
        rho[sel], u[sel], v[sel], p[sel] = r0, u0, v0, p0
    E = p / (gamma - 1) + 0.5 * rho * (u * u + v * v)
    return np.stack([rho, rho * u, rho * v, E], axis=1)


def blast_ic(cloud, gamma=1.4, r0=0.2):
    c = np.full(cloud.dim, 0.5)
    r = np.sqrt(((cloud.pos - c) ** 2).sum(axis=1))
    rho = np.where(r < r0, 1.0, 0.125)
    p = np.where(r < r0, 1.0, 0.1)
    E = p / (gamma - 1)
    U = np.zeros((cloud.n, cloud.dim + 2))
    U[:, 0] = rho
    U[:, -1] = E
    return U
