"""hcc_gb300 — GB300-native explicit right-hand-side path of HyperCloudCore.jl, driven through its C ABI.

Host mirror of the reference's interface for this path (names and argument meaning follow it):

  * physics modules   ``LinearAdvection`` (test/PDEs/linear_advection.jl), ``Euler`` (new), ``KineticRelaxation``
                      (test/kinetic_source.jl) — the ``HyperbolicPDE`` subtypes compiled into the kernels;
  * schemes           ``MUSCL(order, div_order)`` (src/Interpolation/MUSCL.jl:116), ``MOOD(strategy, criterion)``
                      with ``MOODu1`` / ``MOODu2`` / ``MOODPAD`` / ``OnlyMOOD`` / ``NoMOOD`` and ``EPD0/EPD1/EPD2/STRICT_EPD0``
                      (src/TimeStepping/MOOD.jl);
  * stepper           ``GB300RKTimeStepper`` — ``ts(t, dt)`` is ``(ts::GeneralRKTimeStepper)(eq, pg, t, dt)``
                      (src/TimeStepping/TimeSteppers.jl:531) and ``ts.get_time_step()`` is
                      ``get_time_step(pg, eq, interp)`` (src/Grid/ParticleGrids.jl:386);
  * ``Context``       the raw C-ABI handle (include/hcc.h).

All compute runs in libhcc_gb300.so (hand-written sm_103a kernels). There is no CPU fallback: without the
library or a GPU every call raises ``HCCError``.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import _abi
from ._abi import (HccConfig, HccCounters, FP32, FP64, PDE_ADVECTION, PDE_BGK, PDE_EULER, MOOD_NONE, MOOD_ONLY,
                   MOOD_PAD, MOOD_U1, EPD_NONE, EPD0, EPD1, EPD2, STRICT_EPD0, TABLEAUS, BC_KEEP, BC_DIRICHLET, BC_OUTFLOW)
from .cloud import Cloud, rectangular_cloud, morton_permutation, splitmix64_uniform

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ["HCC_GB300_LIB"]) if os.environ.get("HCC_GB300_LIB") else PKG_DIR / "libhcc_gb300.so"


class HCCError(RuntimeError):
    """A failed C-ABI call (status code + the context's last error message)."""

    def __init__(self, status: int, message: str, call: str = ""):
        self.status = status
        name = _abi.STATUS_NAMES[status] if 0 <= status < len(_abi.STATUS_NAMES) else str(status)
        super().__init__(f"{call}: {name}: {message}" if call else f"{name}: {message}")


_LIB: Optional[C.CDLL] = None


def load_library(path: Optional[os.PathLike] = None) -> C.CDLL:
    """Load libhcc_gb300.so (built in-tree by build.build()). Raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise HCCError(_abi.HCC_ERR_STATE, f"{p} is missing: run build() first")
    lib = _abi.bind(C.CDLL(str(p)))
    if path is None:
        _LIB = lib
    return lib


def fp64_fma_rate() -> float:
    """FP64 FMA rate of the current GPU in TFLOP/s (hcc_fp64_fma_rate): the FP64 path's roofline denominator."""
    lib = load_library()
    out = C.c_double(0.0)
    st = lib.hcc_fp64_fma_rate(C.byref(out))
    if st != 0:
        raise HCCError(st, "FP64 FMA-rate kernel failed", "hcc_fp64_fma_rate")
    return out.value


# ------------------------------------------------------------------------------------------ descriptors
@dataclass
class LinearAdvection:
    """Diagonal linear advection: F_d(U)_m = c[d][m] U_m. `velocities[d][m]` (one tuple per axis)."""
    velocities: Sequence[Sequence[float]]
    pde: int = PDE_ADVECTION

    @property
    def dim(self) -> int:
        return len(self.velocities)

    @property
    def n_vars(self) -> int:
        return len(self.velocities[0])


@dataclass
class Euler:
    """Compressible Euler equations of an ideal gas, U = (rho, rho u_1..u_D, E)."""
    dim: int
    gamma: float = 1.4
    pde: int = PDE_EULER

    @property
    def n_vars(self) -> int:
        return self.dim + 2


@dataclass
class KineticRelaxation:
    """Discrete-velocity BGK relaxation: kinetic speeds `speeds[k][d]`, relaxation time `epsilon`, one macro
    moment u = Σ_k f_k advected with `macro_velocity`, Maxwellian M_k = coefficient (u + Σ_d F_d(u) D / v_k,d)."""
    speeds: Sequence[Sequence[float]]
    epsilon: float = 1e-4
    macro_velocity: Sequence[float] = (1.0, 0.0)
    coefficient: Optional[float] = None
    interior_factor: Optional[float] = None
    pde: int = PDE_BGK

    @property
    def dim(self) -> int:
        return len(self.speeds[0])

    @property
    def n_vars(self) -> int:
        return len(self.speeds)

    def maxwellian(self, u) -> np.ndarray:
        """Kinetic state at equilibrium with macro moments `u` (shape (N,)): f_k = coefficient (u + Σ_d a_d u
        interior_factor / v_k,d), a speed component below 1e-14 contributing nothing — the local relaxation
        initialisation set_initial_conditions! (test/kinetic_source.jl:110-131). Returns (N, n_vars) float64."""
        u = np.asarray(u, dtype=np.float64).reshape(-1)
        D, K = self.dim, self.n_vars
        coeff = float(self.coefficient if self.coefficient is not None else 1.0 / K)
        fac = float(self.interior_factor if self.interior_factor is not None else D)
        f = np.empty((u.size, K))
        for k in range(K):
            fd = np.zeros_like(u)
            for d in range(D):
                v = float(self.speeds[k][d])
                if abs(v) > 1e-14:
                    fd = fd + float(self.macro_velocity[d]) * u * (fac / v)
            f[:, k] = coeff * (u + fd)
        return f


@dataclass
class MUSCL:
    """MUSCL(T, D, M, order, limiter, flux; div_order) (src/Interpolation/MUSCL.jl:116). `limiter` is one
    of "none", "bj_soft", "bj_hard", "vk_soft", "vk_hard" (BarthJespersen / Venkatakrishnan, :soft / :hard);
    `flux` is "rusanov" (RusanovFlux) or "aligned" (AlignedRusanovFlux, FluxFunctions.jl:103-111);
    `moment_correction` adds the first-moment-free dissipation of a first-order scheme (MUSCL.jl:57, :224-283)."""
    order: int = 2
    div_order: int = 0
    limiter: str = "none"
    flux: str = "rusanov"
    moment_correction: bool = False


@dataclass
class UpwindDivergence:
    """UpwindDivergence(T, D, 1, 1, algorithm, flux; div_order) with algorithm :Tiwari (per axis the upwind-side
    gradient fit times v_d) or :Praveen (2-D, edge-normal / tangential upwind coefficients), Upwind.jl:158-249."""
    algorithm: str = "Tiwari"
    div_order: int = 0
    order: int = 1


def Upwind(div_order: int = 0, flux: str = "rusanov", algorithm: str = "Classic"):
    """UpwindDivergence(T, D, M, 1, algorithm, flux; div_order) (src/Interpolation/Upwind.jl). :Classic —
    piecewise-constant states, the numerical flux per pair and the MLS divergence of degree 1 — is the first-order
    MUSCL scheme (the reference's unit test unit_core.jl:937-945 holds the two equal to 1e-12); :Tiwari and
    :Praveen are scalar-only schemes of their own."""
    if algorithm == "Classic":
        return MUSCL(1, div_order, "none", flux)
    if algorithm not in _abi.UPWIND_ALGORITHMS:
        raise ValueError(f"unknown upwind algorithm {algorithm!r}")
    return UpwindDivergence(algorithm, div_order)


@dataclass
class WENO:
    """WENO(T, D, M, order; div_order) (src/Interpolation/WENO.jl:43, scalar there): systems component-wise, linear
    fluxes per component with their own velocity, Euler by local Lax-Friedrichs splitting (order <= 2 for M > 1)."""
    order: int = 2
    div_order: int = 0


@dataclass
class CentralDivergence:
    """CentralDivergence(T, D, M, order; div_order) (src/Interpolation/Central.jl:45-88): the divergence of F_j - F_i
    by the MLS intercept fit of degree = the particle's order (capped by div_order), no reconstruction."""
    order: int = 2
    div_order: int = 0


@dataclass
class MOODu1:
    delta: float


@dataclass
class MOODu2:
    """MOODu2(d; plateau = 1e-3, ratio = 1/2) (src/TimeStepping/MOOD.jl:104-130): MOODu1 plus the plateau test and
    the smooth-extremum override from the curvature terms of a degree-2 reconstruction."""
    delta: float
    plateau: float = 1e-3
    ratio: float = 0.5


class MOODPAD:
    pass


class OnlyMOOD:
    pass


class NoMOOD:
    pass


@dataclass
class MOOD:
    strategy: int = EPD1
    criterion: object = field(default_factory=NoMOOD)


def mover(kind: str = "none", *, alpha: float = 1.0, velocity=(0.0, 0.0, 0.0), omega=(0.0, 0.0, 0.0),
          center=(0.0, 0.0, 0.0), full_search_per_stage: bool = False, volume_estimator: str = "shepard",
          shepard_sweeps: int = 1) -> "_abi.HccMover":
    """Grid mover (src/TimeStepping/GridMovers.jl): "none" (NoGridMover), "lagrangian" (LagrangianMover), "scaled"
    (ScaledLagrangianMover(alpha)) or "prescribed" (PrescribedMover with w(x) = velocity + omega x (x - center)).
    `volume_estimator` ("shepard": ShepardVolumes(sweeps) after each step, the reference's default; "none": keep
    the volumes) is GeneralRKTimeStepper's `volume_estimator` (TimeSteppers.jl:145-146)."""
    m = _abi.HccMover()
    m.kind = _abi.MOVERS[kind]
    m.full_search_per_stage = int(bool(full_search_per_stage))
    m.keep_volumes = 0 if volume_estimator == "shepard" else 1
    m.shepard_sweeps = int(shepard_sweeps)
    m.alpha = float(alpha)
    for d in range(3):
        m.velocity[d], m.omega[d], m.center[d] = float(velocity[d]), float(omega[d]), float(center[d])
    return m


def config_defaults() -> HccConfig:
    """Python twin of hcc_config_defaults (include/hcc.h): the reference's defaults."""
    cfg = HccConfig()
    cfg.abi_version = _abi.HCC_ABI_VERSION
    cfg.dim, cfg.n_vars, cfg.pde, cfg.precision = 2, 1, PDE_ADVECTION, FP64
    cfg.muscl_order, cfg.div_order = 2, 0
    cfg.mood_criterion, cfg.mood_strategy = MOOD_U1, EPD1
    cfg.tableau, cfg.mood_substeps, cfg.max_mood_iterations = TABLEAUS["RK3_SSP"], 1, 64
    cfg.weight_alpha, cfg.gamma = 1.0, 1.4
    cfg.bgk_epsilon, cfg.bgk_coefficient, cfg.bgk_interior_factor = 1e-4, 1.0, 2.0
    cfg.u2_plateau, cfg.u2_ratio = 1e-3, 0.5
    for d in range(_abi.HCC_MAX_DIM):
        cfg.dx[d], cfg.canvas_max[d], cfg.domain_max[d] = 1.0, 1.0, 1.0
    return cfg


def make_config(pde, cloud: Cloud, *, scheme: MUSCL = None, mood: MOOD = None, tableau: str = "RK3_SSP",
                precision: str = "fp64", bc_map: Optional[dict] = None, alpha: float = 1.0,
                mood_substeps: bool = True, max_mood_iterations: int = 64,
                reset_orders_per_stage: bool = False) -> HccConfig:
    """The hcc_config of a stepper (the arguments of GeneralRKTimeStepper / MUSCL / ParticleGrid)."""
    scheme = scheme or MUSCL()
    mood = mood or MOOD()
    cfg = config_defaults()
    D = cloud.dim
    if pde.dim != D:
        raise HCCError(_abi.HCC_ERR_INVALID, f"physics dimension {pde.dim} != cloud dimension {D}")
    cfg.dim = D
    cfg.n_vars = pde.n_vars
    cfg.pde = pde.pde
    cfg.precision = FP32 if str(precision).lower() in ("fp32", "f32", "float32") else FP64
    cfg.muscl_order = scheme.order
    cfg.div_order = scheme.div_order
    if isinstance(scheme, WENO):
        cfg.scheme = _abi.SCHEME_WENO
    elif isinstance(scheme, CentralDivergence):
        cfg.scheme = _abi.SCHEME_CENTRAL
    elif isinstance(scheme, UpwindDivergence):
        cfg.scheme = _abi.SCHEME_UPWIND
        cfg.upwind_algorithm = _abi.UPWIND_ALGORITHMS[scheme.algorithm]
    else:
        cfg.scheme = _abi.SCHEME_MUSCL
        cfg.limiter = _abi.LIMITERS[scheme.limiter]
        cfg.flux = _abi.FLUXES[scheme.flux]
        cfg.moment_correction = int(bool(scheme.moment_correction))
    cfg.tableau = TABLEAUS[tableau] if isinstance(tableau, str) else int(tableau)
    cfg.mood_substeps = 1 if mood_substeps else 0
    cfg.max_mood_iterations = max_mood_iterations
    cfg.reset_orders_per_stage = 1 if reset_orders_per_stage else 0
    cfg.mood_strategy = mood.strategy
    crit = mood.criterion
    if isinstance(crit, MOODu1):
        cfg.mood_criterion, cfg.mood_delta = MOOD_U1, float(crit.delta)
    elif isinstance(crit, MOODu2):
        cfg.mood_criterion, cfg.mood_delta = _abi.MOOD_U2, float(crit.delta)
        cfg.u2_plateau, cfg.u2_ratio = float(crit.plateau), float(crit.ratio)
    elif isinstance(crit, MOODPAD):
        cfg.mood_criterion = MOOD_PAD
    elif isinstance(crit, OnlyMOOD):
        cfg.mood_criterion = MOOD_ONLY
    else:
        cfg.mood_criterion = MOOD_NONE
    for d in range(D):
        cfg.periodic[d] = int(cloud.periodic[d])
        cfg.dx[d] = cloud.dx[d]
        cfg.canvas_min[d], cfg.canvas_max[d] = cloud.canvas_min[d], cloud.canvas_max[d]
        cfg.domain_min[d], cfg.domain_max[d] = cloud.domain_min[d], cloud.domain_max[d]
    cfg.radius = cloud.radius
    cfg.weight_alpha = alpha
    for tag, kind in (bc_map or {}).items():
        cfg.bc_by_tag[int(tag) - 1] = int(kind)
    if isinstance(pde, LinearAdvection):
        for d in range(D):
            for m in range(pde.n_vars):
                cfg.velocity[d][m] = float(pde.velocities[d][m])
    elif isinstance(pde, Euler):
        cfg.gamma = float(pde.gamma)
    elif isinstance(pde, KineticRelaxation):
        for k, v in enumerate(pde.speeds):
            for d in range(D):
                cfg.velocity[d][k] = float(v[d])
        cfg.bgk_epsilon = float(pde.epsilon)
        for d in range(D):
            cfg.bgk_macro_velocity[d] = float(pde.macro_velocity[d])
        cfg.bgk_coefficient = float(pde.coefficient if pde.coefficient is not None else 1.0 / pde.n_vars)
        cfg.bgk_interior_factor = float(pde.interior_factor if pde.interior_factor is not None else D)
    return cfg


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Context:
    """Owner of one hcc_ctx (one CUDA stream, library-owned device memory)."""

    def __init__(self, cfg: HccConfig, capacity: int = 0, lib: Optional[C.CDLL] = None):
        self.lib = lib or load_library()
        self.cfg = cfg
        self.D, self.M = cfg.dim, cfg.n_vars
        self.f32 = cfg.precision == FP32
        self._h = C.c_void_p()
        st = self.lib.hcc_create(C.byref(cfg), int(capacity), C.byref(self._h))
        if st != 0:
            msg = self.lib.hcc_last_error(self._h).decode()
            self.lib.hcc_destroy(self._h)
            self._h = None
            raise HCCError(st, msg, "hcc_create")
        self.n = 0

    # -- plumbing
    def _check(self, st: int, call: str):
        if st != 0:
            raise HCCError(st, self.lib.hcc_last_error(self._h).decode(), call)

    def close(self):
        if self._h:
            self.lib.hcc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- cloud and geometry
    def upload_cloud(self, cloud: Cloud):
        pos = np.ascontiguousarray(cloud.pos, dtype=np.float64)
        bnd = np.ascontiguousarray(cloud.is_boundary, dtype=np.uint8)
        tags = np.ascontiguousarray(cloud.tags, dtype=np.int32)
        vol = np.ascontiguousarray(cloud.volumes, dtype=np.float64)
        self._check(self.lib.hcc_upload_cloud(self._h, pos.shape[0], _ptr(pos, C.c_double), _ptr(bnd, C.c_uint8),
                                              _ptr(tags, C.c_int32), _ptr(vol, C.c_double)), "hcc_upload_cloud")
        self.n = pos.shape[0]

    def upload_batch(self, clouds) -> Cloud:
        """Upload independent clouds as one batch (hcc_upload_batch): the library packs them side by side with
        gaps wider than the support; returns the union as a Cloud (positions shifted, the union canvas), whose
        meta holds the per-cloud `offsets` and `shifts`."""
        D = self.D
        offsets = np.zeros(len(clouds) + 1, dtype=np.int64)
        offsets[1:] = np.cumsum([c.n for c in clouds])
        pos = np.ascontiguousarray(np.concatenate([c.pos for c in clouds]), dtype=np.float64)
        bnd = np.ascontiguousarray(np.concatenate([c.is_boundary for c in clouds]), dtype=np.uint8)
        tags = np.ascontiguousarray(np.concatenate([c.tags for c in clouds]), dtype=np.int32)
        vol = np.ascontiguousarray(np.concatenate([c.volumes for c in clouds]), dtype=np.float64)
        shifts = np.zeros((len(clouds), D), dtype=np.float64)
        canvas = np.zeros(2 * D, dtype=np.float64)
        self._check(self.lib.hcc_upload_batch(self._h, len(clouds), _ptr(offsets, C.c_int64), _ptr(pos, C.c_double),
                                              _ptr(bnd, C.c_uint8), _ptr(tags, C.c_int32), _ptr(vol, C.c_double),
                                              _ptr(shifts, C.c_double), _ptr(canvas, C.c_double)),
                    "hcc_upload_batch")
        self.n = int(offsets[-1])
        self._batch_n = len(clouds)
        shifted = pos + np.repeat(shifts, np.diff(offsets), axis=0)
        lo, hi = tuple(canvas[:D]), tuple(canvas[D:])
        c0 = clouds[0]
        return Cloud(shifted, bnd, tags, vol, c0.dx, c0.radius, lo, hi, lo, hi, (False,) * D,
                     {"offsets": offsets, "shifts": shifts, "batch": True})

    def update_volumes(self, sweeps: int = 1):
        """update_volumes!(pg, ShepardVolumes(sweeps)) (Volumes.jl:183-229)."""
        self._check(self.lib.hcc_update_volumes(self._h, int(sweeps)), "hcc_update_volumes")

    def volumes(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.float64)
        self._check(self.lib.hcc_download_volumes(self._h, _ptr(out, C.c_double)), "hcc_download_volumes")
        return out

    def batch_total_mass(self) -> np.ndarray:
        """total_mass per cloud of the last batch: (n_clouds, M)."""
        n = getattr(self, "_batch_n", None)
        if n is None:
            raise HCCError(_abi.HCC_ERR_STATE, "no batch uploaded", "hcc_batch_total_mass")
        out = np.zeros((n, self.M), dtype=np.float64)
        self._check(self.lib.hcc_batch_total_mass(self._h, _ptr(out, C.c_double)), "hcc_batch_total_mass")
        return out

    def batch_time_steps(self) -> np.ndarray:
        """The CFL step of every cloud of the last batch (hcc_batch_time_steps)."""
        n = getattr(self, "_batch_n", None)
        if n is None:
            raise HCCError(_abi.HCC_ERR_STATE, "no batch uploaded", "hcc_batch_time_steps")
        out = np.zeros(n, dtype=np.float64)
        self._check(self.lib.hcc_batch_time_steps(self._h, _ptr(out, C.c_double)), "hcc_batch_time_steps")
        return out

    def step_batch(self, t: float, dts):
        """One step of every cloud of the last batch with its own dt (hcc_batch_step)."""
        d = np.ascontiguousarray(dts, dtype=np.float64)
        n = getattr(self, "_batch_n", None)
        if n is None or d.shape != (n,):
            raise HCCError(_abi.HCC_ERR_INVALID, "one dt per cloud of the batch", "hcc_batch_step")
        self._check(self.lib.hcc_batch_step(self._h, float(t), _ptr(d, C.c_double)), "hcc_batch_step")

    def build_neighbours(self):
        self._check(self.lib.hcc_build_neighbours(self._h), "hcc_build_neighbours")

    def prepare_geometry(self):
        self._check(self.lib.hcc_prepare_geometry(self._h), "hcc_prepare_geometry")

    def neighbours(self):
        """(counts, idx, w, dist) in the reference's row-major order."""
        counts = np.zeros(self.n, dtype=np.int32)
        self._check(self.lib.hcc_download_neighbours(self._h, _ptr(counts, C.c_int32), None, None, None),
                    "hcc_download_neighbours")
        tot = int(counts.sum())
        idx = np.zeros(tot, dtype=np.int32)
        w = np.zeros(tot, dtype=np.float64)
        dist = np.zeros((tot, self.D), dtype=np.float64)
        self._check(self.lib.hcc_download_neighbours(self._h, None, _ptr(idx, C.c_int32), _ptr(w, C.c_double),
                                                     _ptr(dist, C.c_double)), "hcc_download_neighbours")
        return counts, idx, w, dist

    def neighbour_counts(self):
        """Neighbour count of every particle (no list download)."""
        counts = np.zeros(self.n, dtype=np.int32)
        self._check(self.lib.hcc_download_neighbours(self._h, _ptr(counts, C.c_int32), None, None, None),
                    "hcc_download_neighbours")
        return counts

    def neighbours_of(self, ids, max_slots: int):
        """(counts, idx, w, dist) of the selected particles: row q holds the first max_slots slots of ids[q]."""
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        q = len(ids)
        counts = np.zeros(q, dtype=np.int32)
        idx = np.full((q, max_slots), -1, dtype=np.int32)
        w = np.zeros((q, max_slots), dtype=np.float64)
        dist = np.zeros((q, max_slots, self.D), dtype=np.float64)
        self._check(self.lib.hcc_download_neighbours_of(self._h, q, _ptr(ids, C.c_int64), int(max_slots),
                                                        _ptr(counts, C.c_int32), _ptr(idx, C.c_int32),
                                                        _ptr(w, C.c_double), _ptr(dist, C.c_double)),
                    "hcc_download_neighbours_of")
        return counts, idx, w, dist

    def geometry(self, total: int):
        dw = np.zeros((total, self.D), dtype=np.float64)
        okr = np.zeros(self.n, dtype=np.uint8)
        okd = np.zeros(self.n, dtype=np.uint8)
        self._check(self.lib.hcc_download_geometry(self._h, _ptr(dw, C.c_double), _ptr(okr, C.c_uint8),
                                                   _ptr(okd, C.c_uint8)), "hcc_download_geometry")
        return dw, okr, okd

    # -- state
    def upload_state(self, U: np.ndarray):
        if U.dtype == np.float32:
            a = np.ascontiguousarray(U, dtype=np.float32)
            self._check(self.lib.hcc_upload_state_f32(self._h, _ptr(a, C.c_float)), "hcc_upload_state_f32")
        else:
            a = np.ascontiguousarray(U, dtype=np.float64)
            self._check(self.lib.hcc_upload_state(self._h, _ptr(a, C.c_double)), "hcc_upload_state")

    def download_state(self, dtype=np.float64, out: Optional[np.ndarray] = None) -> np.ndarray:
        """The state (N x M) as float64 or float32; `out` (C-contiguous, that shape and dtype — e.g. a view of
        pinned host memory) is filled in place instead of a new array."""
        if out is None:
            out = np.empty((self.n, self.M), dtype=dtype)
        else:
            dtype = out.dtype
            if out.shape != (self.n, self.M) or dtype not in (np.float32, np.float64) or \
                    not out.flags["C_CONTIGUOUS"] or not out.flags["WRITEABLE"]:
                raise ValueError("out must be a writeable C-contiguous (N, M) float32/float64 array")
        if dtype == np.float32:
            self._check(self.lib.hcc_download_state_f32(self._h, _ptr(out, C.c_float)), "hcc_download_state_f32")
        else:
            self._check(self.lib.hcc_download_state(self._h, _ptr(out, C.c_double)), "hcc_download_state")
        return out

    def time_step(self) -> float:
        dt = C.c_double()
        self._check(self.lib.hcc_time_step(self._h, C.byref(dt)), "hcc_time_step")
        return dt.value

    def compute_rhs(self) -> np.ndarray:
        K = np.zeros((self.n, self.M), dtype=np.float64)
        self._check(self.lib.hcc_compute_rhs(self._h, _ptr(K, C.c_double)), "hcc_compute_rhs")
        return K

    def step(self, t: float, dt: float):
        self._check(self.lib.hcc_step(self._h, float(t), float(dt)), "hcc_step")

    def orders(self) -> np.ndarray:
        o = np.zeros(self.n, dtype=np.int32)
        self._check(self.lib.hcc_download_orders(self._h, _ptr(o, C.c_int32)), "hcc_download_orders")
        return o

    def mood_flags(self) -> np.ndarray:
        f = np.zeros(self.n, dtype=np.uint8)
        self._check(self.lib.hcc_download_mood_flags(self._h, _ptr(f, C.c_uint8)), "hcc_download_mood_flags")
        return f

    def counters(self) -> dict:
        c = HccCounters()
        self._check(self.lib.hcc_get_counters(self._h, C.byref(c)), "hcc_get_counters")
        return c.as_dict()

    def total_mass(self) -> np.ndarray:
        out = np.zeros(self.M, dtype=np.float64)
        self._check(self.lib.hcc_total_mass(self._h, _ptr(out, C.c_double)), "hcc_total_mass")
        return out

    def synchronize(self):
        self._check(self.lib.hcc_synchronize(self._h), "hcc_synchronize")

    def set_profiling(self, enable: bool = True):
        self._check(self.lib.hcc_set_profiling(self._h, int(bool(enable))), "hcc_set_profiling")

    def set_mover(self, m):
        """Select the grid mover (see `mover`)."""
        self._check(self.lib.hcc_set_mover(self._h, C.byref(m)), "hcc_set_mover")

    def positions(self) -> np.ndarray:
        out = np.zeros((self.n, self.D), dtype=np.float64)
        self._check(self.lib.hcc_download_positions(self._h, _ptr(out, C.c_double)), "hcc_download_positions")
        return out

    def save_snapshot(self, path):
        """Checkpoint: positions, state, orders, MOOD flags and the step count to a binary file."""
        self._check(self.lib.hcc_save_snapshot(self._h, str(path).encode()), "hcc_save_snapshot")

    def load_snapshot(self, path):
        """Resume from a snapshot of a context with the same configuration and particle count."""
        self._check(self.lib.hcc_load_snapshot(self._h, str(path).encode()), "hcc_load_snapshot")

    def set_tile_staging(self, enable: bool = True):
        """Tile-staged FP32 full passes (the default for 3-D contexts that qualify) or the stream-fed ones."""
        self._check(self.lib.hcc_set_tile_staging(self._h, int(bool(enable))), "hcc_set_tile_staging")

    def tile_staging(self) -> dict:
        """{"active": next step's full passes are tile-staged, "union_entries", "largest_union"}."""
        act, tot, mx = C.c_int32(), C.c_int64(), C.c_int32()
        self._check(self.lib.hcc_get_tile_staging(self._h, C.byref(act), C.byref(tot), C.byref(mx)),
                    "hcc_get_tile_staging")
        return {"active": bool(act.value), "union_entries": tot.value, "largest_union": mx.value}

    def set_step_graphs(self, enable: bool = True):
        """Take each step as one captured CUDA graph (default) or drive the MOOD fixed points from the host."""
        self._check(self.lib.hcc_set_step_graphs(self._h, int(bool(enable))), "hcc_set_step_graphs")

    def tuning(self) -> dict:
        """Launch shapes of the step: flux_block, gather_block, list_blocks_per_sm, drop_blocks_per_sm."""
        t = _abi.HccTuning()
        self._check(self.lib.hcc_get_tuning(self._h, C.byref(t)), "hcc_get_tuning")
        return t.as_dict()

    def set_tuning(self, **shapes):
        """Set some of the launch shapes (the others stay); results are bit-identical across shapes."""
        t = _abi.HccTuning(**{**self.tuning(), **shapes})
        self._check(self.lib.hcc_set_tuning(self._h, C.byref(t)), "hcc_set_tuning")

    def autotune(self, dt: float, steps: int = 5) -> dict:
        """Time the launch-shape candidates over `steps` steps of size dt from the current state and keep the
        fastest (hcc_autotune); the state and counters are left as they were. Returns the report."""
        r = _abi.HccTuneReport()
        self._check(self.lib.hcc_autotune(self._h, float(dt), int(steps), C.byref(r)), "hcc_autotune")
        return {"best": r.best.as_dict(), "default_ms": r.default_ms, "best_ms": r.best_ms,
                "candidates": r.candidates, "steps": r.steps}

    def kernel_times(self, reset: bool = False) -> dict:
        t = _abi.HccKernelTimes()
        self._check(self.lib.hcc_get_kernel_times(self._h, C.byref(t), int(bool(reset))), "hcc_get_kernel_times")
        return t.as_dict()

    def stream(self) -> int:
        return int(self.lib.hcc_stream(self._h) or 0)

    # -- learned troubled-point predictor
    def set_predictor(self, predictor, threshold: float = 0.5):
        """Attach a TroubledPointPredictor (None detaches): each step pre-lowers the particles it predicts."""
        self._predictor = predictor
        h = predictor.handle if predictor is not None else None
        self._check(self.lib.hcc_set_predictor(self._h, h, float(threshold)), "hcc_set_predictor")

    def set_feature_capture(self, enable: bool = True):
        """Keep each step's start-of-step stencil features (for TroubledPointPredictor.collect)."""
        self._check(self.lib.hcc_set_feature_capture(self._h, int(bool(enable))), "hcc_set_feature_capture")

    def features(self) -> np.ndarray:
        """The 24 stencil features (N x 24, FP32) of the current state."""
        out = np.zeros((self.n, _abi.HCC_MLP_FEATURES), dtype=np.float32)
        self._check(self.lib.hcc_download_features(self._h, _ptr(out, C.c_float)), "hcc_download_features")
        return out

    def predicted(self) -> np.ndarray:
        """The particles the predictor pre-lowered in the last step (0/1)."""
        out = np.zeros(self.n, dtype=np.uint8)
        self._check(self.lib.hcc_download_predicted(self._h, _ptr(out, C.c_uint8)), "hcc_download_predicted")
        return out


class GB300RKTimeStepper:
    """The GB300 counterpart of GeneralRKTimeStepper(pde, MUSCL(...), MOOD(...), tableau) on a fixed cloud.

    ``ts(t, dt)`` advances the state one step; ``ts.get_time_step()`` is the CFL step at CFL number 1."""

    def __init__(self, pde, cloud: Cloud, scheme: MUSCL = None, mood: MOOD = None, tableau: str = "RK3_SSP",
                 precision: str = "fp64", bc_map: Optional[dict] = None, **kw):
        self.pde, self.cloud = pde, cloud
        self.cfg = make_config(pde, cloud, scheme=scheme, mood=mood, tableau=tableau, precision=precision,
                               bc_map=bc_map, **kw)
        self.ctx = Context(self.cfg)
        self.ctx.upload_cloud(cloud)
        self.ctx.build_neighbours()
        self.ctx.prepare_geometry()

    def set_state(self, U: np.ndarray):
        self.ctx.upload_state(U)

    def state(self) -> np.ndarray:
        return self.ctx.download_state()

    def get_time_step(self) -> float:
        return self.ctx.time_step()

    def __call__(self, t: float, dt: float):
        self.ctx.step(t, dt)

    def mood_flags(self) -> np.ndarray:
        return self.ctx.mood_flags()

    def particle_orders(self) -> np.ndarray:
        return self.ctx.orders()


from .learned import TroubledPointPredictor  # noqa: E402

__all__ = [
    "TroubledPointPredictor",
    "HCCError", "load_library", "LinearAdvection", "Euler", "KineticRelaxation", "MUSCL", "Upwind", "UpwindDivergence", "WENO", "CentralDivergence", "mover", "MOOD", "MOODu1", "MOODu2",
    "MOODPAD", "OnlyMOOD", "NoMOOD", "EPD_NONE", "EPD0", "EPD1", "EPD2", "STRICT_EPD0", "make_config", "Context",
    "GB300RKTimeStepper", "Cloud", "rectangular_cloud", "morton_permutation", "splitmix64_uniform", "TABLEAUS",
    "BC_KEEP", "BC_DIRICHLET", "BC_OUTFLOW", "HccConfig",
]
