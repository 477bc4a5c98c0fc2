"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of liboracle_hcc.so, the CPU restatement of the reference path.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker; never by the product.
Method names mirror hcc_gb300.Context so parity tests read the same on both sides.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle_hcc.so"


def build(verbose: bool = False) -> Path:
    """Compile the oracle with its Makefile (g++, OpenMP, no floating-point contraction)."""
    r = subprocess.run(["make", "-C", str(ORACLE_DIR), "liboracle_hcc.so"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stdout + r.stderr)
    return LIB_PATH


_LIB = None


def load(abi) -> C.CDLL:
    """Load (building first if needed) the oracle library. `abi` is the package's _abi module (config layout)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    src = ORACLE_DIR / "hcc_oracle.cpp"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        build()
    lib = C.CDLL(str(LIB_PATH))
    dp, ip, up, P = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint8), C.c_void_p
    protos = [
        ("orc_create", C.c_int, [C.POINTER(abi.HccConfig), C.POINTER(P)]),
        ("orc_destroy", C.c_int, [P]),
        ("orc_last_error", C.c_char_p, [P]),
        ("orc_set_threads", C.c_int, [C.c_int]),
        ("orc_upload_cloud", C.c_int, [P, C.c_int64, dp, up, ip, dp]),
        ("orc_build_neighbours", C.c_int, [P]),
        ("orc_neighbour_total", C.c_int, [P, C.POINTER(C.c_int64), ip]),
        ("orc_download_neighbours", C.c_int, [P, ip, ip, dp, dp]),
        ("orc_download_positions", C.c_int, [P, dp]),
        ("orc_neighbour_counts", C.c_int, [P, ip]),
        ("orc_neighbours_of", C.c_int, [P, C.c_int64, C.POINTER(C.c_int64), C.c_int32, ip, ip, dp, dp]),
        ("orc_prepare_geometry", C.c_int, [P]),
        ("orc_download_geometry", C.c_int, [P, dp, up, up]),
        ("orc_upload_state", C.c_int, [P, dp]),
        ("orc_download_state", C.c_int, [P, dp]),
        ("orc_time_step", C.c_int, [P, dp]),
        ("orc_compute_rhs", C.c_int, [P, dp]),
        ("orc_compute_rhs_orders", C.c_int, [P, ip, dp]),
        ("orc_step", C.c_int, [P, C.c_double, C.c_double]),
        ("orc_download_orders", C.c_int, [P, ip]),
        ("orc_upload_orders", C.c_int, [P, ip]),
        ("orc_download_mood_flags", C.c_int, [P, up]),
        ("orc_get_counters", C.c_int, [P, C.POINTER(abi.HccCounters)]),
        ("orc_total_mass", C.c_int, [P, dp]),
        ("orc_set_streamed", C.c_int, [P, C.c_int]),
        ("orc_download_gradients", C.c_int, [P, dp, ip]),
        ("orc_ssp_coefficient", C.c_double, [C.c_int32]),
        ("orc_basis_count", C.c_int32, [C.c_int32, C.c_int32]),
        ("orc_div_idx", C.c_int32, [C.c_int32, C.c_int32]),
        ("orc_divergence_index", C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
        ("orc_basis_exponents", C.c_int32, [C.c_int32, C.c_int32, ip]),
        ("orc_mls_divergence", C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, dp, dp, dp, C.c_double, dp]),
        ("orc_mls_solve", C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, dp, dp, dp, C.c_double, dp]),
        ("orc_cholesky_moment", C.c_int32, [C.c_int32, dp, dp, ip]),
        ("orc_expand_mask", C.c_int, [P, up, C.c_int32]),
        ("orc_interface_orders", C.c_int, [P, C.c_int64, C.c_int64, ip, ip]),
        ("orc_detect_and_drop", C.c_int, [P, dp, dp, C.c_int32, up, C.c_int32, ip]),
        ("orc_apply_bcs", C.c_int, [P, dp]),
        ("orc_criterion_flags", C.c_int, [P, C.c_int64, dp, dp, ip, dp, ip]),
        ("orc_set_mover", C.c_int, [P, C.POINTER(abi.HccMover)]),
        ("orc_features", C.c_int, [P, C.POINTER(C.c_float)]),
        ("orc_update_volumes", C.c_int, [P, C.c_int32]),
        ("orc_download_volumes", C.c_int, [P, dp]),
        ("orc_set_prelowered", C.c_int, [P, up]),
    ]
    for name, res, args in protos:
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    _LIB = lib
    return lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class OracleError(RuntimeError):
    pass


class OracleContext:
    """CPU counterpart of hcc_gb300.Context (same method names and array shapes)."""

    def __init__(self, cfg, abi):
        self.lib = load(abi)
        self.abi = abi
        self.cfg = cfg
        self.D, self.M = cfg.dim, cfg.n_vars
        self._h = C.c_void_p()
        st = self.lib.orc_create(C.byref(cfg), C.byref(self._h))
        if st != 0:
            msg = self.lib.orc_last_error(self._h).decode()
            self.lib.orc_destroy(self._h)
            self._h = None
            raise OracleError(f"orc_create: {st}: {msg}")
        self.n = 0

    def _check(self, st, call):
        if st != 0:
            raise OracleError(f"{call}: {st}: {self.lib.orc_last_error(self._h).decode()}")

    def close(self):
        if self._h:
            self.lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def set_threads(n: int):
        if _LIB is not None:
            _LIB.orc_set_threads(int(n))

    def upload_cloud(self, cloud):
        pos = np.ascontiguousarray(cloud.pos, dtype=np.float64)
        bnd = np.ascontiguousarray(cloud.is_boundary, dtype=np.uint8)
        tags = np.ascontiguousarray(cloud.tags, dtype=np.int32)
        vol = np.ascontiguousarray(cloud.volumes, dtype=np.float64)
        self._check(self.lib.orc_upload_cloud(self._h, pos.shape[0], _p(pos, C.c_double), _p(bnd, C.c_uint8),
                                              _p(tags, C.c_int32), _p(vol, C.c_double)), "orc_upload_cloud")
        self.n = pos.shape[0]

    def build_neighbours(self):
        self._check(self.lib.orc_build_neighbours(self._h), "orc_build_neighbours")

    def prepare_geometry(self):
        self._check(self.lib.orc_prepare_geometry(self._h), "orc_prepare_geometry")

    def set_streamed(self, streamed: bool):
        self._check(self.lib.orc_set_streamed(self._h, int(bool(streamed))), "orc_set_streamed")

    def neighbours(self):
        tot = C.c_int64()
        mx = C.c_int32()
        self._check(self.lib.orc_neighbour_total(self._h, C.byref(tot), C.byref(mx)), "orc_neighbour_total")
        counts = np.zeros(self.n, dtype=np.int32)
        idx = np.zeros(tot.value, dtype=np.int32)
        w = np.zeros(tot.value, dtype=np.float64)
        dist = np.zeros((tot.value, self.D), dtype=np.float64)
        self._check(self.lib.orc_download_neighbours(self._h, _p(counts, C.c_int32), _p(idx, C.c_int32),
                                                     _p(w, C.c_double), _p(dist, C.c_double)), "orc_download_neighbours")
        return counts, idx, w, dist

    def neighbour_counts(self):
        """Neighbour counts of every particle (the count pass alone)."""
        counts = np.zeros(self.n, dtype=np.int32)
        self._check(self.lib.orc_neighbour_counts(self._h, _p(counts, C.c_int32)), "orc_neighbour_counts")
        return counts

    def neighbours_of(self, ids, max_slots: int):
        """(counts, idx, w, dist) of the selected particles in the reference's order, rows of max_slots slots."""
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        q = len(ids)
        counts = np.zeros(q, dtype=np.int32)
        idx = np.full((q, max_slots), -1, dtype=np.int32)
        w = np.zeros((q, max_slots), dtype=np.float64)
        dist = np.zeros((q, max_slots, self.D), dtype=np.float64)
        self._check(self.lib.orc_neighbours_of(self._h, q, ids.ctypes.data_as(C.POINTER(C.c_int64)), int(max_slots),
                                               _p(counts, C.c_int32), _p(idx, C.c_int32), _p(w, C.c_double),
                                               _p(dist, C.c_double)), "orc_neighbours_of")
        return counts, idx, w, dist

    def positions(self):
        out = np.zeros((self.n, self.D), dtype=np.float64)
        self._check(self.lib.orc_download_positions(self._h, _p(out, C.c_double)), "orc_download_positions")
        return out

    def geometry(self, total: int):
        dw = np.zeros((total, self.D), dtype=np.float64)
        okr = np.zeros(self.n, dtype=np.uint8)
        okd = np.zeros(self.n, dtype=np.uint8)
        self._check(self.lib.orc_download_geometry(self._h, _p(dw, C.c_double), _p(okr, C.c_uint8),
                                                   _p(okd, C.c_uint8)), "orc_download_geometry")
        return dw, okr, okd

    def upload_state(self, U):
        a = np.ascontiguousarray(U, dtype=np.float64)
        self._check(self.lib.orc_upload_state(self._h, _p(a, C.c_double)), "orc_upload_state")

    def download_state(self):
        out = np.zeros((self.n, self.M), dtype=np.float64)
        self._check(self.lib.orc_download_state(self._h, _p(out, C.c_double)), "orc_download_state")
        return out

    def time_step(self) -> float:
        dt = C.c_double()
        self._check(self.lib.orc_time_step(self._h, C.byref(dt)), "orc_time_step")
        return dt.value

    def compute_rhs(self):
        K = np.zeros((self.n, self.M), dtype=np.float64)
        self._check(self.lib.orc_compute_rhs(self._h, _p(K, C.c_double)), "orc_compute_rhs")
        return K

    def compute_rhs_orders(self, orders):
        o = np.ascontiguousarray(orders, dtype=np.int32)
        K = np.zeros((self.n, self.M), dtype=np.float64)
        self._check(self.lib.orc_compute_rhs_orders(self._h, _p(o, C.c_int32), _p(K, C.c_double)),
                    "orc_compute_rhs_orders")
        return K

    def step(self, t, dt):
        self._check(self.lib.orc_step(self._h, float(t), float(dt)), "orc_step")

    def orders(self):
        o = np.zeros(self.n, dtype=np.int32)
        self._check(self.lib.orc_download_orders(self._h, _p(o, C.c_int32)), "orc_download_orders")
        return o

    def set_orders(self, orders):
        a = np.ascontiguousarray(orders, dtype=np.int32)
        self._check(self.lib.orc_upload_orders(self._h, _p(a, C.c_int32)), "orc_upload_orders")

    def mood_flags(self):
        f = np.zeros(self.n, dtype=np.uint8)
        self._check(self.lib.orc_download_mood_flags(self._h, _p(f, C.c_uint8)), "orc_download_mood_flags")
        return f

    def counters(self) -> dict:
        c = self.abi.HccCounters()
        self._check(self.lib.orc_get_counters(self._h, C.byref(c)), "orc_get_counters")
        return c.as_dict()

    def total_mass(self):
        out = np.zeros(self.M, dtype=np.float64)
        self._check(self.lib.orc_total_mass(self._h, _p(out, C.c_double)), "orc_total_mass")
        return out

    def gradients(self):
        br = C.c_int32()
        self._check(self.lib.orc_download_gradients(self._h, None, C.byref(br)), "orc_download_gradients")
        g = np.zeros((self.n, br.value, self.M), dtype=np.float64)
        self._check(self.lib.orc_download_gradients(self._h, _p(g, C.c_double), C.byref(br)), "orc_download_gradients")
        return g

    # ---- kernel-level helpers for known-answer tests
    def expand_mask(self, mask, hops):
        m = np.ascontiguousarray(mask, dtype=np.uint8).copy()
        self._check(self.lib.orc_expand_mask(self._h, _p(m, C.c_uint8), int(hops)), "orc_expand_mask")
        return m

    def interface_orders(self, i, j):
        a, b = C.c_int32(), C.c_int32()
        self._check(self.lib.orc_interface_orders(self._h, int(i), int(j), C.byref(a), C.byref(b)),
                    "orc_interface_orders")
        return a.value, b.value

    def detect_and_drop(self, prev, cand, full=True, dirty=None, with_eq=True) -> bool:
        p = np.ascontiguousarray(prev, dtype=np.float64)
        c = np.ascontiguousarray(cand, dtype=np.float64)
        ch = C.c_int32()
        dptr = None
        if dirty is not None:
            d = np.ascontiguousarray(dirty, dtype=np.uint8)
            dptr = _p(d, C.c_uint8)
        self._check(self.lib.orc_detect_and_drop(self._h, _p(p, C.c_double), _p(c, C.c_double), int(bool(full)), dptr,
                                                 int(bool(with_eq)), C.byref(ch)), "orc_detect_and_drop")
        return bool(ch.value)

    def set_mover(self, mover):
        """mover: an HccMover (see hcc_gb300.mover())."""
        self._check(self.lib.orc_set_mover(self._h, C.byref(mover)), "orc_set_mover")

    def criterion_flags(self, p, prev, grads, orders, cand) -> bool:
        """The MOOD criterion of particle p for hand-set states, gradients (N x Br x M), orders and candidate."""
        pv = np.ascontiguousarray(prev, dtype=np.float64)
        g = np.ascontiguousarray(grads, dtype=np.float64)
        o = np.ascontiguousarray(orders, dtype=np.int32)
        c = np.ascontiguousarray(cand, dtype=np.float64)
        f = C.c_int32()
        self._check(self.lib.orc_criterion_flags(self._h, int(p), _p(pv, C.c_double), _p(g, C.c_double),
                                                 _p(o, C.c_int32), _p(c, C.c_double), C.byref(f)),
                    "orc_criterion_flags")
        return bool(f.value)

    def update_volumes(self, sweeps=1):
        self._check(self.lib.orc_update_volumes(self._h, int(sweeps)), "orc_update_volumes")

    def volumes(self):
        out = np.zeros(self.n, dtype=np.float64)
        self._check(self.lib.orc_download_volumes(self._h, _p(out, C.c_double)), "orc_download_volumes")
        return out

    def features(self):
        """Stencil features of the learned troubled-point predictor (N x 24, FP32) of the current state."""
        out = np.zeros((self.n, 24), dtype=np.float32)
        self._check(self.lib.orc_features(self._h, _p(out, C.c_float)), "orc_features")
        return out

    def set_prelowered(self, mask):
        """Particles the next step pre-lowers by one order (None: none)."""
        if mask is None:
            self._check(self.lib.orc_set_prelowered(self._h, None), "orc_set_prelowered")
            return
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        self._check(self.lib.orc_set_prelowered(self._h, _p(m, C.c_uint8)), "orc_set_prelowered")

    def apply_bcs(self, buf):
        b = np.ascontiguousarray(buf, dtype=np.float64).copy()
        self._check(self.lib.orc_apply_bcs(self._h, _p(b, C.c_double)), "orc_apply_bcs")
        return b
