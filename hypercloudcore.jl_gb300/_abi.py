"""ctypes mirror of include/hcc.h (structures, enums and prototypes)."""
from __future__ import annotations

import ctypes as C

HCC_ABI_VERSION = 1
HCC_MAX_DIM = 3
HCC_MAX_VARS = 16
HCC_MAX_TAGS = 16
HCC_NOALLOC_MAX_PARTICLES = 65536 * 256

# hcc_status
HCC_OK, HCC_ERR_INVALID, HCC_ERR_CAPACITY, HCC_ERR_CUDA, HCC_ERR_STATE, HCC_ERR_NONFINITE, HCC_ERR_TIMEOUT, \
    HCC_ERR_UNSUPPORTED = range(8)
STATUS_NAMES = ["HCC_OK", "HCC_ERR_INVALID", "HCC_ERR_CAPACITY", "HCC_ERR_CUDA", "HCC_ERR_STATE",
                "HCC_ERR_NONFINITE", "HCC_ERR_TIMEOUT", "HCC_ERR_UNSUPPORTED"]
# hcc_pde_kind
PDE_ADVECTION, PDE_EULER, PDE_BGK = 0, 1, 2
# hcc_precision
FP64, FP32 = 0, 1
# hcc_mood_criterion
MOOD_NONE, MOOD_U1, MOOD_PAD, MOOD_ONLY, MOOD_U2 = 0, 1, 2, 3, 4
FLUXES = {"rusanov": 0, "aligned": 1}
# hcc_mood_strategy
EPD_NONE, EPD0, EPD1, EPD2, STRICT_EPD0 = 0, 1, 2, 3, 4
# hcc_tableau
TABLEAUS = {
    "RK1_Euler": 0, "RK2_SSP": 1, "RK2_Ralston": 2, "RK3_SSP": 3, "RK4_Classical": 4, "RK4_SSP": 5,
    "IMEX_Euler": 6, "IMEX_ARS233": 7, "IMEX_ARS222": 8, "IMEX_PRSSP3": 9, "IMEX_SSP2332": 10,
}
# hcc_scheme / hcc_limiter
SCHEME_MUSCL, SCHEME_WENO, SCHEME_CENTRAL, SCHEME_UPWIND = 0, 1, 2, 3
UPWIND_ALGORITHMS = {"Tiwari": 1, "Praveen": 2}
LIMITERS = {"none": 0, "bj_soft": 1, "bj_hard": 2, "vk_soft": 3, "vk_hard": 4}
# hcc_bc_kind
BC_KEEP, BC_DIRICHLET, BC_OUTFLOW = 0, 1, 2


class HccConfig(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("dim", C.c_int32), ("n_vars", C.c_int32), ("pde", C.c_int32),
        ("precision", C.c_int32), ("muscl_order", C.c_int32), ("div_order", C.c_int32),
        ("mood_criterion", C.c_int32), ("mood_strategy", C.c_int32), ("tableau", C.c_int32),
        ("mood_substeps", C.c_int32), ("periodic", C.c_int32 * HCC_MAX_DIM),
        ("bc_by_tag", C.c_int32 * HCC_MAX_TAGS), ("max_mood_iterations", C.c_int32),
        ("scheme", C.c_int32), ("limiter", C.c_int32), ("slot_capacity", C.c_int32), ("flux", C.c_int32),
        ("reset_orders_per_stage", C.c_int32), ("upwind_algorithm", C.c_int32), ("moment_correction", C.c_int32),
        ("reserved_i", C.c_int32 * 1),
        ("dx", C.c_double * HCC_MAX_DIM), ("radius", C.c_double), ("weight_alpha", C.c_double),
        ("canvas_min", C.c_double * HCC_MAX_DIM), ("canvas_max", C.c_double * HCC_MAX_DIM),
        ("domain_min", C.c_double * HCC_MAX_DIM), ("domain_max", C.c_double * HCC_MAX_DIM),
        ("mood_delta", C.c_double), ("velocity", (C.c_double * HCC_MAX_VARS) * HCC_MAX_DIM),
        ("gamma", C.c_double), ("bgk_epsilon", C.c_double), ("bgk_macro_velocity", C.c_double * HCC_MAX_DIM),
        ("bgk_coefficient", C.c_double), ("bgk_interior_factor", C.c_double), ("u2_plateau", C.c_double),
        ("u2_ratio", C.c_double), ("reserved_d", C.c_double * 6),
    ]


class HccCounters(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64), ("n_interior", C.c_int64), ("max_neighbours", C.c_int32),
        ("min_neighbours_interior", C.c_int32), ("total_neighbours", C.c_int64), ("mood_iterations", C.c_int64),
        ("mood_flagged", C.c_int64), ("inadmissible", C.c_int64), ("kernel_launches", C.c_int64),
        ("steps", C.c_int64), ("kernel_launches_total", C.c_int64),
        ("graph_steps", C.c_int64), ("predicted", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class HccMover(C.Structure):
    _fields_ = [("kind", C.c_int32), ("full_search_per_stage", C.c_int32), ("alpha", C.c_double),
                ("velocity", C.c_double * HCC_MAX_DIM), ("omega", C.c_double * HCC_MAX_DIM),
                ("center", C.c_double * HCC_MAX_DIM), ("keep_volumes", C.c_int32), ("shepard_sweeps", C.c_int32)]


MOVERS = {"none": 0, "lagrangian": 1, "scaled": 2, "prescribed": 3}


HCC_MLP_FEATURES = 24
HCC_MLP_HIDDEN = 64
HCC_MLP_NPARAMS = 64 * 24 + 64 + 64 * 64 + 64 + 64 + 1


class HccMlpConfig(C.Structure):
    _fields_ = [("capacity", C.c_int64), ("neg_keep", C.c_double), ("seed", C.c_uint64), ("lr", C.c_double),
                ("beta1", C.c_double), ("beta2", C.c_double), ("adam_eps", C.c_double), ("pos_weight", C.c_double),
                ("reserved", C.c_double * 4)]


class HccKernelTimes(C.Structure):
    _fields_ = [("gather_ms", C.c_double), ("gather_launches", C.c_int64), ("flux_ms", C.c_double),
                ("flux_launches", C.c_int64), ("recompute_ms", C.c_double), ("recompute_launches", C.c_int64),
                ("steps", C.c_int64), ("predict_ms", C.c_double), ("predict_launches", C.c_int64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class HccTuning(C.Structure):
    _fields_ = [("flux_block", C.c_int32), ("gather_block", C.c_int32), ("list_blocks_per_sm", C.c_int32),
                ("drop_blocks_per_sm", C.c_int32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class HccTuneReport(C.Structure):
    _fields_ = [("best", HccTuning), ("default_ms", C.c_double), ("best_ms", C.c_double),
                ("candidates", C.c_int32), ("steps", C.c_int32)]


P = C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)

# (name, restype, argtypes) of every entry point of include/hcc.h
PROTOTYPES = [
    ("hcc_config_defaults", None, [C.POINTER(HccConfig)]),
    ("hcc_create", C.c_int, [C.POINTER(HccConfig), C.c_int64, C.POINTER(P)]),
    ("hcc_destroy", C.c_int, [P]),
    ("hcc_last_error", C.c_char_p, [P]),
    ("hcc_status_string", C.c_char_p, [C.c_int]),
    ("hcc_upload_cloud", C.c_int, [P, C.c_int64, _dp, _u8p, _i32p, _dp]),
    ("hcc_build_neighbours", C.c_int, [P]),
    ("hcc_download_neighbours", C.c_int, [P, _i32p, _i32p, _dp, _dp]),
    ("hcc_download_neighbours_of", C.c_int, [P, C.c_int64, C.POINTER(C.c_int64), C.c_int32, _i32p, _i32p, _dp, _dp]),
    ("hcc_prepare_geometry", C.c_int, [P]),
    ("hcc_download_geometry", C.c_int, [P, _dp, _u8p, _u8p]),
    ("hcc_upload_state", C.c_int, [P, _dp]),
    ("hcc_download_state", C.c_int, [P, _dp]),
    ("hcc_upload_state_f32", C.c_int, [P, _fp]),
    ("hcc_download_state_f32", C.c_int, [P, _fp]),
    ("hcc_time_step", C.c_int, [P, _dp]),
    ("hcc_compute_rhs", C.c_int, [P, _dp]),
    ("hcc_step", C.c_int, [P, C.c_double, C.c_double]),
    ("hcc_download_orders", C.c_int, [P, _i32p]),
    ("hcc_download_mood_flags", C.c_int, [P, _u8p]),
    ("hcc_get_counters", C.c_int, [P, C.POINTER(HccCounters)]),
    ("hcc_total_mass", C.c_int, [P, _dp]),
    ("hcc_set_profiling", C.c_int, [P, C.c_int]),
    ("hcc_set_step_graphs", C.c_int, [P, C.c_int]),
    ("hcc_set_mover", C.c_int, [P, C.POINTER(HccMover)]),
    ("hcc_download_positions", C.c_int, [P, C.POINTER(C.c_double)]),
    ("hcc_save_snapshot", C.c_int, [P, C.c_char_p]),
    ("hcc_load_snapshot", C.c_int, [P, C.c_char_p]),
    ("hcc_get_kernel_times", C.c_int, [P, C.POINTER(HccKernelTimes), C.c_int]),
    ("hcc_cfl_time_step_noalloc", C.c_int, [C.POINTER(HccConfig), C.c_int64, C.c_int64, P, P, P, P, P, P, _dp]),
    ("hcc_upload_batch", C.c_int, [P, C.c_int32, C.POINTER(C.c_int64), _dp, _u8p, _i32p, _dp, _dp, _dp]),
    ("hcc_batch_total_mass", C.c_int, [P, _dp]),
    ("hcc_batch_time_steps", C.c_int, [P, _dp]),
    ("hcc_batch_step", C.c_int, [P, C.c_double, _dp]),
    ("hcc_batch_layout", C.c_int, [C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_int64), _dp, _dp, _dp]),
    ("hcc_update_volumes", C.c_int, [P, C.c_int32]),
    ("hcc_download_volumes", C.c_int, [P, _dp]),
    ("hcc_build_info", C.c_char_p, []),
    ("hcc_fp64_fma_rate", C.c_int, [_dp]),
    ("hcc_set_tile_staging", C.c_int, [P, C.c_int32]),
    ("hcc_get_tile_staging", C.c_int, [P, _i32p, C.POINTER(C.c_int64), _i32p]),
    ("hcc_get_tuning", C.c_int, [P, C.POINTER(HccTuning)]),
    ("hcc_set_tuning", C.c_int, [P, C.POINTER(HccTuning)]),
    ("hcc_autotune", C.c_int, [P, C.c_double, C.c_int32, C.POINTER(HccTuneReport)]),
    ("hcc_mlp_create", C.c_int, [C.POINTER(HccMlpConfig), C.POINTER(P)]),
    ("hcc_mlp_destroy", None, [P]),
    ("hcc_mlp_last_error", C.c_char_p, [P]),
    ("hcc_mlp_get_params", C.c_int, [P, _fp, _fp]),
    ("hcc_mlp_set_params", C.c_int, [P, _fp, _fp]),
    ("hcc_mlp_collect", C.c_int, [P, P]),
    ("hcc_mlp_add_rows", C.c_int, [P, _fp, _u8p, C.c_int64]),
    ("hcc_mlp_rows", C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("hcc_mlp_clear", C.c_int, [P]),
    ("hcc_mlp_fit_norm", C.c_int, [P, C.c_double]),
    ("hcc_mlp_train", C.c_int, [P, C.c_int64, C.c_int64, C.c_double, _dp]),
    ("hcc_mlp_evaluate", C.c_int, [P, C.c_double, C.c_double, C.POINTER(C.c_int64)]),
    ("hcc_mlp_loss_grad", C.c_int, [P, _fp, _u8p, C.c_int64, _fp, _dp]),
    ("hcc_mlp_predict_rows", C.c_int, [P, _fp, C.c_int64, _fp]),
    ("hcc_set_predictor", C.c_int, [P, P, C.c_double]),
    ("hcc_set_feature_capture", C.c_int, [P, C.c_int]),
    ("hcc_download_features", C.c_int, [P, _fp]),
    ("hcc_download_predicted", C.c_int, [P, _u8p]),
    ("hcc_synchronize", C.c_int, [P]),
    ("hcc_stream", P, [P]),
]


def bind(lib: C.CDLL, prototypes=PROTOTYPES) -> C.CDLL:
    for name, res, args in prototypes:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
