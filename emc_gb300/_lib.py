"""ctypes binding of libemc_gb300.so (the C ABI declared in include/emc_gb300.h).

The library is loaded from emc_gb300/_build/ (built in-tree by
emc_gb300.build).  There is no fallback: if the library is missing, loading
raises, so nothing can silently run on the CPU instead of the CUDA path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_BUILD = Path(__file__).resolve().parent / "_build"
LIB_PATH = _BUILD / "libemc_gb300.so"

EMC_OK = 0
ERRORS = {
    -1: "EMC_ERR_INVALID",
    -2: "EMC_ERR_CUDA",
    -3: "EMC_ERR_TIMEOUT",
    -4: "EMC_ERR_NONFINITE",
    -5: "EMC_ERR_INTERNAL",
    -6: "EMC_ERR_NOMEM",
    -7: "EMC_ERR_UNSUPPORTED",
}

DIFF_ABSOLUTE, DIFF_POISSON, DIFF_RELATIVE, DIFF_TRUE_POISSON = 0, 1, 2, 3
INTERP_NEAREST, INTERP_TRILINEAR = 0, 1
PREC_FP32, PREC_MIXED = 0, 1
INSERT_ATOMIC, INSERT_DETERMINISTIC, INSERT_SORTED = 0, 1, 2

P = C.c_void_p
I = C.c_int
F = C.c_float
D = C.c_double


class PlanDesc(C.Structure):
    _fields_ = [
        ("side", I), ("n_images", I), ("n_rot", I), ("diff", I), ("interp", I),
        ("precision", I), ("insert_mode", I), ("known_intensity", I),
        ("normalize_images", I), ("blur_sigma", F),
    ]


class IterStats(C.Structure):
    _fields_ = [
        ("total_loglik", D), ("model_mean_before", D), ("captured_mass", D),
        ("bad_pairs", I), ("reserved", I),
    ]


class PruneInfo(C.Structure):
    _fields_ = [
        ("pruned", I), ("fallback", I), ("active_fraction", D), ("core_fraction", D),
        ("margin_mass", D),
        ("nn_angle", D), ("pruned_iterations", C.c_longlong),
        ("fallback_iterations", C.c_longlong), ("full_iterations", C.c_longlong),
    ]


PATH_MAX = 512


class Config(C.Structure):
    """emc_config (the keys of the reference's Configuration)."""
    _fields_ = [
        ("model_side", I), ("read_stride", I), ("slice_chunk", I), ("N_images", I),
        ("max_iterations", I), ("rotations_n", I), ("wavelength", D), ("pixel_size", D),
        ("detector_size", I), ("detector_distance", D), ("sigma_start", D), ("sigma_final", D),
        ("sigma_half_life", I), ("diff", I), ("blur_image", I), ("blur_sigma", D),
        ("mask_file", C.c_char * PATH_MAX), ("image_prefix", C.c_char * PATH_MAX),
        ("normalize_images", I), ("known_intensity", I), ("model_input", I),
        ("model_file", C.c_char * PATH_MAX), ("exclude_images", I), ("exclude_ratio", D),
        ("model_blur", D), ("isDebug", I), ("isOutput", I), ("output_loop", I),
        ("output_period", I), ("nGPUs", I),
    ]


# name -> (restype, argtypes); every function declared in include/emc_gb300.h.
SIGNATURES: dict[str, tuple] = {
    "emc_ctx_create": (I, [C.POINTER(P), I]),
    "emc_ctx_destroy": (I, [P]),
    "emc_ctx_device": (I, [P]),
    "emc_last_error": (C.c_char_p, [P]),
    "emc_set_stream": (I, [P, P]),
    "emc_get_stream": (P, [P]),
    "emc_sync": (I, [P]),
    "emc_kernel_launches": (C.c_longlong, [P]),
    "emc_rotation_count": (I, [I]),
    "emc_generate_rotations": (I, [I, P, P, I]),
    "emc_calculate_coordinates": (I, [I, F, F, F, P, P, P]),
    "emc_sigma_schedule": (F, [I, D, D, I]),
    "emc_get_slices": (I, [P, P, I, P, P, P, P, P, I, I, I]),
    "emc_update_scaling_full": (I, [P, P, P, P, P, I, I, I, I, I]),
    "emc_calculate_responsabilities": (I, [P, P, P, P, F, P, P, P, I, I, I, I, I]),
    "emc_max_vector": (I, [P, P, I, I, P]),
    "emc_respons_max_expf": (I, [P, P, P, I, I, P]),
    "emc_respons_max_expf_noalloc": (I, [P, P, I, I, P, P]),
    "emc_norm_respons_sumexpf": (I, [P, P, P, P, I, I]),
    "emc_log_sum_max": (I, [P, P, P, P, I]),
    "emc_update_slices": (I, [P, P, P, P, P, P, P, I, I, I, I, I, P, P, P, P, P, P]),
    "emc_divide_model_by_weight": (I, [P, I, P, P]),
    "emc_normalize_model": (I, [P, I, P, P]),
    "emc_model_max": (I, [P, P, I, P]),
    "emc_model_average": (I, [P, P, I, P]),
    "emc_blur_model": (I, [P, P, I, F]),
    "emc_reset_real": (I, [P, P, I]),
    "emc_copy_real_to_device": (I, [P, P, P, I]),
    "emc_copy_real_to_host": (I, [P, P, P, I]),
    "emc_copy_real_d2d": (I, [P, P, P, I, I]),
    "emc_copy_int_to_device": (I, [P, P, P, I]),
    "emc_allocate_real": (I, [P, C.POINTER(P), C.c_size_t]),
    "emc_allocate_int": (I, [P, C.POINTER(P), C.c_size_t]),
    "emc_mem_free": (I, [P, P]),
    "emc_config_defaults": (I, [P]),
    "emc_config_parse": (I, [C.c_char_p, P, C.c_char_p, I]),
    "emc_config_read": (I, [C.c_char_p, P, C.c_char_p, I]),
    "emc_plan_create": (I, [P, C.POINTER(PlanDesc), C.POINTER(P)]),
    "emc_plan_destroy": (I, [P]),
    "emc_plan_workspace_bytes": (C.c_size_t, [P]),
    "emc_plan_bind": (I, [P, P, P, P, P, P, P, P]),
    "emc_iterate": (I, [P, P, P, F, C.POINTER(IterStats)]),
    "emc_iterate_async": (I, [P, P, P, F]),
    "emc_random_rotations": (I, [C.c_ulonglong, I, P]),
    "emc_bin_images": (I, [P, P, P, I, I, I, I, I, P, P]),
    "emc_normalize_images": (I, [P, P, P, P, I, I]),
    "emc_mask_images": (I, [P, P, P, I, I]),
    "emc_model_init_radial": (I, [P, P, I, I, P]),
    "emc_model_init_orientations": (I, [P, P, P, I, I, P, P, P, P, P, P]),
    "emc_plan_wait": (I, [P, C.POINTER(IterStats)]),
    "emc_plan_capture": (I, [P, P, P]),
    "emc_plan_replay": (I, [P, F]),
    "emc_plan_set_pruning": (I, [P, I, F, F, I]),
    "emc_plan_prune_info": (I, [P, C.POINTER(PruneInfo)]),
    "emc_plan_pattern_order": (I, [P, P]),
    "emc_plan_rotation_order": (I, [P, P]),
    "emc_plan_best_quaternions": (I, [P, P]),
    "emc_plan_set_proposals": (I, [P, P, I, F, I]),
    "emc_proposal_create": (I, [P, C.c_ulonglong, C.POINTER(P)]),
    "emc_proposal_destroy": (I, [P]),
    "emc_proposal_param_count": (I, [P]),
    "emc_proposal_params": (I, [P, P, I]),
    "emc_proposal_set_data": (I, [P, P, P, I, I, I]),
    "emc_proposal_stats": (I, [P, P, I]),
    "emc_proposal_inputs": (I, [P, I, I, P]),
    "emc_proposal_loss_grad": (I, [P, P, I, P, C.POINTER(F), P]),
    "emc_proposal_train": (I, [P, P, P, I, I, I, F, C.c_ulonglong, I, P]),
    "emc_proposal_predict": (I, [P, P]),
    "emc_batch_create": (I, [P, P, P, I, C.POINTER(P)]),
    "emc_batch_run": (I, [P, P]),
    "emc_batch_wait": (I, [P, P]),
    "emc_batch_destroy": (I, [P]),
    "emc_plan_results": (I, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "emc_rank_estep": (I, [P, P, F, P, P]),
    "emc_rank_mstep": (I, [P, P, P, P]),
    "emc_model_from_sums": (I, [P, P, P, I, P, P]),
    "emc_plan_set_profiling": (I, [P, I]),
    "emc_plan_set_option": (I, [P, I, I]),
    "emc_plan_get_option": (I, [P, I, P]),
    "emc_plan_autotune": (I, [P, P, F, C.POINTER(I), C.POINTER(F)]),
    "emc_plan_time_likelihood": (I, [P, P, F, I, I, I, C.POINTER(F), C.POINTER(I)]),
    "emc_tc_gemm_selftest": (I, [P, P, P, P, I, I]),
    "emc_plan_phase_ms": (I, [P, P, I]),
}

_lib = None


def load() -> C.CDLL:
    """Loads the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} not built: run __graft_entry__.build()")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class EmcError(RuntimeError):
    pass
