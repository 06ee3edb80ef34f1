"""ctypes binding of libcdet_gb300.so (the C ABI in include/cdet_gb300.h).

There is no fallback: if the library is missing or does not load, every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB_PATH

CDET_OK = 0
CDET_ERR_INVALID = 1
CDET_ERR_STATE = 2
CDET_ERR_CUDA = 3
CDET_ERR_VALUE = 4

CONFIG_NONFINITE = 1
CONFIG_FPM_FALLBACK = 2
CONFIG_BAD_INPUT = 4

TWISTED_UP, TWISTED_DOWN, ORDINARY_UP, ORDINARY_DOWN = 0, 1, 2, 3
KIND_NAMES = ("twisted_up", "twisted_down", "ordinary_up", "ordinary_down")

# Every symbol include/cdet_gb300.h declares.
EXPORTED = (
    "cdet_create", "cdet_destroy", "cdet_upload_table", "cdet_bind_device_table",
    "cdet_alias_table", "cdet_reserve", "cdet_integrand_device", "cdet_all_subsets_device",
    "cdet_integrand_host", "cdet_all_subsets_host", "cdet_counters", "cdet_last_error",
    "cdet_last_launch_count", "cdet_profile_enable", "cdet_profile_read",
    "cdet_set_assembly", "cdet_prepare_split", "cdet_assemble_device",
    "cdet_integrand_device_noalloc", "cdet_diagonal_order1_density",
    "cdet_mcmcmc_create", "cdet_mcmcmc_run", "cdet_mcmcmc_end_warmup", "cdet_mcmcmc_state",
    "cdet_mcmcmc_destroy", "cdet_mcmcmc_set_histogram", "cdet_mcmcmc_learn_histogram", "cdet_mcmcmc_result",
    "cdet_mcmcmc_summary", "cdet_mcmcmc_estimates", "cdet_write_mcmcmc_checkpoint", "cdet_read_mcmcmc_checkpoint",
    "cdet_mcmcmc_save_checkpoints", "cdet_mcmcmc_load_checkpoints", "cdet_mcmcmc_launch_count", "cdet_set_all_subsets_form", "cdet_all_subsets_form_tuned", "cdet_load_chunks",
    "cdet_split_counters", "cdet_set_integrand_form", "cdet_integrand_form_tuned",
    "cdet_mcmcmc_set_green_reuse", "cdet_set_integrand_real",
)

ASSEMBLY_FP64 = 0
ASSEMBLY_SPLIT_BF16 = 1

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)


class McmcmcConfig(C.Structure):
    """cdet_mcmcmc_config (include/cdet_gb300.h)."""
    _fields_ = [("order_min", C.c_int32), ("order_max", C.c_int32), ("envelope_order", C.c_int32),
                ("lambda_adapt_interval", C.c_int32), ("lambda_adapt_rate", C.c_double)]


class HistogramConfig(C.Structure):
    """cdet_histogram_config (include/cdet_gb300.h)."""
    _fields_ = [("learning_steps", C.c_int32), ("tau_bins", C.c_int32), ("uniform_mix", C.c_double),
                ("pseudo_count", C.c_double)]


MAX_ENVELOPE = 24  # CDET_MCMCMC_MAX_ENVELOPE


class RunningStats(C.Structure):
    """cdet_running_stats: RunningStatsLongDouble in the host's long double."""
    _fields_ = [("count", C.c_uint64), ("mean", C.c_longdouble), ("m2", C.c_longdouble)]


class ChainResult(C.Structure):
    """cdet_mcmcmc_chain_result (MCMCMCChainResult)."""
    _fields_ = [("seed", C.c_uint64), ("warmup_proposed_steps", C.c_uint64),
                ("warmup_accepted_steps", C.c_uint64), ("production_proposed_steps", C.c_uint64),
                ("production_accepted_steps", C.c_uint64),
                ("warmup_chosen_counts", C.c_uint64 * (MAX_ENVELOPE + 1)),
                ("production_chosen_counts", C.c_uint64 * (MAX_ENVELOPE + 1)),
                ("warmup_retained_fraction_stats", RunningStats),
                ("production_retained_fraction_stats", RunningStats),
                ("order_signal_stats", RunningStats * (MAX_ENVELOPE + 1))]


class Checkpoint(C.Structure):
    """cdet_mcmcmc_checkpoint: one CDET_MCMCMC_CHAIN_CHECKPOINT_V1 file."""
    _fields_ = [("chain_index", C.c_uint64), ("seed", C.c_uint64), ("order_min", C.c_int32),
                ("order_max", C.c_int32), ("envelope_order", C.c_int32), ("normalization_order", C.c_int32),
                ("lambda_warmup_steps", C.c_int32), ("production_steps", C.c_int32), ("seed_mode", C.c_char * 16),
                ("rng_state", C.c_uint64 * 313), ("lambdas", C.c_double * (MAX_ENVELOPE + 1)),
                ("warmup_block_counts", C.c_uint64 * (MAX_ENVELOPE + 1)),
                ("vertices", (C.c_double * 4) * MAX_ENVELOPE), ("result", ChainResult)]


class DD(C.Structure):
    _fields_ = [("hi", C.c_double), ("lo", C.c_double)]


class DDScalars(C.Structure):
    """cdet_dd_scalars: the DoubleDouble parameters of the double-double integrand."""
    _fields_ = [(name, DD) for name in ("beta", "u", "alpha_up", "alpha_down", "tol_fpm", "fpm_shift",
                                        "z_eps0", "z_safety")]


INTEGRAND_REAL_DOUBLE = 0
INTEGRAND_REAL_DOUBLE_DOUBLE = 1


class RunInfo(C.Structure):
    """cdet_mcmcmc_run_info."""
    _fields_ = [("normalization_order", C.c_int32), ("lambda_warmup_steps", C.c_int32),
                ("production_steps", C.c_int32)]


class RuntimeScalars(C.Structure):
    _fields_ = [("n1", C.c_int32), ("n2", C.c_int32), ("cheb_nu", C.c_int32),
                ("cheb_nv", C.c_int32), ("beta", C.c_double), ("u", C.c_double),
                ("branch_eps", C.c_double), ("scale", C.c_double),
                ("diag_up_shift", C.c_double), ("diag_down_shift", C.c_double),
                ("tol_fpm", C.c_double), ("fpm_shift", C.c_double),
                ("z_eps0", C.c_double), ("z_safety", C.c_double)]


class TableView(C.Structure):
    _fields_ = [("upper_coeffs", C.c_void_p), ("lower_coeffs", C.c_void_p),
                ("upper_corners", C.c_void_p), ("lower_corners", C.c_void_p)]


_LIB = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads the library (once) and declares the prototypes."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with __graft_entry__.build() (nvcc, sm_103a); "
            "the CDet integrand has no CPU fallback")
    lib = C.CDLL(path)
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int
    lib.cdet_create.argtypes = [C.POINTER(RuntimeScalars), i32, C.POINTER(vp)]
    lib.cdet_destroy.argtypes = [vp]
    lib.cdet_destroy.restype = None
    lib.cdet_upload_table.argtypes = [vp, i32, C.POINTER(TableView), C.c_size_t, C.c_size_t]
    lib.cdet_bind_device_table.argtypes = [vp, i32, C.POINTER(TableView), C.c_size_t, C.c_size_t]
    lib.cdet_alias_table.argtypes = [vp, i32, i32]
    lib.cdet_reserve.argtypes = [vp, i64, i32]
    lib.cdet_integrand_device.argtypes = [vp, vp, vp, i64, i32, vp, vp, vp]
    lib.cdet_all_subsets_device.argtypes = [vp, vp, i32, i64, vp, vp, vp]
    lib.cdet_integrand_host.argtypes = [vp, vp, vp, i64, i32, vp, vp]
    lib.cdet_all_subsets_host.argtypes = [vp, vp, i32, i64, vp, vp]
    lib.cdet_counters.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.cdet_diagonal_order1_density.argtypes = [vp, C.c_double, C.c_double, _DP]
    _UP = C.POINTER(C.c_uint64)
    lib.cdet_mcmcmc_create.argtypes = [vp, C.POINTER(McmcmcConfig), C.c_int64, _UP, _DP, C.POINTER(vp)]
    lib.cdet_mcmcmc_run.argtypes = [vp, C.c_int, C.c_int64, _UP, _DP, _DP]
    lib.cdet_mcmcmc_end_warmup.argtypes = [vp]
    lib.cdet_mcmcmc_state.argtypes = [vp, _DP, _DP, _UP]
    lib.cdet_mcmcmc_destroy.argtypes = [vp]
    lib.cdet_mcmcmc_set_histogram.argtypes = [vp, C.c_int32, _DP, _DP, _DP]
    _LDP = C.POINTER(C.c_longdouble)
    lib.cdet_mcmcmc_result.argtypes = [vp, C.c_int64, C.POINTER(ChainResult)]
    lib.cdet_mcmcmc_summary.argtypes = [vp, C.c_int32, C.POINTER(RunningStats), _LDP]
    lib.cdet_mcmcmc_estimates.argtypes = [vp, C.c_double, C.c_double, _LDP, _LDP, _LDP, _LDP]
    lib.cdet_write_mcmcmc_checkpoint.argtypes = [C.c_char_p, C.POINTER(Checkpoint)]
    lib.cdet_read_mcmcmc_checkpoint.argtypes = [C.c_char_p, C.POINTER(Checkpoint)]
    lib.cdet_mcmcmc_save_checkpoints.argtypes = [vp, C.c_char_p, C.POINTER(RunInfo)]
    lib.cdet_mcmcmc_load_checkpoints.argtypes = [vp, C.c_char_p, C.POINTER(RunInfo), C.c_int,
                                                 C.POINTER(C.c_int64)]
    lib.cdet_set_all_subsets_form.argtypes = [vp, i32]
    lib.cdet_all_subsets_form_tuned.argtypes = [vp, i32, i32, i64, C.POINTER(C.c_int)]
    lib.cdet_set_integrand_form.argtypes = [vp, i32, i32, i32, i32]
    lib.cdet_mcmcmc_set_green_reuse.argtypes = [vp, i32]
    lib.cdet_set_integrand_real.argtypes = [vp, i32, C.POINTER(DDScalars)]
    lib.cdet_integrand_form_tuned.argtypes = [vp, i32, i32, i64] + [C.POINTER(C.c_int)] * 4
    lib.cdet_mcmcmc_launch_count.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.cdet_mcmcmc_learn_histogram.argtypes = [vp, C.POINTER(McmcmcConfig), C.POINTER(HistogramConfig), C.c_uint64,
                                                _DP, _DP, _DP, _DP]
    lib.cdet_load_chunks.argtypes = [vp, C.c_char_p, _DP]
    lib.cdet_last_error.restype = C.c_char_p
    lib.cdet_last_launch_count.argtypes = [vp]
    lib.cdet_integrand_device_noalloc.argtypes = [vp, vp, vp, i64, i32, vp, vp, vp]
    lib.cdet_set_assembly.argtypes = [vp, i32]
    lib.cdet_prepare_split.argtypes = [vp]
    lib.cdet_assemble_device.argtypes = [vp, vp, vp, i64, i32, vp, vp, vp, vp]
    lib.cdet_profile_enable.argtypes = [vp, i32]
    lib.cdet_profile_read.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.cdet_split_counters.argtypes = [vp, C.POINTER(C.c_uint64)]
    _LIB = lib
    return lib


def last_error() -> str:
    return load().cdet_last_error().decode()


def check(rc: int) -> None:
    if rc != CDET_OK:
        raise RuntimeError(last_error() or f"cdet call failed with code {rc}")
