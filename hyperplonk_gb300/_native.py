"""ctypes binding of libhp_cuda.so (the C ABI in include/hp_cuda.h).

This is the Python counterpart of the reference's Rust FFI block
(backend/src/ascend910b3/ffi.rs:34-173).  Loading fails loudly when the
library has not been built: there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes
import pathlib

_LIB_PATH = pathlib.Path(__file__).resolve().parent / "_build" / "libhp_cuda.so"

c_size = ctypes.c_size_t
c_u8p = ctypes.POINTER(ctypes.c_uint8)
c_voidp = ctypes.c_void_p
c_voidpp = ctypes.POINTER(ctypes.c_void_p)
c_sizep = ctypes.POINTER(ctypes.c_size_t)


class Status(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("native_code", ctypes.c_int32)]


class MsmTuning(ctypes.Structure):
    """HpCudaMsmTuning (include/hp_cuda.h)."""
    _fields_ = [("size", ctypes.c_uint64), ("mode", ctypes.c_uint32), ("window_bits", ctypes.c_uint32),
                ("segment", ctypes.c_uint32), ("chunk", ctypes.c_uint32), ("model_ms", ctypes.c_double),
                ("tuned_ms", ctypes.c_double)]


class RoundTuning(ctypes.Structure):
    """HpCudaRoundTuning (include/hp_cuda.h)."""
    _fields_ = [("pairs", ctypes.c_uint64), ("kernel", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("default_kernel", ctypes.c_uint32), ("default_blocks_per_sm", ctypes.c_uint32),
                ("default_us", ctypes.c_double), ("tuned_us", ctypes.c_double)]


class RuntimeCounters(ctypes.Structure):
    """HpCudaRuntimeCounters (include/hp_cuda.h)."""
    _fields_ = [(name, ctypes.c_uint64) for name in (
        "device_allocs", "host_allocs", "pool_allocs", "pool_alloc_bytes", "frees", "h2d_copies", "h2d_bytes",
        "d2h_copies", "d2h_bytes", "d2d_copies", "d2d_bytes", "other_copies", "other_bytes", "memsets", "syncs",
        "injected_failures")]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


INJECT_NONE, INJECT_POOL_ALLOCATION, INJECT_SYNCHRONIZE = 0, 1, 2


# name -> argument types (all return Status)
SIGNATURES: dict[str, list] = {
    "hp_cuda_v1_context_create": [ctypes.c_int32, c_voidpp],
    "hp_cuda_v1_context_destroy": [c_voidp],
    "hp_cuda_v1_buffer_retire": [c_voidp, c_voidp],
    "hp_cuda_v1_context_stream": [c_voidp, c_voidpp],
    "hp_cuda_v1_mle_upload": [c_voidp, c_size, c_u8p, c_size, c_voidpp],
    "hp_cuda_v1_mle_upload_many": [c_voidp, c_size, ctypes.POINTER(c_u8p), c_size, c_size, c_voidpp],
    "hp_cuda_v1_mle_upload_async": [c_voidp, c_size, ctypes.POINTER(c_u8p), c_size, c_size, c_voidpp],
    "hp_cuda_v1_mle_upload_wait": [c_voidp, c_voidpp, c_size],
    "hp_cuda_v1_mle_download": [c_voidp, c_voidp, c_size, c_u8p, c_size],
    "hp_cuda_v1_mle_linear_combination": [c_voidp, c_size, c_voidpp, c_u8p, c_size, c_voidpp],
    "hp_cuda_v1_mle_evaluate": [c_voidp, c_voidp, c_size, c_u8p, c_u8p],
    "hp_cuda_v1_mle_build_eq_x_r": [c_voidp, c_u8p, c_size, c_voidpp],
    "hp_cuda_v1_mle_compute_frac_poly": [c_voidp, c_size, c_voidpp, c_voidpp, c_size, c_voidpp],
    "hp_cuda_v1_mle_compute_product_poly": [c_voidp, c_voidp, c_size, c_voidpp],
    "hp_cuda_v1_mle_compute_nums_and_denoms": [c_voidp, c_size, c_u8p, c_u8p, c_voidpp, c_voidpp,
                                               c_voidpp, c_size, c_voidpp, c_voidpp],
    "hp_cuda_v1_mle_compute_product_factors": [c_voidp, c_voidp, c_voidp, c_size, c_voidpp, c_voidpp],
    "hp_cuda_v1_multilinear_kzg_params_create": [c_voidp, c_size, c_voidpp],
    "hp_cuda_v1_multilinear_kzg_params_upload_layer": [c_voidp, c_voidp, c_size, c_u8p, c_size],
    "hp_cuda_v1_multilinear_kzg_params_destroy": [c_voidp, c_voidp],
    "hp_cuda_v1_multilinear_kzg_commit": [c_voidp, c_voidp, c_voidp, c_size, c_u8p],
    "hp_cuda_v1_multilinear_kzg_multi_commit": [c_voidp, c_voidp, c_voidpp, c_sizep, c_size, c_u8p],
    "hp_cuda_v1_multilinear_kzg_open": [c_voidp, c_voidp, c_voidp, c_size, c_u8p, c_u8p, c_u8p],
    "hp_cuda_v1_sumcheck_prover_state_create": [c_voidp, c_size, c_size, c_voidpp, c_size, c_u8p,
                                                c_sizep, c_size, c_sizep, c_size, c_voidpp],
    "hp_cuda_v1_sumcheck_prover_state_round": [c_voidp, c_voidp, c_u8p, c_u8p, c_size],
    "hp_cuda_v1_sumcheck_prover_state_destroy": [c_voidp, c_voidp],
    "hp_cuda_v1_sumcheck_prover_state_final_evaluations": [c_voidp, c_voidp, c_u8p, c_u8p, c_size],
    "hp_cuda_v1_msm": [c_voidp, c_u8p, c_u8p, c_size, c_u8p],
    "hp_cuda_v1_batch_msm": [c_voidp, c_voidp, c_size, c_voidpp, c_sizep, c_size, c_u8p],
    "hp_cuda_v1_batch_sumcheck_round": [c_voidp, c_voidpp, c_voidpp, c_voidpp, c_sizep, c_size],
    "hp_cuda_v1_mle_evaluate_noalloc": [c_voidp, c_size, c_u8p, c_u8p, c_voidp],
    "hp_cuda_v1_mle_evaluate_many": [c_voidp, c_size, c_voidpp, c_sizep, c_u8p, c_u8p],
    "hp_cuda_v1_context_profile": [c_voidp, ctypes.c_int32],
    "hp_cuda_v1_context_profile_read": [c_voidp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_uint64)],
    "hp_cuda_v1_kernel_launch_count": [ctypes.POINTER(ctypes.c_uint64)],
    "hp_cuda_v1_fixture_random_fr": [ctypes.c_uint64, ctypes.c_uint64, c_size, c_u8p],
    "hp_cuda_v1_srs_generate": [c_voidp, c_size, ctypes.c_uint64, c_u8p, c_size],
    "hp_cuda_v1_fixture_vanilla_plonk": [ctypes.c_uint64, c_size, c_u8p, c_u8p, c_u8p],
    "hp_cuda_v1_fixture_vanilla_plonk_witness": [ctypes.c_uint64, ctypes.c_uint64, c_size, c_u8p],
    "hp_cuda_v1_fixture_vanilla_plonk_wired": [ctypes.c_uint64, c_size, c_u8p, c_u8p, c_u8p],
    "hp_cuda_v1_context_memory": [c_voidp, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)],
    "hp_cuda_v1_debug_runtime_counters": [ctypes.POINTER(RuntimeCounters)],
    "hp_cuda_v1_debug_inject_failure": [ctypes.c_int32, ctypes.c_uint64],
    "hp_host_v1_merlin_new": [c_u8p, c_size, c_voidpp],
    "hp_host_v1_merlin_append": [c_voidp, c_u8p, c_size, c_u8p, c_size],
    "hp_host_v1_merlin_challenge": [c_voidp, c_u8p, c_size, c_u8p, c_size],
    "hp_host_v1_merlin_clone": [c_voidp, c_voidpp],
    "hp_host_v1_merlin_free": [c_voidp],
    "hp_host_v1_keccak_f1600": [c_u8p],
    "hp_cuda_v1_sumcheck_prove_rounds": [c_voidp, c_voidp, c_voidp, c_size, c_u8p, c_u8p],
    "hp_cuda_v1_msm_autotune": [c_voidp, c_voidp, c_sizep, c_size, ctypes.c_int32, ctypes.POINTER(MsmTuning)],
    "hp_cuda_v1_msm_tuning_query": [ctypes.c_int32, c_size, ctypes.POINTER(ctypes.c_uint32)],
    "hp_cuda_v1_msm_tuning_save": [ctypes.c_char_p],
    "hp_cuda_v1_msm_tuning_load": [ctypes.c_char_p, ctypes.c_char_p],
    "hp_cuda_v1_msm_tuning_clear": [],
    "hp_cuda_v1_sumcheck_autotune": [c_voidp, c_voidp, ctypes.POINTER(RoundTuning), c_size, c_sizep],
    "hp_cuda_v1_sumcheck_route_query": [c_size, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_uint32)],
}

_lib = None


def library_path() -> pathlib.Path:
    return _LIB_PATH


def load() -> ctypes.CDLL:
    """Load libhp_cuda.so and bind every declared entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise RuntimeError(
            f"{_LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA backend has no CPU fallback)")
    lib = ctypes.CDLL(str(_LIB_PATH))
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue  # entry not compiled into this build; calling it raises AttributeError
        fn.argtypes = argtypes
        fn.restype = Status
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    lib = load()
    return [n for n in SIGNATURES if getattr(lib, n, None) is not None]


def buf(data) -> ctypes.Array:
    """A ctypes uint8 view of a bytes-like object (no copy for bytearray/numpy)."""
    if data is None:
        return None
    if isinstance(data, (bytes,)):
        return ctypes.cast(ctypes.c_char_p(data), c_u8p)
    import numpy as np
    arr = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8)) if not isinstance(data, np.ndarray) else data
    return arr.ctypes.data_as(c_u8p)


def runtime_counters() -> dict:
    """The library's CUDA runtime call counters (hp_cuda_v1_debug_runtime_counters)."""
    from .errors import check_status
    c = RuntimeCounters()
    check_status(load().hp_cuda_v1_debug_runtime_counters(ctypes.byref(c)), "debug_runtime_counters")
    return c.as_dict()


def inject_failure(what: int, nth: int) -> None:
    """Arms (nth >= 1) or disarms (nth = 0) an injected failure
    (hp_cuda_v1_debug_inject_failure)."""
    from .errors import check_status
    check_status(load().hp_cuda_v1_debug_inject_failure(what, nth), "debug_inject_failure")

