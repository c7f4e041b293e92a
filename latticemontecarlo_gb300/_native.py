"""ctypes binding of the C ABI in ``include/lmc_gb300.h``.

The shared library is built in-tree (``latticemontecarlo_gb300/liblmc_gb300.so``)
by :mod:`latticemontecarlo_gb300.build`. There is no fallback: importing this
module without the library raises, and every non-zero status from the library
raises :class:`LmcError` carrying ``lmc_last_error()``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "liblmc_gb300.so"

LMC_OK = 0
LMC_ERR_INVALID_ARGUMENT = 1
LMC_ERR_OUT_OF_RANGE = 2
LMC_ERR_IO = 3
LMC_ERR_CUDA = 4
LMC_ERR_NO_DEVICE = 5
LMC_ERR_NUMERIC = 6
LMC_ERR_STOPPED = 7
LMC_ERR_UNSUPPORTED = 8

LMC_BARRIER_QUARTIC = 0
LMC_BARRIER_E0 = 1
LMC_RNG_MT19937_64 = 0
LMC_RNG_PHILOX = 1
LMC_EVAL_SPARSE = 0
LMC_FEATURES_ONEHOT = 0
LMC_FEATURES_SOLUTE = 1
LMC_EVAL_DENSE = 1
LMC_RATES_FP32 = 0
LMC_RATES_FP64 = 1
LMC_CMC_REFERENCE_BATCH = 0
LMC_CMC_THROUGHPUT = 1


class LmcError(RuntimeError):
    """A non-zero lmc_status; ``code`` is the status value."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (lmc status {code})")
        self.code = code


class QuarticParams(C.Structure):
    _fields_ = [
        ("k_mmm", C.c_int), ("k_mm2", C.c_int),
        ("mu_x_mmm", C.POINTER(C.c_double)), ("sigma_x_mmm", C.POINTER(C.c_double)),
        ("mu_x_mm2", C.POINTER(C.c_double)), ("sigma_x_mm2", C.POINTER(C.c_double)),
        ("u_mmm", C.POINTER(C.c_double)), ("u_mm2", C.POINTER(C.c_double)),
        ("theta_d", C.POINTER(C.c_double)), ("theta_ks", C.POINTER(C.c_double)),
        ("mu_d", C.c_double), ("sigma_d", C.c_double), ("mu_ks", C.c_double), ("sigma_ks", C.c_double),
    ]


class E0Params(C.Structure):
    _fields_ = [
        ("k_mmm", C.c_int),
        ("mu_x_mmm", C.POINTER(C.c_double)), ("sigma_x_mmm", C.POINTER(C.c_double)),
        ("u_mmm", C.POINTER(C.c_double)), ("theta_e0", C.POINTER(C.c_double)),
        ("mu_e0", C.c_double), ("sigma_e0", C.c_double),
    ]


class KmcOptions(C.Structure):
    _fields_ = [
        ("rng", C.c_int), ("seed", C.c_uint64), ("barrier_kind", C.c_int), ("rate_corrector", C.c_int),
        ("tt_time", C.POINTER(C.c_double)), ("tt_temp", C.POINTER(C.c_double)), ("tt_len", C.c_int),
        ("warps_per_replica", C.c_int), ("replicas_per_block", C.c_int), ("evaluation", C.c_int),
        ("early_stop", C.c_int), ("chain", C.c_int), ("rates", C.c_int),
    ]


class KmcStep(C.Structure):
    _fields_ = [
        ("vacancy", C.c_int64), ("target", C.c_int64), ("selected", C.c_int32), ("slot", C.c_int32),
        ("ea", C.c_double), ("de", C.c_double), ("total_rate", C.c_double), ("time", C.c_double),
        ("energy", C.c_double),
    ]


class CmcOptions(C.Structure):
    _fields_ = [("mode", C.c_int), ("seed", C.c_uint64), ("batch", C.c_int), ("candidates", C.c_int),
                ("energy_trace", C.POINTER(C.c_double))]


_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_I32P = C.POINTER(C.c_int32)
_I8P = C.POINTER(C.c_int8)
_DP = C.POINTER(C.c_double)
_U64P = C.POINTER(C.c_uint64)

# name -> (restype, argtypes); every symbol declared in include/lmc_gb300.h
SIGNATURES = {
    "lmc_strerror": (C.c_char_p, [C.c_int]),
    "lmc_last_error": (C.c_char_p, []),
    "lmc_version": (C.c_char_p, []),
    "lmc_model_create": (C.c_int, [C.POINTER(C.c_char_p), C.c_int, C.POINTER(_P)]),
    "lmc_model_load_json": (C.c_int, [C.c_char_p, C.POINTER(C.c_char_p), C.c_int, C.POINTER(_P)]),
    "lmc_model_destroy": (None, [_P]),
    "lmc_model_num_species": (C.c_int, [_P]),
    "lmc_model_species_code": (C.c_int, [_P, C.c_char_p]),
    "lmc_model_alphabet": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "lmc_model_layout": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "lmc_model_feature_orbit_sizes": (C.c_int, [_P, C.c_int, _I32P]),
    "lmc_model_set_base_theta": (C.c_int, [_P, _DP, C.c_int]),
    "lmc_model_set_quartic": (C.c_int, [_P, C.c_char_p, C.POINTER(QuarticParams)]),
    "lmc_model_set_e0": (C.c_int, [_P, C.c_char_p, C.POINTER(E0Params)]),
    "lmc_geom_neighbors": (C.c_int, [C.c_int, C.c_int64, _I64P]),
    "lmc_geom_pair_lists": (C.c_int, [C.c_int, C.c_int64, C.c_int64, _I64P, _I64P, _I64P]),
    "lmc_geom_site_list": (C.c_int, [C.c_int, C.c_int64, _I64P]),
    "lmc_geom_mapping_sizes": (C.c_int, [C.POINTER(C.c_int)]),
    "lmc_geom_env_mapping": (C.c_int, [C.c_int, _I32P, C.c_int, C.POINTER(C.c_int)]),
    "lmc_host_encode_pair": (C.c_int, [_P, C.c_int, _I8P, C.c_int64, C.c_int64, _I32P, _I32P, _I32P, _I32P, _I32P]),
    "lmc_ctx_create": (C.c_int, [_P, C.c_int, C.POINTER(_P)]),
    "lmc_ctx_destroy": (None, [_P]),
    "lmc_ctx_synchronize": (C.c_int, [_P]),
    "lmc_ctx_set_lattices": (C.c_int, [_P, C.c_int, _I32P, _I8P]),
    "lmc_ctx_get_lattices": (C.c_int, [_P, _I8P]),
    "lmc_ctx_total_sites": (C.c_int64, [_P]),
    "lmc_ctx_replica_offset": (C.c_int64, [_P, C.c_int]),
    "lmc_ctx_species_device_ptr": (_P, [_P]),
    "lmc_barrier_batch": (C.c_int, [_P, C.c_int, C.c_int, _I64P, C.c_int, _DP, _DP, _DP, _DP]),
    "lmc_barrier_batch_device": (C.c_int, [_P, C.c_int, C.c_int, _P, C.c_int, _P, _P]),
    "lmc_encode_batch": (C.c_int, [_P, C.c_int, _I64P, C.c_int, _I32P, _I32P, _I32P, _I32P, _I32P]),
    "lmc_de_pairs": (C.c_int, [_P, C.c_int, _I64P, C.c_int, _DP]),
    "lmc_energy": (C.c_int, [_P, C.c_int, _DP, _I64P]),
    "lmc_energy_noalloc": (C.c_int, [_P, _P, C.c_int, _P]),
    "lmc_fastmath_check": (C.c_int, [_P, C.c_int, _DP, C.c_int64, _DP, _DP]),
    "lmc_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(_P)]),
    "lmc_mlp_destroy": (None, [_P]),
    "lmc_mlp_layout": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), _I64P]),
    "lmc_mlp_get_params": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "lmc_mlp_set_params": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "lmc_mlp_set_label_scale": (C.c_int, [_P, C.c_float, C.c_float]),
    "lmc_mlp_gradients": (C.c_int, [_P, _P, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float),
                                    C.POINTER(C.c_float)]),
    "lmc_mlp_train": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_uint64,
                                C.POINTER(C.c_float)]),
    "lmc_mlp_predict": (C.c_int, [_P, _P, C.c_int64, _P, _P]),
    "lmc_mlp_set_inference_path": (C.c_int, [_P, C.c_int]),
    "lmc_mlp_set_train_path": (C.c_int, [_P, C.c_int]),
    "lmc_surrogate_set_encoding": (C.c_int, [_P, C.c_int]),
    "lmc_surrogate_feature_count": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "lmc_surrogate_dataset": (C.c_int, [_P, C.c_uint64, C.c_int64, C.c_double, C.c_double, C.c_int, C.c_int, _P, _P,
                                        _P, _P]),
    "lmc_surrogate_features": (C.c_int, [_P, C.c_int, _P, C.c_int, C.c_int, _P]),
    "lmc_surrogate_predict_device": (C.c_int, [_P, _P, C.c_int, _P, C.c_int, _P, _P]),
    "lmc_surrogate_barrier_batch_device": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, C.c_int, C.c_float, _P, _P,
                                                     C.POINTER(C.c_int)]),
    "lmc_kmc_init": (C.c_int, [_P, _DP, C.POINTER(KmcOptions)]),
    "lmc_kmc_run": (C.c_int, [_P, C.c_uint64, C.c_int, C.POINTER(KmcStep), _DP]),
    "lmc_kmc_get_state": (C.c_int, [_P, _I64P, _U64P, _DP, _DP]),
    "lmc_kmc_get_escaped": (C.c_int, [_P, C.POINTER(C.c_uint8)]),
    "lmc_last_run_ms": (C.c_int, [_P, _DP]),
    "lmc_kmc_launch_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), _I64P]),
    "lmc_kmc_run_graph": (C.c_int, [_P, C.c_uint64, C.c_int]),
    "lmc_sa_init": (C.c_int, [_P, C.c_int, C.c_uint64, C.c_uint64, C.c_double, C.c_double]),
    "lmc_site_jump_energetics": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_double, _I64P, C.c_int64, _DP, _DP,
                                           _I64P, _DP, _DP]),
    "lmc_site_de_batch": (C.c_int, [_P, C.c_int, _I64P, C.POINTER(C.c_int8), C.POINTER(C.c_int8), C.c_int64,
                                    C.c_int64, C.c_int, _DP]),
    "lmc_exit_time_energies": (C.c_int, [_P, C.c_int, C.c_int, _DP, _DP, _DP]),
    "lmc_ctx_set_barrier_evaluation": (C.c_int, [_P, C.c_int]),
    "lmc_exit_time_clusters": (C.c_int, [_P, C.c_int, C.c_int, C.c_double, _I64P, _I64P, C.c_int64, _DP, _DP, _I64P,
                                         _DP, _DP]),
    "lmc_solute_clusters": (C.c_int, [_P, C.c_int, C.c_int, C.c_int64, C.c_int64, _DP, _I64P, _I64P]),
    "lmc_solute_cluster_get": (C.c_int, [_P, _I64P, _I64P, _DP]),
    "lmc_sa_run": (C.c_int, [_P, C.c_uint64, _P]),
    "lmc_sa_get_state": (C.c_int, [_P, _U64P, _DP, _DP, _DP]),
    "lmc_kmc_multi_init": (C.c_int, [_P, _DP, C.c_uint64, C.c_int, C.c_int]),
    "lmc_kmc_multi_run": (C.c_int, [_P, C.c_uint64, C.c_int, C.POINTER(KmcStep)]),
    "lmc_kmc_multi_slots": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "lmc_kmc_multi_get_state": (C.c_int, [_P, _I64P, _U64P, _DP, _DP]),
    "lmc_kmc_multi_set_rates": (C.c_int, [_P, C.c_int]),
    "lmc_kmc_multi_surrogate_run": (C.c_int, [_P, _P, C.c_uint64, C.c_float, C.POINTER(KmcStep), _DP, _U64P]),
    "lmc_cmc_rounds": (C.c_int, [_P, _U64P]),
    "lmc_kmc_autotune": (C.c_int, [_P, C.c_uint64, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "lmc_cmc_run": (C.c_int, [_P, C.c_int, C.c_double, C.c_uint64, C.POINTER(CmcOptions), _DP, _U64P, _U64P]),
    "lmc_request_stop": (C.c_int, [_P, C.c_int]),
}


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(status: int) -> None:
    if status != LMC_OK:
        raise LmcError(status, lib.lmc_last_error().decode())


def ptr(arr, ctype):
    """ctypes pointer to a contiguous numpy array."""
    return arr.ctypes.data_as(C.POINTER(ctype))


def cstrings(names):
    arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
    return arr
