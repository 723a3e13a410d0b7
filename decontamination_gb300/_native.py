"""ctypes binding of libsomgb.so (include/somgb.h).

The library is the only compute path: there is no CPU fallback. Loading fails
loudly when the library has not been built (``python -m
decontamination_gb300.build``), and every entry point's status is checked.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libsomgb.so')

SOMGB_OK = 0
SOMGB_ERR_INVALID = 1
SOMGB_ERR_CUDA = 2
SOMGB_ERR_WORKSPACE = 3
SOMGB_ERR_UNSUPPORTED = 4
SOMGB_ERR_TIMEOUT = 5

ALGO_FP32 = 0
ALGO_TC = 1
ALGO_AUTO = 2
ALGOS = {'fp32': ALGO_FP32, 'tc': ALGO_TC, 'auto': ALGO_AUTO}

OP_FIND_BMUS = 0
OP_COUNT_BMUS = 1
OP_ERRORS = 2
OP_EPOCH = 3

P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
D = ctypes.c_double
SZ = ctypes.c_size_t

# name -> argument types (all return int status unless listed in _RESTYPES)
SIGNATURES = {
    'somgb_version': [],
    'somgb_last_error': [ctypes.c_char_p, SZ],
    'somgb_workspace_bytes': [I32, I64, I64, I32, I32],
    'somgb_last_recheck_count': [P, P],
    'somgb_kernel_launches': [],
    'somgb_algo_supported': [I32, I64, I64, I32],
    'somgb_device_status': [P, I32, P],
    'somgb_set_kernel_timer': [P, P],
    'somgb_train_bmu_pass': [P, P, I64, I32, P, P, I64, D, I32, P, P, P, SZ, P],
    'somgb_workspace_status': [P, P, I32, P],
    'somgb_debug_tc_withhold': [I64, ctypes.c_uint],
    'somgb_debug_iter_withhold': [ctypes.c_int, ctypes.c_uint],
    'somgb_accumulate': [P, P, P, I64, I32, I64, P, P, P, P],
    'somgb_feature_bounds': [P, P, I64, I32, P, P],
    'somgb_accumulate_f64': [P, P, P, I64, I32, I64, P, P, P],
    'somgb_weighted_moments': [P, P, I64, I32, P, P],
    'somgb_footprint_maps': [P, P, I64, I32, P, I64, I32, P, P, P, P, SZ, P],
    'somgb_footprint_maps_f64': [P, P, I64, I32, P, I64, P, P, P, P],
    'somgb_bmu_histograms': [P, P, I64, I64, P, P, P],
    'somgb_neighbourhood_grid_workspace_bytes': [I64, I64, I32],
    'somgb_sort_rows_workspace_bytes': [I64],
    'somgb_last_sweep2_tiles': [P, P],
    'somgb_sort_rows': [P, P, P, I64, I32, I64, P, P, P, SZ, P],
    'somgb_neighbourhood_update_grid': [P, P, P, I64, I64, I32, D, P, P, P, P, SZ, P],
    'somgb_neighbourhood_update_grid_f64': [P, P, P, I64, I64, I32, D, P, P, P, P, SZ, P],
    'somgb_weighted_moments_f64': [P, P, I64, I32, P, P],
    'somgb_find_bmus': [P, I64, I32, P, I64, I32, P, P, SZ, P],
    'somgb_find_bmus_f64': [P, I64, I32, P, I64, P, P],
    'somgb_find_bmus_noalloc': [P, I64, I32, P, I64, I32, P, P],
    'somgb_find_bmus_noalloc_scratch_bytes': [],
    'somgb_count_bmus': [P, P, I64, I32, P, I64, I32, P, P, SZ, P],
    'somgb_count_bmus_f64': [P, P, I64, I32, P, I64, P, P],
    'somgb_compute_errors': [P, P, I64, I32, P, P, I64, D, I32, P, P, SZ, P],
    'somgb_compute_errors_f64': [P, P, I64, I32, P, P, I64, D, P, P],
    'somgb_train_epoch_pass': [P, P, I64, I32, P, P, I64, D, I32, P, P, P, P, P, SZ, P],
    'somgb_train_epoch_pass_f64': [P, P, I64, I32, P, P, I64, D, P, P, P, P, SZ, P],
    'somgb_neighbourhood_update': [P, P, P, I64, I32, D, P, P, P, P],
    'somgb_neighbourhood_update_f64': [P, P, P, I64, I32, D, P, P, P, P],
    'somgb_train_iter_pass': [P, P, I64, I32, P, P, I64, D, I64, I64, P, P, P, SZ, P],
    'somgb_train_iter_pass_f64': [P, P, I64, I32, P, P, I64, D, I64, I64, P, P, P, SZ, P],
    'somgb_train_iter_pass_grid': [P, P, I64, I32, P, P, I64, I64, D, I64, I64, I32, P, P, P, SZ, P],
    'somgb_divide': [P, P, I64, I32, P, P],
    'somgb_divide_f64': [P, P, I64, I32, P, P],
}
_RESTYPES = {'somgb_last_error': SZ, 'somgb_workspace_bytes': SZ, 'somgb_kernel_launches': I64,
             'somgb_find_bmus_noalloc_scratch_bytes': SZ, 'somgb_neighbourhood_grid_workspace_bytes': SZ,
             'somgb_sort_rows_workspace_bytes': SZ}


class SomgbError(RuntimeError):
    """A libsomgb entry point returned a non-zero status."""

    def __init__(self, status, message):
        super().__init__(f'libsomgb status {status}: {message}')
        self.status = status


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f'{LIB_PATH} is missing: build it with `python -m decontamination_gb300.build` '
                               '(there is no CPU fallback)')
        handle = ctypes.CDLL(LIB_PATH)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, I32)
        _lib = handle
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().somgb_last_error(buf, len(buf))
    return buf.value.decode(errors='replace')


def call(name, *args):
    status = getattr(lib(), name)(*args)
    if status != SOMGB_OK:
        raise SomgbError(status, last_error())
    return status


def workspace_bytes(op, n, m, d, algo):
    return int(lib().somgb_workspace_bytes(op, n, m, d, algo))
