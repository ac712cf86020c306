"""Loader for the GB300 learner library (``lib/libbkgpu.so``).

The library is the product: CUDA kernels for sm_103a plus the C-ABI declared in
``include/bkgpu.h``. There is no CPU fallback; if the library is missing, ``load()`` raises.
"""
import ctypes
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libbkgpu.so")

_lib = None


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(
                "libbkgpu.so is not built (%s); run build_ext.build() first — there is no CPU fallback" % LIB_PATH)
        import importlib.util
        spec = importlib.util.spec_from_file_location("bk_build_ext", os.path.join(PKG_DIR, "build_ext.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = ctypes.CDLL(LIB_PATH)
    _declare(lib)
    _lib = lib
    return lib


def _declare(lib):
    c = ctypes
    P = c.c_void_p
    i32, i64, u32, f64 = c.c_int32, c.c_int64, c.c_uint32, c.c_double
    lib.bk_find_bin_numerical.restype = i32
    lib.bk_find_bin_numerical.argtypes = [P, i64, i64, i32, i32, i32, i32, i32, i32, P, i32, P, P]
    lib.bk_values_to_group_bins.restype = None
    lib.bk_values_to_group_bins.argtypes = [P, i64, i64, P, i32, i32, i32, P]
    lib.bk_find_bin_categorical.restype = i32
    lib.bk_find_bin_categorical.argtypes = [P, i64, i64, i32, i32, i32, i32, i32, i32, P, i32, P, P]
    lib.bk_values_to_group_bins_categorical.restype = None
    lib.bk_values_to_group_bins_categorical.argtypes = [P, i64, i64, P, i32, i32, P]
    if hasattr(lib, "bk_last_error"):
        lib.bk_last_error.restype = c.c_char_p
        lib.bk_last_error.argtypes = []
    for name, res, args in _GPU_SIGNATURES:
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args


c = ctypes
_P, _i32, _i64, _u32, _f64 = c.c_void_p, c.c_int32, c.c_int64, c.c_uint32, c.c_double
# (name, restype, argtypes) of the learner entry points declared in include/bkgpu.h
_GPU_SIGNATURES = [
    ("bk_learner_create", _i32, [_P, _i32, _P, _i64, _P, _i32, _P]),
    ("bk_learner_create_device_bins", _i32, [_P, _i32, _P, _i64, _P, _i32, _P]),
    ("bk_bin_dense_device", _i32, [_P, _i32, _i64, _i32, _P, _i32, _P, _P, _P, _P]),
    ("bk_learner_train", _i32, [_P, _P, _P, _i32, _P, _i64, _P, _P, _P, _P]),
    ("bk_learners_train_batch", _i32, [_P, _i32, _P, _P, _i32, _f64, _P, _P, _P, _P, _P]),
    ("bk_learner_group_create", _i32, [_P, _i32, _P]),
    ("bk_learner_group_train", _i32, [_P, _P, _P, _f64, _P, _P, _P, _P, _P]),
    ("bk_learner_group_destroy", _i32, [_P]),
    ("bk_learner_group_autotune", _i32, [_P, _P, _P, _i32, _P]),
    ("bk_learner_add_prediction_to_score", _i32, [_P, _P, _P, _i32]),
    ("bk_learner_row_leaf", _i32, [_P, _P]),
    ("bk_learner_set_loop_mode", _i32, [_P, _i32]),
    ("bk_learner_set_launch_overlap", _i32, [_P, _i32]),
    ("bk_learner_reset_constant_hessian", _i32, [_P, _i32]),
    ("bk_learner_histogram_cache_capacity", _i32, [_P, _P]),
    ("bk_learner_search_threads", _i32, [_P, _P]),
    ("bk_learner_reset_histogram_pool_config", _i32, [_P]),
    ("bk_learner_set_feature_mask", _i32, [_P, _P]),
    ("bk_learner_set_bynode", _i32, [_P, _f64, _i32, _u32]),
    ("bk_learner_bynode_state", _i32, [_P, _P]),
    ("bk_learner_set_interaction_constraints", _i32, [_P, _P, _P, _i32]),
    ("bk_learner_autotune", _i32, [_P, _P, _P, _i32, _i32, _P]),
    ("bk_learner_launch_shape", _i32, [_P, _P]),
    ("bk_learner_set_launch_shape", _i32, [_P, _P]),
    ("bk_learner_last_timing", _i32, [_P, _P, _P, _P]),
    ("bk_learner_set_timing", _i32, [_P, _i32]),
    ("bk_learner_last_phase_timing", _i32, [_P, _P, _P]),
    ("bk_learner_last_step_timing", _i32, [_P, _P]),
    ("bk_learner_gradient_buffers", _i32, [_P, _P, _P]),
    ("bk_learner_objective_gradients", _i32, [_P, _i32, _P, _P, _f64]),
    ("bk_learner_objective_loss", _i32, [_P, _i32, _P, _P, _P]),
    ("bk_learner_set_objective_weights", _i32, [_P, _P, _f64, _f64]),
    ("bk_learner_predict_add", _i32, [_P, _i32, _P, _P, _P, _P, _P, _P, _P, _P, _i64, _P]),
    ("bk_learner_leaf_histogram", _i32, [_P, _i32, _i32, _P, _P]),
    ("bk_learner_stream", _i32, [_P, _P]),
    ("bk_learner_destroy", _i32, [_P]),
    ("bk_partition_split_noalloc", _i32, [_P, _i64, _P, _i64, _P, _P, _P, _P]),
]

# every symbol include/bkgpu.h declares
EXPORTED = [name for name, _, _ in _GPU_SIGNATURES] + ["bk_last_error", "bk_find_bin_numerical",
                                                        "bk_values_to_group_bins", "bk_find_bin_categorical",
                                                        "bk_values_to_group_bins_categorical"]


def last_error() -> str:
    lib = load()
    msg = lib.bk_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise RuntimeError("%s failed: %s" % (what or "bkgpu call", last_error()))
