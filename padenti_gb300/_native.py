"""ctypes binding of libpadenti_gb300.so (the C ABI in include/padenti_gb300.h).

The library is built in-tree by padenti_gb300.build.  Nothing here falls back to
another implementation: if the library is missing or fails to load, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

# PADENTI_GB300_LIB selects another build of the library (same C ABI).
LIB_PATH = pathlib.Path(os.environ.get("PADENTI_GB300_LIB") or
                        pathlib.Path(__file__).resolve().parent / "_build" / "libpadenti_gb300.so")

PD_OK = 0
PD_IMG_U8, PD_IMG_U16, PD_IMG_I16, PD_IMG_I32, PD_IMG_F32 = 1, 2, 3, 4, 5
PD_FEAT_I16, PD_FEAT_I32 = 1, 2
PD_PLUGIN_DEPTH_DIFF2, PD_PLUGIN_DEPTH_DIFF1, PD_PLUGIN_CHANNEL_DIFF = 1, 2, 3
PD_PLUGIN_USER = 100
PD_MAX_FEAT_DIM = 8

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "unsupported", -5: "bad state"}


class Config(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("plugin", "img_type", "n_channels", "feat_type", "feat_dim", "n_classes")]


class TrainParams(C.Structure):
    _fields_ = [
        ("n_features", C.c_uint32),
        ("n_thresholds", C.c_uint32),
        ("feat_low", C.c_int32 * PD_MAX_FEAT_DIM),
        ("feat_up", C.c_int32 * PD_MAX_FEAT_DIM),
        ("thr_low", C.c_int32),
        ("thr_up", C.c_int32),
        ("per_leaf_samples_thr", C.c_uint32),
    ]


class DatasetDesc(C.Structure):
    _fields_ = [
        ("n_images", C.c_uint32),
        ("pixels", C.c_void_p),
        ("pix_off", C.c_void_p),
        ("width", C.c_void_p),
        ("height", C.c_void_p),
        ("labels", C.c_void_p),
        ("lab_off", C.c_void_p),
        ("samples", C.c_void_p),
        ("samp_off", C.c_void_p),
    ]


class TrainStats(C.Structure):
    _fields_ = [
        ("evals", C.c_uint64),
        ("nodes_trained", C.c_uint64),
        ("nodes_split", C.c_uint64),
        ("hist_launches", C.c_uint64),
        ("split_rechecked", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("hist_bytes", C.c_uint64),
        ("h2d_bytes", C.c_uint64),
        ("d2h_bytes", C.c_uint64),
        ("ms_candidates", C.c_double),
        ("ms_hist", C.c_double),
        ("ms_split", C.c_double),
        ("ms_reassign", C.c_double),
        ("ms_total", C.c_double),
    ]


class Sampler(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("n_samples", C.c_uint32),
        ("seed", C.c_uint32),
        ("n_classes", C.c_uint32),
        ("weights", C.c_void_p),
        ("pixel_bytes", C.c_uint32),
    ]


# int exchange(void *user, uint32 n_nodes, uint32 n_classes, int64 *gain_key, int64 *cand_index, uint32 *left_counts)
EXCHANGE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                          C.POINTER(C.c_uint32))


class Tuning(C.Structure):
    _fields_ = [("chunk", C.c_int32), ("hist_spi", C.c_int32), ("fuse_max", C.c_int32), ("cand_order", C.c_int32),
                ("persist", C.c_int32), ("ms_start", C.c_double), ("ms_best", C.c_double), ("trials", C.c_int32),
                ("from_cache", C.c_int32)]


class Record(C.Structure):
    """pd_record: one split node of a trained tree (learned proposals)."""
    _fields_ = [("depth", C.c_uint32), ("count", C.c_uint32), ("node", C.c_uint32), ("tree", C.c_uint32),
                ("gain", C.c_double), ("feat", C.c_int32 * 8), ("thr", C.c_int32), ("class_count", C.c_uint32 * 64)]


class SampleStats(C.Structure):
    _fields_ = [
        ("images", C.c_uint64),
        ("data_bytes", C.c_uint64),
        ("label_bytes", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("h2d_bytes", C.c_uint64),
        ("d2h_bytes", C.c_uint64),
        ("ms_scan", C.c_double),
        ("ms_draw", C.c_double),
        ("ms_total", C.c_double),
    ]


PD_SAMPLER_UNIFORM = 1
PD_SAMPLER_CLASS_WEIGHTED = 2

# name -> (restype, argtypes)
_P = C.c_void_p
class UploadStats(C.Structure):
    _fields_ = [("ms_samples", C.c_double), ("ms_device", C.c_double), ("ms_total", C.c_double)]


_SIGS = {
    "pd_last_error": (C.c_char_p, []),
    "pd_version": (C.c_int, []),
    "pd_ctx_create": (C.c_int, [C.POINTER(Config), C.c_int, C.POINTER(_P)]),
    "pd_ctx_destroy": (C.c_int, [_P]),
    "pd_plugin_compile": (C.c_int, [_P, C.c_char_p]),
    "pd_plugin_check": (C.c_int, [C.POINTER(Config), C.c_char_p, C.c_char_p, C.c_size_t]),
    "pd_ctx_set_hist_budget": (C.c_int, [_P, C.c_uint64]),
    "pd_ctx_set_tuning": (C.c_int, [_P, C.c_char_p, C.c_int64]),
    "pd_ctx_sync": (C.c_int, [_P]),
    "pd_ctx_stream": (_P, [_P]),
    "pd_ctx_transfer_bytes": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "pd_dataset_upload": (C.c_int, [_P, C.POINTER(DatasetDesc)]),
    "pd_dataset_info": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]),
    "pd_dataset_upload_stats": (C.c_int, [_P, C.POINTER(UploadStats)]),
    "pd_train_tree": (C.c_int, [_P, C.POINTER(TrainParams), C.c_uint32, C.c_uint32, C.c_uint32, _P, _P, _P, _P, _P]),
    "pd_train_get_stats": (C.c_int, [_P, C.POINTER(TrainStats)]),
    "pd_train_sample_nodes": (C.c_int, [_P, _P]),
    "pd_candidates": (C.c_int, [_P, C.POINTER(TrainParams), C.c_uint32, _P, C.c_uint32, _P, _P]),
    "pd_hist": (C.c_int, [_P, C.POINTER(TrainParams), C.c_uint32, _P, _P, C.c_uint32, _P]),
    "pd_split": (C.c_int, [_P, C.POINTER(TrainParams), _P, _P, C.c_uint32, _P, _P, _P]),
    "pd_log2_table": (C.c_int, [_P, C.c_uint32, _P]),
    "pd_train_records": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "pd_autotune": (C.c_int, [_P, C.POINTER(TrainParams), C.c_uint32, C.c_uint32, C.c_char_p, C.POINTER(Tuning)]),
    "pd_train_tree_sharded": (C.c_int, [_P, C.POINTER(TrainParams), C.c_uint32, C.c_uint32, _P, _P, C.c_uint32,
                                        C.c_uint32, C.c_uint32, _P, _P, _P, _P, _P]),
    "pd_proposer_create": (C.c_int, [_P, C.POINTER(TrainParams), C.c_uint64, C.POINTER(_P)]),
    "pd_proposer_destroy": (C.c_int, [_P]),
    "pd_proposer_dims": (C.c_int, [_P, _P, C.POINTER(C.c_uint64)]),
    "pd_proposer_get_params": (C.c_int, [_P, _P]),
    "pd_proposer_set_params": (C.c_int, [_P, _P]),
    "pd_proposer_forward": (C.c_int, [_P, _P, C.c_uint32, _P]),
    "pd_proposer_loss_grad": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.POINTER(C.c_float), _P]),
    "pd_proposer_fit": (C.c_int, [_P, _P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_float, _P,
                                  C.POINTER(C.c_float)]),
    "pd_train_tree_proposed": (C.c_int, [_P, _P, C.POINTER(TrainParams), C.c_uint32, C.c_uint32, C.c_uint32,
                                         C.c_uint32, _P, _P, _P, _P, _P]),
    "pd_split_noalloc": (C.c_int, [C.POINTER(TrainParams), C.c_uint32, _P, _P, C.c_uint32, _P, _P, _P, _P]),
    "pd_forest_clear": (C.c_int, [_P]),
    "pd_forest_add_tree": (C.c_int, [_P, C.c_uint32, _P, _P, _P, _P]),
    "pd_forest_size": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "pd_predict_posterior": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32, _P, _P]),
    "pd_predict_leaf": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, C.c_uint32, _P, _P]),
    "pd_predict_posterior_batch": (C.c_int, [_P, C.c_uint32, _P, _P, _P, _P, _P]),
    "pd_predict_posterior_device": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, C.c_uint32, _P, _P]),
    "pd_sampler_stride": (C.c_int, [C.POINTER(Sampler), C.POINTER(C.c_uint32)]),
    "pd_sample": (C.c_int, [_P, C.POINTER(Sampler), C.c_uint32, _P, _P, _P, _P, C.c_uint32, _P, _P]),
    "pd_sample_device": (C.c_int, [_P, C.POINTER(Sampler), C.c_uint32, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32,
                                   _P, _P]),
    "pd_sample_get_stats": (C.c_int, [_P, C.POINTER(SampleStats)]),
    "pd_rgb_to_labels": (C.c_int, [_P, C.c_uint32, _P, _P, _P, C.c_uint32, _P, C.c_uint32, _P]),
    "pd_rgb_to_labels_device": (C.c_int, [_P, C.c_uint64, _P, C.c_uint32, _P, C.c_uint32, _P,
                                          C.POINTER(C.c_float)]),
    "pd_image_roi": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_int32, C.c_uint32, _P]),
    "pd_measure_smem_atomics": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "pd_synth_depth": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                 C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _P, _P, _P]),
    "pd_synth_rgb": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                               C.c_uint32, _P, _P, _P]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def lib() -> C.CDLL:
    """The loaded native library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m padenti_gb300.build`")
        l = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


class PadentiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != PD_OK:
        msg = lib().pd_last_error()
        raise PadentiError(rc, msg.decode() if msg else "")
