"""ctypes view of include/falx_gpu.h. Loading fails loudly if the engine
library is missing: there is no CPU fallback."""

import ctypes
import os
from ctypes import (POINTER, Structure, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_uint32, c_uint64,
                    c_void_p)

from . import build

FALX_OK = 0
FALX_ERR_INVALID = -1
FALX_ERR_CAPACITY = -2
FALX_ERR_INPUT_TOO_LARGE = -3
FALX_ERR_SCHEMA = -4
FALX_ERR_TIMEOUT = -5
FALX_ERR_CUDA = -6
FALX_ERR_OVERFLOW = -7
FALX_ERR_FORMAT = -8

CSV, CSV_HASH, TSV, LOGFMT, NDJSON = 0, 1, 2, 3, 4
I64, U32, F64, STR, BYTES = 0, 1, 2, 3, 4
MAX_COLUMNS = 32


class falx_column(Structure):
    _fields_ = [("field", c_uint32), ("type", c_uint32)]


class falx_schema(Structure):
    _fields_ = [("dialect", c_int32), ("ncols", c_uint32), ("cols", falx_column * MAX_COLUMNS)]


class falx_column_out(Structure):
    _fields_ = [("values", c_void_p), ("valid", c_void_p), ("str_data", c_void_p), ("str_cap", c_uint64),
                ("str_len", c_uint64)]


class falx_columns(Structure):
    _fields_ = [("rows_cap", c_uint64), ("rows", c_uint64), ("cols", falx_column_out * MAX_COLUMNS)]


class falx_geo_stats(Structure):
    _fields_ = [("records", c_uint64), ("values", c_uint64 * 2), ("checksum", c_uint64 * 2),
                ("sum_e6", c_int64 * 2), ("inexact", c_uint64 * 2), ("sum_f64", c_double * 2)]


class falx_geo_text_stats(Structure):
    _fields_ = [("records", c_uint64), ("city_values", c_uint64), ("city_bytes", c_uint64),
                ("city_checksum", c_uint64), ("latitude_values", c_uint64), ("longitude_values", c_uint64),
                ("latitude_checksum", c_uint64), ("longitude_checksum", c_uint64)]


class falx_gz_block(Structure):
    _fields_ = [("in_off", c_uint64), ("out_off", c_uint64), ("in_len", c_uint32), ("out_len", c_uint32)]


class falx_field_byte_stats(Structure):
    _fields_ = [("fields", c_uint64), ("bytes", c_uint64)]


class falx_outputs(Structure):
    _fields_ = [("index", c_void_p), ("index_cap", c_uint64), ("n_index", c_uint64),
                ("seps", c_void_p), ("seps_cap", c_uint64), ("n_seps", c_uint64),
                ("ends", c_void_p), ("ends_cap", c_uint64), ("n_ends", c_uint64),
                ("columns", POINTER(falx_columns)), ("field_bytes", POINTER(falx_field_byte_stats)),
                ("stats", POINTER(falx_geo_stats)), ("stats_fields", c_uint32 * 2)]


class falx_ndjson_stats(Structure):
    _fields_ = [("records", c_uint64), ("sum_id", c_int64), ("sum_score_e6", c_int64),
                ("total_e6_lo", c_int64), ("total_e6_hi", c_int64), ("total_f64", c_double)]


class falx_spec_stats(Structure):
    _fields_ = [("tiles", c_uint64), ("mispredicted", c_uint64)]


class falx_shard_summary(Structure):
    _fields_ = [("states", c_uint32), ("exit", c_uint32 * 4), ("structurals", c_uint64 * 4),
                ("terminators", c_uint64 * 4), ("rows", c_uint64 * 4), ("last_byte", c_int32)]


class falx_doc(Structure):
    _fields_ = [("data", c_void_p), ("len", c_uint64), ("dialect", c_int32), ("field0", c_uint32),
                ("field1", c_uint32), ("index", c_void_p), ("index_cap", c_uint64), ("col0", c_void_p),
                ("col1", c_void_p), ("valid0", c_void_p), ("valid1", c_void_p), ("rows_cap", c_uint64),
                ("n_index", c_uint64), ("rows", c_uint64), ("status", c_int32)]


class falx_batch_config(Structure):
    _fields_ = [("chunk_bytes", c_uint32), ("ctas_per_sm", c_uint32), ("staging", c_uint32)]


# Every symbol the header declares, with its signature.
SIGNATURES = {
    "falx_create": (c_int, [c_int, POINTER(c_void_p)]),
    "falx_destroy": (None, [c_void_p]),
    "falx_set_stream": (c_int, [c_void_p, c_void_p]),
    "falx_set_option": (c_int, [c_void_p, c_int, c_int]),
    "falx_last_timings": (c_int, [c_void_p, POINTER(c_float), c_int]),
    "falx_test_stalled_lookback": (c_int, [c_void_p, POINTER(falx_schema), c_void_p, c_uint64, POINTER(falx_columns),
                                           c_uint64]),
    "falx_strerror": (c_char_p, [c_int]),
    "falx_index_structurals": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_void_p, c_uint64, POINTER(c_uint64)]),
    "falx_parse_tape": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_void_p, c_uint64, c_void_p, c_uint64,
                                POINTER(c_uint64), POINTER(c_uint64)]),
    "falx_parse_columns": (c_int, [c_void_p, POINTER(falx_schema), c_void_p, c_uint64, POINTER(falx_columns)]),
    "falx_stats_count_sum": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_uint32, c_uint32,
                                     POINTER(falx_geo_stats)]),
    "falx_field_bytes": (c_int, [c_void_p, c_int, c_void_p, c_uint64, POINTER(falx_field_byte_stats)]),
    "falx_csv_geo_text_stats": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_uint32, c_uint32, c_uint32,
                                        POINTER(falx_geo_text_stats)]),
    "falx_parse": (c_int, [c_void_p, POINTER(falx_schema), c_void_p, c_uint64, POINTER(falx_outputs)]),
    "falx_ndjson_id_score": (c_int, [c_void_p, c_void_p, c_uint64, POINTER(falx_ndjson_stats)]),
    "falx_index_structurals_host": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_void_p, c_uint64,
                                            POINTER(c_uint64)]),
    "falx_parse_host": (c_int, [c_void_p, POINTER(falx_schema), c_void_p, c_uint64, POINTER(falx_outputs)]),
    "falx_index_structurals_noalloc": (c_int, [c_int, c_int, c_void_p, c_uint64, c_void_p, c_uint64,
                                               POINTER(c_uint64), c_void_p]),
    "falx_bgzf_scan": (c_int, [c_void_p, c_uint64, c_void_p, c_uint64, POINTER(c_uint64), POINTER(c_uint64)]),
    "falx_bgzf_inflate": (c_int, [c_void_p, c_void_p, c_uint64, c_void_p, c_uint64, c_void_p, c_uint64, c_void_p,
                                  POINTER(c_uint64)]),
    "falx_parse_gz_host": (c_int, [c_void_p, POINTER(falx_schema), c_void_p, c_uint64, c_void_p, c_uint64,
                                   POINTER(falx_outputs)]),
    "falx_model_param_count": (c_uint64, []),
    "falx_model_create": (c_int, [c_void_p, c_uint64, POINTER(c_void_p)]),
    "falx_model_destroy": (None, [c_void_p]),
    "falx_model_set_confidence": (c_int, [c_void_p, c_float]),
    "falx_model_get": (c_int, [c_void_p, c_void_p, c_void_p, c_uint64]),
    "falx_model_set": (c_int, [c_void_p, c_void_p, c_void_p, c_uint64]),
    "falx_byte_classes": (c_int, [c_void_p, c_void_p, c_uint64, c_void_p, c_uint32, c_void_p]),
    "falx_model_forward": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p]),
    "falx_model_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, POINTER(c_float)]),
    "falx_model_train": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint64, c_uint32, c_uint32, c_float,
                                 POINTER(c_float)]),
    "falx_region_states": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_void_p, c_uint64, POINTER(c_uint64)]),
    "falx_predict_tiles": (c_int, [c_void_p, c_void_p, c_void_p, c_uint64, c_void_p, c_uint64, POINTER(c_uint64)]),
    "falx_index_structurals_assumed": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_void_p, c_void_p, c_uint64,
                                               POINTER(c_uint64), POINTER(falx_spec_stats)]),
    "falx_index_structurals_speculative": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_uint64, c_void_p,
                                                   c_uint64, POINTER(c_uint64), POINTER(falx_spec_stats)]),
    "falx_summarize_shard": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_int, POINTER(falx_shard_summary)]),
    "falx_parse_tape_seeded": (c_int, [c_void_p, c_int, c_void_p, c_uint64, c_int, c_uint32, c_uint64, c_uint64,
                                       c_void_p, c_uint64, c_void_p, c_uint64, c_void_p, c_uint64,
                                       POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64)]),
    "falx_batch_create": (c_int, [c_void_p, POINTER(falx_doc), c_uint32, POINTER(falx_batch_config),
                                  POINTER(c_void_p)]),
    "falx_batch_run": (c_int, [c_void_p, POINTER(falx_doc)]),
    "falx_batch_info": (c_int, [c_void_p, POINTER(falx_batch_config), POINTER(c_uint32), POINTER(c_uint32),
                                POINTER(c_int)]),
    "falx_batch_destroy": (None, [c_void_p]),
    "falx_batch_tune": (c_int, [c_void_p, POINTER(falx_doc), c_uint32, POINTER(falx_batch_config),
                                POINTER(c_float)]),
    "falx_batch_plan": (c_int, [c_void_p, c_uint32, c_uint32, c_void_p, c_uint32, POINTER(c_uint32)]),
}

OPT_ROWS_PATH = 1
OPT_CTAS_PER_SM = 2
OPT_TIMING = 3
OPT_PIPELINE = 4
MLP_BYTES = 256
SPEC_TILE = 16384

NOALLOC_MAX_BYTES = 256 << 20

_lib = None


def lib_path():
    return build.GPU_LIB


def load(build_if_missing=True):
    """Load the engine library (building it in-tree if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("falx_gb300: CUDA engine library %s is missing (run falx_gb300.build)" % path)
        build.build_gpu()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class FalxError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        msg = load().falx_strerror(code).decode()
        super().__init__("%s failed: %s (%d)" % (what, msg, code))


def check(code, what):
    if code != FALX_OK:
        raise FalxError(code, what)
    return code
