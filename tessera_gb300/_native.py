"""ctypes bindings of libtessera_gb300.so (include/tessera_gb300.h).

The library is the only implementation of the hot path: there is no CPU fallback. If it is not
built, or a call fails, an exception says why.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libtessera_gb300.so"

TG_OK, TG_DECLINED = 0, 1
TG_ERR_INVALID, TG_ERR_CUDA, TG_ERR_NOMEM, TG_ERR_STATE = -1, -2, -3, -4


class TesseraError(RuntimeError):
    """A failed library call: `code` is the TG_ERR_* status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (status {code})")
        self.code = code


class InvalidInput(TesseraError, ValueError):
    pass


class Config(ctypes.Structure):
    _fields_ = [("level_budget_bytes", ctypes.c_uint64), ("level_min_entries", ctypes.c_uint64),
                ("lde_group_bytes", ctypes.c_uint64), ("tree_flags", ctypes.c_uint64)]


TG_TREE_SUM_Q1 = 1


class TranscriptState(ctypes.Structure):
    _fields_ = [("state", ctypes.c_uint8 * 32), ("counter", ctypes.c_uint64)]


class TableC(ctypes.Structure):
    _fields_ = [("values", ctypes.c_void_p), ("is_ext", ctypes.c_int), ("is_public", ctypes.c_int)]


class InstanceC(ctypes.Structure):
    _fields_ = [("tables", ctypes.POINTER(TableC)), ("ntables", ctypes.c_int), ("vars", ctypes.c_int)]


class CommitJobC(ctypes.Structure):
    _fields_ = [("log_k", ctypes.c_uint32), ("log_inv_rate", ctypes.c_uint32), ("row_block", ctypes.c_uint32),
                ("commitment_id", ctypes.c_uint8 * 32), ("rows", ctypes.c_void_p), ("npolys", ctypes.c_size_t),
                ("codewords", ctypes.c_void_p), ("nodes", ctypes.c_void_p), ("root", ctypes.c_uint8 * 32)]


class EncodeTuningC(ctypes.Structure):
    _fields_ = [("log_k", ctypes.c_uint32), ("log_inv_rate", ctypes.c_uint32), ("npolys", ctypes.c_uint64),
                ("split_log", ctypes.c_int32), ("candidates", ctypes.c_int32), ("group", ctypes.c_uint64),
                ("ms_default", ctypes.c_double), ("ms_tuned", ctypes.c_double), ("from_cache", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class ProofRequestC(ctypes.Structure):
    _fields_ = [("log_k", ctypes.c_uint32), ("log_inv_rate", ctypes.c_uint32), ("row_block", ctypes.c_uint32),
                ("commitment_id", ctypes.c_uint8 * 32), ("rows", ctypes.c_void_p), ("npolys", ctypes.c_size_t),
                ("degree", ctypes.c_int), ("ntables", ctypes.c_int), ("vars", ctypes.c_int),
                ("tables", ctypes.POINTER(ctypes.c_void_p)), ("transcript", TranscriptState), ("prefix", ctypes.c_char_p),
                ("queries", ctypes.c_uint32)]


class ProofResultC(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("root", ctypes.c_uint8 * 32), ("gamma", ctypes.c_uint64 * 2),
                ("rounds", ctypes.c_void_p), ("challenges", ctypes.c_void_p), ("final_evals", ctypes.c_void_p),
                ("transcript", TranscriptState), ("queued_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("query_indices", ctypes.c_void_p), ("columns", ctypes.c_void_p), ("siblings", ctypes.c_void_p),
                ("n_distinct", ctypes.c_uint32), ("n_siblings", ctypes.c_uint32), ("stage_ms", ctypes.c_double * 3)]


class ServerStatsC(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("peak_inflight", ctypes.c_uint64),
                ("peak_bytes", ctypes.c_size_t)]


class LeafGenC(ctypes.Structure):
    _fields_ = [("key_seed", ctypes.c_uint64), ("value_seed", ctypes.c_uint64), ("mult_seed", ctypes.c_uint64),
                ("unit", ctypes.c_int), ("alpha", ctypes.c_uint64 * 2), ("beta", ctypes.c_uint64 * 2)]


class TreeC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("s", ctypes.c_uint32), ("height", ctypes.c_uint32), ("leaves", ctypes.c_void_p),
                ("denominators", ctypes.c_void_p), ("sent", ctypes.c_void_p), ("base_leaves", ctypes.c_uint32),
                ("gen", ctypes.c_void_p)]


class TreeLevelProofC(ctypes.Structure):
    _fields_ = [("level", ctypes.c_int), ("n_root_challenges", ctypes.c_int), ("root_challenges", ctypes.c_void_p),
                ("gamma", ctypes.c_uint64 * 2), ("has_lambda", ctypes.c_int), ("lambda_", ctypes.c_uint64 * 2),
                ("n_max", ctypes.c_int), ("rounds", ctypes.c_void_p), ("challenges", ctypes.c_void_p),
                ("claims", ctypes.c_void_p), ("n_evals", ctypes.c_int), ("evals", ctypes.c_void_p),
                ("rho", ctypes.c_uint64 * 2), ("n_present", ctypes.c_int), ("present", ctypes.c_void_p)]


class SumcheckJobC(ctypes.Structure):
    _fields_ = [("transcript", ctypes.c_void_p), ("prefix", ctypes.c_char_p), ("degree", ctypes.c_int),
                ("instances", ctypes.POINTER(InstanceC)), ("ninstances", ctypes.c_int),
                ("gamma", ctypes.c_uint64 * 2), ("rounds", ctypes.c_void_p), ("challenges", ctypes.c_void_p),
                ("final_evals", ctypes.c_void_p), ("n_evals", ctypes.c_size_t)]


_lib = None

V, U32, U64, SZ, INT = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_int
CSTR = ctypes.c_char_p

# name -> argument types (every function returns int unless listed in _RESTYPE)
SIGNATURES = {
    "tg_version": [],
    "tg_last_error": [],
    "tg_device_open": [INT, V, V],
    "tg_device_close": [V],
    "tg_device_sync": [V],
    "tg_device_launches": [V, V],
    "tg_measure_int_peaks": [V, V],
    "tg_check_lazy_arith": [V, V, SZ, V],
    "tg_check_grid_meet": [V, INT, INT, INT, U32, V, V],
    "tg_fill_splitmix": [V, V, SZ, U64, V],
    "tg_fill_counter": [V, V, SZ, U64, V],
    "tg_device_trim": [V],
    "tg_device_stream": [V, V],
    "tg_profile_enable": [V, INT],
    "tg_profile_read": [V, V, SZ, V, V, V, SZ, V],
    "tg_encode_rows_dev": [V, U32, U32, U32, V, SZ, V, V, V],
    "tg_encode_rows": [V, U32, U32, U32, V, SZ, V, V],
    "tg_encode_rows_noalloc_dev": [V, U32, U32, U32, V, SZ, V, V, V],
    "tg_advice_masks_dev": [V, V, SZ, U64, SZ, V, V],
    "tg_advice_masks": [V, V, SZ, U64, SZ, V],
    "tg_ntt_dev": [V, U32, V, SZ, V],
    "tg_intt_dev": [V, U32, V, SZ, V],
    "tg_coset_ntt_dev": [V, U32, U64, V, SZ, V],
    "tg_coset_intt_dev": [V, U32, U64, V, SZ, V],
    "tg_ntt": [V, U32, V, SZ],
    "tg_intt": [V, U32, V, SZ],
    "tg_coset_ntt": [V, U32, U64, V, SZ],
    "tg_coset_intt": [V, U32, U64, V, SZ],
    "tg_column_init_dev": [V, V, U64, V, V],
    "tg_column_absorb_dev": [V, V, U64, V, SZ, U32, V],
    "tg_merkle_tree_dev": [V, V, SZ, V, V],
    "tg_column_merge_dev": [V, V, SZ, U64, V, V],
    "tg_commit_unmasked_dev": [V, U32, U32, U32, V, V, SZ, V, V, V, V],
    "tg_commit_unmasked": [V, U32, U32, U32, V, V, SZ, V, V],
    "tg_merge_segments": [V, V, SZ, U64, V, V],
    "tg_advice_sink_open": [V, U32, U32, U32, U32, V, V],
    "tg_sink_absorb": [V, V, SZ, V],
    "tg_sink_finish": [V, V],
    "tg_sink_close": [V],
    "tg_matrix_open": [V, U32, U32, U32, V, V, SZ, V],
    "tg_matrix_absorb": [V, V, SZ, V],
    "tg_matrix_finish": [V, V],
    "tg_matrix_close": [V],
    "tg_hash": [CSTR, V, SZ, V],
    "tg_transcript_init": [V, V, SZ],
    "tg_transcript_absorb": [V, CSTR, V, SZ],
    "tg_transcript_absorb_fp2s": [V, CSTR, V, SZ],
    "tg_transcript_squeeze": [V, CSTR, V],
    "tg_transcript_challenge_fp": [V, CSTR, V],
    "tg_transcript_challenge_fp2": [V, CSTR, V],
    "tg_transcript_challenge_indices": [V, CSTR, U32, U32, V],
    "tg_transcript_check_grind": [V, CSTR, U32, U64, V],
    "tg_transcript_grind": [V, V, CSTR, U32, V],
    "tg_prove_batch": [V, V, CSTR, INT, V, INT, INT, V, V, V, V, V],
    "tg_prove_many": [V, V, INT, INT],
    "tg_commit_many": [V, V, INT, INT],
    "tg_commit_plan_create": [V, V, INT, INT, V],
    "tg_commit_plan_launch": [V, V],
    "tg_commit_plan_info": [V, V, V, V],
    "tg_commit_plan_tuning": [V, V, INT, V],
    "tg_host_prefault": [V, SZ],
    "tg_commit_plan_destroy": [V],
    "tg_column_sink_open": [V, U32, U32, U32, U32, V, SZ, V],
    "tg_column_sink_select": [V, V, SZ, V, V],
    "tg_column_sink_select_combining": [V, V, SZ, V, V, SZ, V],
    "tg_column_sink_combined": [V, V, SZ],
    "tg_column_sink_close": [V],
    "tg_leaf_stage_open": [V, V, INT, INT, V],
    "tg_leaf_stage_height": [V, V, V],
    "tg_leaf_stage_root": [V, INT, V],
    "tg_leaf_stage_prove_level": [V, V, V],
    "tg_leaf_stage_claim": [V, INT, V, V, V, V],
    "tg_leaf_stage_close": [V],
    "tg_logup_leaves": [V, U64, U64, INT, U64, V, V, SZ, V, V],
    "tg_server_open": [V, SZ, INT, V],
    "tg_server_submit": [V, V, V, V],
    "tg_server_wait": [V, U64, INT],
    "tg_server_stats_read": [V, V],
    "tg_server_close": [V],
    "tg_level_load": [V, INT, V, V, INT, SZ, V],
    "tg_level_sums": [V, V, V, SZ, U32, V],
    "tg_level_bind": [V, V],
    "tg_level_firsts": [V, V],
    "tg_level_free": [V],
}
_RESTYPE = {"tg_last_error": ctypes.c_char_p}


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"libtessera_gb300 is not built ({LIB_PATH} missing): run "
                "`python -c 'import tessera_gb300.build as b; b.build()'` with the CUDA toolkit")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = L
    return _lib


def check(rc: int) -> int:
    """Raises for a negative status; returns TG_OK or TG_DECLINED."""
    if rc < 0:
        msg = lib().tg_last_error().decode(errors="replace")
        cls = InvalidInput if rc == TG_ERR_INVALID else TesseraError
        raise cls(rc, msg)
    return rc


def call(name: str, *args) -> int:
    return check(getattr(lib(), name)(*args))
