"""ctypes binding of the C ABI in include/fbk.h and include/fbk_synth.h.

The device library is loaded from fastbact_gb300/_lib/libfbk.so and the seeded
input generator from fastbact_gb300/_lib/libfbk_synth.so (both built in-tree by
fastbact_gb300.build).  There is no fallback: if a library is missing, anything
that needs it raises, so no CPU path can stand in for the device kernels.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfbk.so"
SYNTH_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfbk_synth.so"

u8p = C.POINTER(C.c_uint8)
u16p = C.POINTER(C.c_uint16)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
vp = C.c_void_p

FBK_OK = 0
STATUS_NAMES = {
    0: "FBK_OK", 1: "FBK_ERR_INVALID", 2: "FBK_ERR_CUDA", 3: "FBK_ERR_OOM", 4: "FBK_ERR_TABLE_FULL",
    5: "FBK_ERR_TIMEOUT", 6: "FBK_ERR_IO", 7: "FBK_ERR_FORMAT", 8: "FBK_ERR_EMPTY", 9: "FBK_ERR_BUSY",
    10: "FBK_ERR_NOT_READY", 11: "FBK_ERR_NO_DEVICE",
}


class ArenaView(C.Structure):
    _fields_ = [("data", u64p), ("n_words", C.c_uint64), ("offsets", u64p), ("lengths", u32p),
                ("n_seqs", C.c_uint64), ("pair_idx", u32p)]


class CountStats(C.Structure):
    _fields_ = [("exact_read_pairs", C.c_uint64), ("total_bases_r1", C.c_uint64), ("total_bases_r2", C.c_uint64),
                ("total_bases", C.c_uint64), ("min_read_len", C.c_uint64), ("max_read_len", C.c_uint64),
                ("mean_read_len", C.c_double), ("median_read_len", C.c_uint64)]


class GenomeEstimate(C.Structure):
    _fields_ = [("genome_size", C.c_uint64), ("exact_read_pairs", C.c_uint64), ("total_bases", C.c_uint64),
                ("median_read_len", C.c_uint64), ("max_read_len", C.c_uint64), ("estimated_cov", C.c_double),
                ("subsample_factor", C.c_double), ("kmers", C.c_uint64 * 8), ("n_kmers", C.c_uint64),
                ("confidence", C.c_int32), ("_pad", C.c_int32), ("u_ge_1", C.c_uint64), ("u_ge_2", C.c_uint64),
                ("sample_kmer_depth", C.c_double), ("pairs_sampled", C.c_uint64), ("m_sample", C.c_uint64)]


class EstimatorParams(C.Structure):
    _fields_ = [("k", C.c_uint32), ("cms_log2_width", C.c_uint32), ("hll_p", C.c_uint32), ("_pad", C.c_uint32),
                ("sample_cap", C.c_uint64), ("max_pairs", C.c_uint64), ("target_cov", C.c_double)]


class Subsample(C.Structure):
    _fields_ = [("factor", C.c_double), ("seed", C.c_uint64)]


class BuildParams(C.Structure):
    _fields_ = [("k", C.c_uint32), ("key_bits", C.c_uint32), ("cms_log2_width", C.c_uint32),
                ("counter_bits", C.c_uint32), ("t_solid", C.c_uint32), ("min_trans_cov", C.c_uint32),
                ("table_log2_cap", C.c_uint32), ("_pad", C.c_uint32), ("genome_size", C.c_uint64)]


class SubsamplePolicy(C.Structure):
    _fields_ = [("no_subsample", C.c_int32), ("enable_auto_subsample", C.c_int32), ("has_genome_size", C.c_int32),
                ("_pad", C.c_int32), ("genome_size", C.c_uint64), ("depth", C.c_double), ("threshold_ratio", C.c_double)]


class BatchParams(C.Structure):
    _fields_ = [("k", C.c_uint32), ("key_bits", C.c_uint32), ("cms_log2_width", C.c_uint32), ("counter_bits", C.c_uint32),
                ("t_solid", C.c_uint32), ("min_trans_cov", C.c_uint32), ("use_graphs", C.c_uint32), ("autotune", C.c_uint32),
                ("keep_sketch", C.c_uint32), ("max_wave", C.c_uint32), ("est_max_pairs", C.c_uint64),
                ("subsample_seed", C.c_uint64), ("max_wave_bytes", C.c_uint64), ("policy", SubsamplePolicy)]


class BatchResult(C.Structure):
    _fields_ = [("state", C.c_int32), ("subsample_reason", C.c_int32), ("fallback", C.c_int32), ("wave", C.c_int32),
                ("subsample_factor", C.c_double), ("estimate", GenomeEstimate), ("n_keys", C.c_uint64),
                ("n_solid", C.c_uint64), ("digest", C.c_uint64), ("pushes", C.c_uint64), ("kmers", C.c_uint64),
                ("table_capacity", C.c_uint64), ("status", C.c_int32), ("_pad", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("isolates_done", C.c_uint64), ("waves", C.c_uint64), ("fallbacks", C.c_uint64),
                ("graph_launches", C.c_uint64), ("kernel_launches", C.c_uint64), ("ms_estimate", C.c_double),
                ("ms_phase_a", C.c_double), ("ms_phase_b", C.c_double), ("ms_host", C.c_double),
                ("pass1_block", C.c_int32), ("pass1_grid", C.c_int32), ("pass1_rows", C.c_int32),
                ("solid_block", C.c_int32), ("solid_grid", C.c_int32), ("solid_rows", C.c_int32),
                ("emit_block", C.c_int32), ("emit_grid", C.c_int32), ("upsert_block", C.c_int32),
                ("upsert_grid", C.c_int32), ("tuned", C.c_int32), ("emit_form", C.c_int32), ("tune_ms", C.c_double)]


class IngestStatsC(C.Structure):
    _fields_ = [("input_read_pairs", C.c_uint64), ("retained_read_pairs", C.c_uint64), ("bases_before_trim", C.c_uint64),
                ("bases_after_trim", C.c_uint64), ("merged_pairs_count", C.c_uint64), ("merged_bases", C.c_uint64),
                ("unmerged_pairs_count", C.c_uint64)]


class ServerParams(C.Structure):
    _fields_ = [("batch", BatchParams), ("workers", C.c_uint32), ("_pad", C.c_uint32), ("budget_bytes", C.c_uint64)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("t_submit_ms", C.c_double), ("t_admit_ms", C.c_double),
                ("t_done_ms", C.c_double), ("t_uploaded_ms", C.c_double), ("t_estimated_ms", C.c_double),
                ("t_counted_ms", C.c_double), ("reserved_bytes", C.c_uint64), ("result", BatchResult)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("done", C.c_uint64), ("failed", C.c_uint64), ("waves_a", C.c_uint64),
                ("waves_b", C.c_uint64), ("isolates_a", C.c_uint64), ("isolates_b", C.c_uint64),
                ("reserved_bytes", C.c_uint64), ("peak_reserved_bytes", C.c_uint64), ("budget_bytes", C.c_uint64),
                ("peak_in_flight", C.c_uint64), ("busy_ms", C.c_double), ("ms_estimate", C.c_double),
                ("ms_phase_a", C.c_double), ("ms_phase_b", C.c_double)]


class SynthParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("genome_len", C.c_uint64), ("gc", C.c_double), ("n_repeats", C.c_uint32),
                ("repeat_len", C.c_uint32), ("repeat_identity", C.c_double), ("tandem_copies", C.c_uint32),
                ("tandem_unit", C.c_uint32), ("read_len", C.c_uint32), ("_pad", C.c_uint32),
                ("coverage", C.c_double), ("frag_mean", C.c_double), ("frag_sd", C.c_double),
                ("sub_rate", C.c_double), ("indel_rate", C.c_double), ("q_lo", C.c_uint32), ("q_hi", C.c_uint32),
                ("tail_len", C.c_uint32), ("tail_q", C.c_uint32)]


S = C.c_int  # fbk_status
P = C.POINTER

# name -> (restype, argtypes); every symbol the headers declare.
SIGNATURES = {
    "fbk_status_str": (C.c_char_p, [S]),
    "fbk_version": (C.c_char_p, []),
    "fbk_ctx_create": (S, [C.c_int, C.c_uint64, P(vp)]),
    "fbk_ctx_destroy": (S, [vp]),
    "fbk_ctx_fork": (S, [vp, P(vp)]),
    "fbk_ctx_pool_free": (S, [vp, u64p, u64p]),
    "fbk_last_error": (S, [vp, C.c_char_p, C.c_size_t]),
    "fbk_ctx_sync": (S, [vp]),
    "fbk_ctx_set_timing": (S, [vp, C.c_int]),
    "fbk_ctx_timing": (S, [vp, C.c_char_p, P(C.c_double), u64p]),
    "fbk_ctx_timing_reset": (S, [vp]),
    "fbk_ctx_event_record": (S, [vp, C.c_int]),
    "fbk_ctx_event_elapsed": (S, [vp, C.c_int, C.c_int, P(C.c_double)]),
    "fbk_ctx_set_tuning": (S, [vp, C.c_char_p, C.c_double]),
    "fbk_ctx_get_tuning": (S, [vp, C.c_char_p, P(C.c_double)]),
    "fbk_ctx_launch_count": (S, [vp, u64p]),
    "fbk_ctx_mem_info": (S, [vp, u64p, u64p]),
    "fbk_bank_upload": (S, [vp, P(ArenaView), P(vp)]),
    "fbk_bank_upload_async": (S, [vp, P(ArenaView), P(vp)]),
    "fbk_bank_wait": (S, [vp]),
    "fbk_bank_info": (S, [vp, u64p, u64p]),
    "fbk_bank_release": (S, [vp]),
    "fbk_cms_width_for_genome_size": (C.c_uint64, [C.c_uint64]),
    "fbk_cms_create": (S, [vp, C.c_uint32, C.c_uint32, P(vp)]),
    "fbk_cms_clear": (S, [vp]),
    "fbk_cms_add_keys": (S, [vp, u64p, C.c_uint64]),
    "fbk_cms_estimate_keys": (S, [vp, u64p, C.c_uint64, u32p]),
    "fbk_cms_add_bank": (S, [vp, vp, C.c_uint32, C.c_uint32, P(Subsample)]),
    "fbk_cms_build": (S, [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, P(vp)]),
    "fbk_cms_add_contigs": (S, [vp, u8p, u64p, C.c_uint64, C.c_uint32, C.c_uint32]),
    "fbk_cms_nbytes": (S, [vp, u64p]),
    "fbk_cms_export": (S, [vp, u8p, C.c_uint64]),
    "fbk_cms_import": (S, [vp, u8p, C.c_uint64]),
    "fbk_cms_merge": (S, [vp, vp]),
    "fbk_cms_release": (S, [vp]),
    "fbk_hll_create": (S, [vp, C.c_uint32, P(vp)]),
    "fbk_hll_add_hashes": (S, [vp, u64p, C.c_uint64]),
    "fbk_hll_add_canonical_hashes": (S, [vp, u64p, C.c_uint64]),
    "fbk_hll_merge": (S, [vp, vp]),
    "fbk_hll_export": (S, [vp, u8p, C.c_uint64]),
    "fbk_hll_estimate": (S, [vp, P(C.c_double)]),
    "fbk_hll_release": (S, [vp]),
    "fbk_hll_estimate_registers": (C.c_double, [u8p, C.c_uint32]),
    "fbk_nthash_arena": (S, [vp, P(ArenaView), C.c_uint32, u64p, C.c_uint64, u64p]),
    "fbk_canonical_kmers_arena": (S, [vp, P(ArenaView), C.c_uint32, C.c_uint32, u64p, u8p, C.c_uint64, u64p]),
    "fbk_solid_build": (S, [vp, vp, vp, P(BuildParams), P(Subsample), u8p, u64p, C.c_uint64, P(vp)]),
    "fbk_build_front": (S, [vp, vp, P(BuildParams), P(Subsample), u8p, u64p, C.c_uint64, P(vp), P(vp)]),
    "fbk_table_info": (S, [vp, u64p, u64p, u64p]),
    "fbk_table_export": (S, [vp, u64p, u16p, u8p, C.c_uint64, u64p]),
    "fbk_table_export_async": (S, [vp, u64p, u16p, u8p, C.c_uint64, u64p]),
    "fbk_table_export_wait": (S, [vp]),
    "fbk_table_export_acc": (S, [vp, u64p, u16p, u16p, C.c_uint64, u64p]),
    "fbk_table_pushes": (S, [vp, u64p]),
    "fbk_table_flags": (S, [vp, u32p]),
    "fbk_table_digest": (S, [vp, u64p, u64p]),
    "fbk_table_acc_digest": (S, [vp, u64p, u64p]),
    "fbk_table_export_acc_owned": (S, [vp, C.c_uint32, vp, C.c_uint64, u64p]),
    "fbk_table_from_acc_rows": (S, [vp, C.c_uint32, C.c_uint32, C.c_uint32, vp, C.c_uint64, P(vp)]),
    "fbk_cms_counts_device": (S, [vp, P(vp), u64p]),
    "fbk_cms_clamp_counts": (S, [vp]),
    "fbk_table_release": (S, [vp]),
    "fbk_estimator_defaults": (None, [P(EstimatorParams)]),
    "fbk_estimate_sample": (S, [vp, P(ArenaView), C.c_uint64, P(CountStats), P(EstimatorParams), P(GenomeEstimate), u8p, u8p]),
    "fbk_estimate_bank": (S, [vp, vp, u32p, C.c_uint64, P(CountStats), P(EstimatorParams), P(GenomeEstimate), u8p, u8p]),
    "fbk_est_shard_plan": (S, [u32p, C.c_uint64, P(CountStats), P(EstimatorParams), u64p, u32p]),
    "fbk_est_shard_firstpos": (S, [vp, vp, u32p, C.c_uint64, C.c_uint64, C.c_uint64, P(EstimatorParams), u32p]),
    "fbk_est_shard_segments": (S, [vp, vp, u32p, C.c_uint64, C.c_uint64, C.c_uint64, P(EstimatorParams), u32p, u8p]),
    "fbk_est_shard_finish": (S, [u32p, C.c_uint64, P(CountStats), P(EstimatorParams), u8p, P(GenomeEstimate), u8p, u8p]),
    "fbk_estimate_sample_noalloc": (S, [C.c_int, vp, P(ArenaView), C.c_uint64, P(CountStats), P(EstimatorParams),
                                        P(GenomeEstimate), u8p, u8p, C.c_char_p, C.c_size_t]),
    "fbk_count_fastx_exact": (S, [C.c_char_p, C.c_char_p, P(CountStats), C.c_char_p, C.c_size_t]),
    "fbk_estimate_genome": (S, [vp, C.c_char_p, C.c_char_p, C.c_uint64, C.c_double, P(GenomeEstimate)]),
    "fbk_compute_dynamic_kmers": (C.c_int, [C.c_uint64, C.c_int64, u64p, C.c_int]),
    "fbk_subsample_mask": (S, [vp, C.c_uint64, P(Subsample), u64p]),
    "fbk_compact": (S, [vp, P(vp)]),
    "fbk_unitigs_info": (S, [vp, u64p, u64p, u64p]),
    "fbk_unitigs_export": (S, [vp, u8p, u64p, P(C.c_float), u8p]),
    "fbk_unitigs_edges": (S, [vp, u32p, C.c_uint64, u64p]),
    "fbk_unitigs_release": (S, [vp]),
    "fbk_filter_active_reads": (S, [vp, vp, u8p, u64p, u8p, u32p, u32p, C.c_uint64, C.c_uint32, u8p, u64p]),
    "fbk_index_terminal_kmers": (S, [vp, u8p, u64p, C.c_uint64, C.c_uint32, C.c_uint32, u64p, u32p, u8p, u32p, C.c_uint64, u64p]),
    "fbk_ingest_fastq_device": (S, [vp, u8p, C.c_uint64, u8p, C.c_uint64, C.c_double, C.c_uint64, C.c_uint32, C.c_int, C.c_int,
                                    C.c_uint64, P(vp), P(IngestStatsC)]),
    "fbk_bank_export": (S, [vp, u64p, u64p, u32p, u32p]),
    "fbk_bank_arena_counts": (S, [vp, u64p]),
    "fbk_bank_words": (S, [vp, u64p]),
    "fbk_subsample_policy_defaults": (None, [P(SubsamplePolicy)]),
    "fbk_subsample_decide": (S, [P(SubsamplePolicy), P(GenomeEstimate), P(C.c_double), P(C.c_int32)]),
    "fbk_batch_defaults": (None, [P(BatchParams)]),
    "fbk_batch_create": (S, [vp, P(BatchParams), P(vp)]),
    "fbk_batch_submit": (S, [vp, P(ArenaView), P(ArenaView), C.c_uint64, P(CountStats), u64p]),
    "fbk_batch_run": (S, [vp]),
    "fbk_batch_get_result": (S, [vp, C.c_uint64, P(BatchResult)]),
    "fbk_batch_take_table": (S, [vp, C.c_uint64, P(vp)]),
    "fbk_batch_drop": (S, [vp, C.c_uint64]),
    "fbk_batch_get_stats": (S, [vp, P(BatchStats)]),
    "fbk_batch_release": (S, [vp]),
    "fbk_server_defaults": (None, [P(ServerParams)]),
    "fbk_server_create": (S, [vp, P(ServerParams), P(vp)]),
    "fbk_server_submit": (S, [vp, P(ArenaView), P(ArenaView), C.c_uint64, P(CountStats), u64p]),
    "fbk_server_poll": (S, [vp, C.c_uint64, P(RequestInfo)]),
    "fbk_server_wait": (S, [vp, C.c_uint64, C.c_double, P(RequestInfo)]),
    "fbk_server_take_table": (S, [vp, C.c_uint64, P(vp)]),
    "fbk_server_release_request": (S, [vp, C.c_uint64]),
    "fbk_server_get_stats": (S, [vp, P(ServerStats)]),
    "fbk_server_destroy": (S, [vp]),
    "fbk_ingest_fastq": (S, [C.c_char_p, C.c_char_p, C.c_double, C.c_uint64, C.c_uint32, C.c_int, C.c_int, C.c_uint64,
                             P(vp), C.c_char_p, C.c_size_t]),
    "fbk_hbank_arena": (S, [vp, C.c_int, P(ArenaView)]),
    "fbk_hbank_stats": (S, [vp, u64p, u64p, u64p, u64p, u64p, u64p]),
    "fbk_hbank_free": (None, [vp]),
    "fbk_trim_adapter": (C.c_uint64, [u8p, C.c_uint64]),
    "fbk_trim_quality": (C.c_int64, [u8p, u8p, C.c_uint64, C.c_uint32, C.c_uint64]),
    "fbk_merge_read_pair": (C.c_int64, [u8p, u8p, C.c_uint64, u8p, u8p, C.c_uint64, C.c_uint64, C.c_double, u8p, u64p, u64p]),
}

# include/fbk_synth.h, exported by libfbk_synth.so (with the host-bank accessors of
# the banks it returns)
SYNTH_SIGNATURES = {
    "fbk_synth_defaults": (None, [P(SynthParams)]),
    "fbk_synth_n_pairs": (C.c_uint64, [P(SynthParams)]),
    "fbk_synth_genome": (S, [P(SynthParams), u8p]),
    "fbk_synth_pairs": (S, [P(SynthParams), u8p, C.c_uint64, C.c_uint64, u8p, u8p, u8p, u8p]),
    "fbk_synth_write_fastq": (S, [P(SynthParams), C.c_char_p, C.c_char_p]),
    "fbk_synth_isolate": (S, [P(SynthParams), C.c_int, C.c_uint64, C.c_uint32, C.c_int, C.c_int, P(vp), C.c_uint64, P(vp),
                              P(CountStats)]),
    "fbk_hbank_arena": (S, [vp, C.c_int, P(ArenaView)]),
    "fbk_hbank_stats": (S, [vp, u64p, u64p, u64p, u64p, u64p, u64p]),
    "fbk_hbank_free": (None, [vp]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads libfbk.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: run fastbact_gb300.build.build() (the device kernels have no fallback)")
        L = C.CDLL(str(LIB_PATH), mode=C.RTLD_GLOBAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


_synth_lib = None


def synth_lib() -> C.CDLL:
    """Loads libfbk_synth.so, the seeded input generator (raises if it was not built)."""
    global _synth_lib
    if _synth_lib is None:
        if not SYNTH_LIB_PATH.exists():
            raise RuntimeError(f"{SYNTH_LIB_PATH} is missing: run fastbact_gb300.build.build()")
        L = C.CDLL(str(SYNTH_LIB_PATH))
        for name, (res, args) in SYNTH_SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _synth_lib = L
    return _synth_lib


class FbkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status
        self.msg = msg


def check(status: int, ctx=None, what: str = "") -> None:
    if status == FBK_OK:
        return
    msg = what
    if ctx is not None:
        buf = C.create_string_buffer(4096)
        lib().fbk_last_error(ctx, buf, len(buf))
        if buf.value:
            msg = f"{what}: {buf.value.decode(errors='replace')}" if what else buf.value.decode(errors="replace")
    raise FbkError(status, msg)


def ptr(a: np.ndarray | None, ctype=None):
    """Pointer to a contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be contiguous"
    t = ctype or {np.dtype(np.uint8): C.c_uint8, np.dtype(np.uint16): C.c_uint16,
                  np.dtype(np.uint32): C.c_uint32, np.dtype(np.uint64): C.c_uint64}[a.dtype]
    return a.ctypes.data_as(C.POINTER(t))


def arena_view(data: np.ndarray, offsets: np.ndarray, lengths: np.ndarray, pair_idx: np.ndarray | None = None) -> ArenaView:
    v = ArenaView()
    v.data = ptr(data)
    v.n_words = data.size
    v.offsets = ptr(offsets)
    v.lengths = ptr(lengths)
    v.n_seqs = offsets.size
    v.pair_idx = ptr(pair_idx) if pair_idx is not None else None
    return v


def exported_symbols() -> list[str]:
    return sorted(set(SIGNATURES) | set(SYNTH_SIGNATURES))


os.environ.setdefault("CUDA_MODULE_LOADING", "LAZY")
