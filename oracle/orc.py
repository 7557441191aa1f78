"""ctypes wrapper of the oracle library (oracle/_build/liborc.so).

TEST INFRASTRUCTURE ONLY: the oracle the device kernels are checked against, and the
timed CPU baseline.  Builds the library on first use with oracle/build_oracle.sh.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liborc.so"

u8p = C.POINTER(C.c_uint8)
u16p = C.POINTER(C.c_uint16)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
vp = C.c_void_p


class OrcArena(C.Structure):
    _fields_ = [("data", u64p), ("n_words", C.c_uint64), ("offsets", u64p), ("lengths", u32p), ("n_seqs", C.c_uint64)]


class OrcCountStats(C.Structure):
    _fields_ = [("exact_read_pairs", C.c_uint64), ("total_bases_r1", C.c_uint64), ("total_bases_r2", C.c_uint64),
                ("total_bases", C.c_uint64), ("min_read_len", C.c_uint64), ("max_read_len", C.c_uint64),
                ("mean_read_len", C.c_double), ("median_read_len", C.c_uint64)]


class OrcEstimate(C.Structure):
    _fields_ = [("genome_size", C.c_uint64), ("exact_read_pairs", C.c_uint64), ("total_bases", C.c_uint64),
                ("median_read_len", C.c_uint64), ("max_read_len", C.c_uint64), ("estimated_cov", C.c_double),
                ("subsample_factor", C.c_double), ("kmers", C.c_uint64 * 8), ("n_kmers", C.c_uint64),
                ("confidence", C.c_int32), ("_pad", C.c_int32), ("u_ge_1", C.c_uint64), ("u_ge_2", C.c_uint64),
                ("sample_kmer_depth", C.c_double), ("pairs_sampled", C.c_uint64), ("m_sample", C.c_uint64)]


_SIG = {
    "orc_splitmix64": (C.c_uint64, [C.c_uint64]),
    "orc_rev_comp_word": (C.c_uint64, [C.c_uint64, C.c_uint]),
    "orc_cms_width_for_genome_size": (C.c_uint64, [C.c_uint64]),
    "orc_kmer_from_ascii": (C.c_int, [C.c_int, u8p, C.c_uint, u64p]),
    "orc_kmer_rev_comp": (C.c_int, [C.c_int, u64p, C.c_uint, u64p]),
    "orc_kmer_to_u64": (C.c_uint64, [C.c_int, u64p]),
    "orc_rolling_canonicals": (C.c_int, [C.c_int, u8p, C.c_uint64, C.c_uint, u64p, u8p]),
    "orc_nthash_fwd": (C.c_uint64, [u8p, C.c_uint]),
    "orc_nthash_rev": (C.c_uint64, [u8p, C.c_uint]),
    "orc_nthash_canonical": (C.c_uint64, [u8p, C.c_uint]),
    "orc_nthash_rolling_all": (C.c_int, [u8p, C.c_uint64, C.c_uint, u64p]),
    "orc_hll_new": (vp, [C.c_uint]),
    "orc_hll_free": (None, [vp]),
    "orc_hll_add_hash": (None, [vp, C.c_uint64]),
    "orc_hll_add_hashes": (None, [vp, u64p, C.c_uint64]),
    "orc_hll_add_canonical_hashes": (None, [vp, u64p, C.c_uint64]),
    "orc_hll_merge": (None, [vp, vp]),
    "orc_hll_estimate": (C.c_double, [vp]),
    "orc_hll_estimate_regs": (C.c_double, [u8p, C.c_uint]),
    "orc_hll_registers": (None, [vp, u8p]),
    "orc_cms_new": (vp, [C.c_uint64, C.c_int]),
    "orc_cms_free": (None, [vp]),
    "orc_cms_width": (C.c_uint64, [vp]),
    "orc_cms_add": (None, [vp, C.c_uint64]),
    "orc_cms_add_many": (None, [vp, u64p, C.c_uint64]),
    "orc_cms_estimate": (C.c_uint32, [vp, C.c_uint64]),
    "orc_cms_add_and_estimate": (C.c_uint32, [vp, C.c_uint64]),
    "orc_cms_nbytes": (C.c_uint64, [vp]),
    "orc_cms_export": (None, [vp, u8p]),
    "orc_cms_import": (None, [vp, u8p]),
    "orc_compact": (vp, [C.c_int, C.c_uint, u64p, u16p, u8p, C.c_uint64]),
    "orc_compact_count": (C.c_uint64, [vp]),
    "orc_compact_bases": (C.c_uint64, [vp]),
    "orc_compact_n_edges": (C.c_uint64, [vp]),
    "orc_compact_export": (None, [vp, u8p, u64p, C.POINTER(C.c_float), u8p, u32p]),
    "orc_compact_free": (None, [vp]),
    "orc_index_terminal_kmers": (C.c_uint64, [C.c_int, C.c_uint, u8p, u64p, C.c_uint64, u64p, u32p, u8p, u32p, C.c_uint64]),
    "orc_filter_active_reads": (C.c_uint64, [C.POINTER(OrcArena), u8p, u64p, u8p, u32p, u32p, C.c_uint64, C.c_uint, u8p]),
    "orc_build_pass1": (C.c_int, [C.POINTER(OrcArena), C.c_uint, C.c_int, vp, C.c_int, u64p, C.POINTER(u32p)]),
    "orc_build_pass1_contigs": (C.c_int, [u8p, u64p, C.c_uint64, C.c_uint, C.c_int, vp]),
    "orc_build_pass2": (vp, [C.POINTER(OrcArena), C.c_uint, C.c_int, vp, C.c_uint, C.c_int, u64p, C.POINTER(u32p), u8p,
                             u64p, C.c_uint64]),
    "orc_table_free": (None, [vp]),
    "orc_table_n_keys": (C.c_uint64, [vp]),
    "orc_table_export_acc": (C.c_uint64, [vp, u64p, u16p, u16p, C.c_uint64]),
    "orc_table_export_solid": (C.c_uint64, [vp, C.c_uint, u64p, u16p, u8p, C.c_uint64]),
    "orc_table_solid_digest": (C.c_uint64, [vp, C.c_uint, u64p]),
    "orc_table_acc_digest": (C.c_uint64, [vp, u64p]),
    "orc_trim_adapter": (C.c_uint64, [u8p, C.c_uint64]),
    "orc_trim_quality": (C.c_int64, [u8p, C.c_uint64, C.c_uint, C.c_uint64]),
    "orc_merge_read_pair": (C.c_int64, [u8p, u8p, C.c_uint64, u8p, u8p, C.c_uint64, C.c_uint64, C.c_double, u8p, u64p,
                                        u64p]),
    "orc_ingest_fastq": (vp, [C.c_char_p, C.c_char_p, C.c_double, C.c_uint64, C.c_uint, C.c_int, C.c_int, C.c_uint64,
                              C.c_char_p, C.c_int]),
    "orc_ingest_sizes": (None, [vp, C.c_int, u64p, u64p]),
    "orc_ingest_export": (None, [vp, C.c_int, u64p, u64p, u32p, u32p]),
    "orc_ingest_stats": (None, [vp, u64p]),
    "orc_ingest_free": (None, [vp]),
    "orc_compute_dynamic_kmers": (C.c_int, [C.c_uint64, C.c_int64, u64p, C.c_int]),
    "orc_subsample_keep": (C.c_int, [C.c_uint64, C.c_double, C.c_uint64]),
    "orc_estimate_from_reads": (C.c_int, [u8p, u64p, C.c_uint64, C.POINTER(OrcCountStats), C.c_uint64, C.c_double, C.c_uint,
                                          C.c_uint64, C.c_uint, C.POINTER(OrcEstimate), u8p, u8p]),
    "orc_est_firstpos": (None, [u8p, u64p, C.c_uint64, C.c_uint64, C.c_uint, C.c_uint64, u32p]),
    "orc_est_segments": (None, [u8p, u64p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint, C.c_uint64, C.c_uint, u32p, u8p]),
    "orc_count_fastx_exact": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(OrcCountStats), C.c_char_p, C.c_int]),
    "orc_estimate_genome": (C.c_int, [C.c_char_p, C.c_char_p, C.c_uint64, C.c_double, C.POINTER(OrcEstimate), u8p, u8p,
                                      C.c_char_p, C.c_int]),
}

_lib = None


def build() -> Path:
    src = HERE / "fbk_oracle.cpp"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["sh", str(HERE / "build_oracle.sh")], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        for n, (r, a) in _SIG.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def p(a: np.ndarray):
    if a is None:
        return None
    t = {np.dtype(np.uint8): C.c_uint8, np.dtype(np.uint16): C.c_uint16, np.dtype(np.uint32): C.c_uint32,
         np.dtype(np.uint64): C.c_uint64}[a.dtype]
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(t))


def arenas3(bank) -> C.Array:
    """Three OrcArena views of a fastbact_gb300.api.ReadBank-like object."""
    arr = (OrcArena * 3)()
    for i, a in enumerate([bank.merged_reads, bank.pe_forward, bank.pe_reverse]):
        arr[i] = OrcArena(p(a.data), a.data.size, p(a.offsets), p(a.lengths), a.offsets.size)
    return arr


def pair_idx3(bank):
    arr = (u32p * 3)()
    for i, a in enumerate([bank.merged_reads, bank.pe_forward, bank.pe_reverse]):
        arr[i] = p(a.pair_idx) if a.pair_idx is not None and a.pair_idx.size else None
    return arr


class Cms:
    def __init__(self, width: int, counter_bits: int = 4):
        self.h = lib().orc_cms_new(width, counter_bits)
        assert self.h

    def add(self, keys):
        k = np.ascontiguousarray(np.atleast_1d(np.asarray(keys, np.uint64)))
        lib().orc_cms_add_many(self.h, p(k), k.size)

    def estimate(self, key: int) -> int:
        return lib().orc_cms_estimate(self.h, key)

    def export(self) -> np.ndarray:
        out = np.zeros(lib().orc_cms_nbytes(self.h), np.uint8)
        lib().orc_cms_export(self.h, p(out))
        return out

    def load(self, raw: np.ndarray) -> None:
        """Replaces the counters with raw bytes in the export layout."""
        raw = np.ascontiguousarray(raw, dtype=np.uint8)
        assert raw.size == lib().orc_cms_nbytes(self.h)
        lib().orc_cms_import(self.h, p(raw))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_cms_free(self.h)
            self.h = None


class Hll:
    def __init__(self, pp: int = 14):
        self.pp = pp
        self.h = lib().orc_hll_new(pp)

    def add_hash(self, xs):
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(xs, np.uint64)))
        lib().orc_hll_add_hashes(self.h, p(a), a.size)

    def add_canonical_hash(self, xs):
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(xs, np.uint64)))
        lib().orc_hll_add_canonical_hashes(self.h, p(a), a.size)

    def merge(self, o: "Hll"):
        lib().orc_hll_merge(self.h, o.h)

    def estimate(self) -> float:
        return lib().orc_hll_estimate(self.h)

    def registers(self) -> np.ndarray:
        r = np.zeros(1 << self.pp, np.uint8)
        lib().orc_hll_registers(self.h, p(r))
        return r

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_hll_free(self.h)
            self.h = None


class Table:
    def __init__(self, h, key_bits: int):
        self.h, self.nw = h, key_bits // 64

    def n_keys(self) -> int:
        return lib().orc_table_n_keys(self.h)

    def export_acc(self):
        n = self.n_keys()
        keys = np.zeros((n, self.nw), np.uint64)
        cov = np.zeros(n, np.uint16)
        edges = np.zeros((n, 8), np.uint16)
        lib().orc_table_export_acc(self.h, p(keys.reshape(-1)), p(cov), p(edges.reshape(-1)), n)
        return keys, cov, edges

    def export_solid(self, min_trans_cov: int):
        n = self.n_keys()
        keys = np.zeros((n, self.nw), np.uint64)
        cov = np.zeros(n, np.uint16)
        mask = np.zeros(n, np.uint8)
        m = lib().orc_table_export_solid(self.h, min_trans_cov, p(keys.reshape(-1)), p(cov), p(mask), n)
        return keys[:m], cov[:m], mask[:m]

    def digest(self, min_trans_cov: int):
        n = C.c_uint64()
        d = lib().orc_table_solid_digest(self.h, min_trans_cov, C.byref(n))
        return d, n.value

    def acc_digest(self):
        """(order-free digest of every accumulated key with its KmerAcc, n_keys)."""
        n = C.c_uint64()
        d = lib().orc_table_acc_digest(self.h, C.byref(n))
        return d, n.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_table_free(self.h)
            self.h = None


def build_front(bank, k: int, key_bits: int, log2w: int, counter_bits: int = 4, target_solid_cov=None, threads: int = 0,
                keep_mask=None, contigs=None):
    """Oracle of build.rs:84-328 for a ReadBank: returns (Cms, Table, t_solid, min_trans_cov)."""
    cms = Cms(1 << log2w, counter_bits)
    ar = arenas3(bank)
    pidx = pair_idx3(bank) if keep_mask is not None else None
    km = p(keep_mask) if keep_mask is not None else None
    rc = lib().orc_build_pass1(ar, k, key_bits, cms.h, threads, km, pidx)
    assert rc == 0
    ca, co, nc = None, None, 0
    if contigs:
        ascii = np.frombuffer(b"".join(contigs), np.uint8).copy()
        offs = np.zeros(len(contigs) + 1, np.uint64)
        offs[1:] = np.cumsum([len(c) for c in contigs])
        ca, co, nc = ascii, offs, len(contigs)
        assert lib().orc_build_pass1_contigs(p(ca), p(co), nc, k, key_bits, cms.h) == 0
    t_solid = 2 if target_solid_cov is None else target_solid_cov
    mtc = 3 if target_solid_cov is None else target_solid_cov
    h = lib().orc_build_pass2(ar, k, key_bits, cms.h, t_solid, threads, km, pidx, p(ca) if ca is not None else None,
                              p(co) if co is not None else None, nc)
    assert h
    return cms, Table(h, key_bits), t_solid, mtc


def estimate_from_reads(seqs_r1r2: list[bytes], stats: OrcCountStats, max_pairs: int, target_cov: float, k: int = 21,
                        cms_width: int = 1 << 23, hll_p: int = 14):
    """Estimator oracle over in-memory raw reads (R1,R2 interleaved)."""
    buf = np.frombuffer(b"".join(seqs_r1r2), np.uint8).copy() if seqs_r1r2 else np.zeros(1, np.uint8)
    offs = np.zeros(len(seqs_r1r2) + 1, np.uint64)
    if seqs_r1r2:
        offs[1:] = np.cumsum([len(s) for s in seqs_r1r2])
    e = OrcEstimate()
    rt = np.zeros(1 << hll_p, np.uint8)
    rs = np.zeros(1 << hll_p, np.uint8)
    rc = lib().orc_estimate_from_reads(p(buf), p(offs), len(seqs_r1r2) // 2, C.byref(stats), max_pairs, target_cov, k,
                                       cms_width, hll_p, C.byref(e), p(rt), p(rs))
    return rc, e, rt, rs


def _reads_buf(seqs_r1r2: list[bytes]):
    buf = np.frombuffer(b"".join(seqs_r1r2), np.uint8).copy() if seqs_r1r2 else np.zeros(1, np.uint8)
    offs = np.zeros(len(seqs_r1r2) + 1, np.uint64)
    if seqs_r1r2:
        offs[1:] = np.cumsum([len(s) for s in seqs_r1r2])
    return buf, offs


def est_firstpos(seqs_r1r2: list[bytes], pair_begin: int, pair_end: int, k: int, cms_width: int) -> np.ndarray:
    """A rank's first-touch array of the sharded estimator (pairs [pair_begin, pair_end))."""
    buf, offs = _reads_buf(seqs_r1r2)
    first = np.zeros(4 * cms_width, np.uint32)
    lib().orc_est_firstpos(p(buf), p(offs), pair_begin, pair_end, k, cms_width, p(first))
    return first


def est_segments(seqs_r1r2: list[bytes], n_use: int, pair_begin: int, pair_end: int, k: int, cms_width: int, hll_p: int,
                 first: np.ndarray) -> np.ndarray:
    """A rank's per-segment HLL register maxima of the sharded estimator."""
    buf, offs = _reads_buf(seqs_r1r2)
    n_segs = 1 if n_use <= 6000 else 1 + (n_use - 6000 + 1999) // 2000
    regs = np.zeros(2 * n_segs << hll_p, np.uint8)
    first = np.ascontiguousarray(first, np.uint32)
    lib().orc_est_segments(p(buf), p(offs), n_use, pair_begin, pair_end, k, cms_width, hll_p, p(first), p(regs))
    return regs


def count_stats(**kw) -> OrcCountStats:
    s = OrcCountStats()
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def compact(keys: np.ndarray, cov: np.ndarray, mask: np.ndarray, k: int, key_bits: int):
    """Oracle of build.rs:330-594: SolidKmerNode rows -> (seqs list[bytes], cov f32[n],
    circular bool[n], edges u32[m, 6] = from id, from side, to id, to rc, overlap, support)."""
    keys = np.ascontiguousarray(keys, np.uint64).reshape(-1)
    cov = np.ascontiguousarray(cov, np.uint16)
    mask = np.ascontiguousarray(mask, np.uint8)
    h = lib().orc_compact(key_bits, k, p(keys), p(cov), p(mask), len(cov))
    assert h
    try:
        n = lib().orc_compact_count(h)
        nb = lib().orc_compact_bases(h)
        ne = lib().orc_compact_n_edges(h)
        seqs = np.zeros(max(nb, 1), np.uint8)
        offs = np.zeros(n + 1, np.uint64)
        cv = np.zeros(max(n, 1), np.float32)
        circ = np.zeros(max(n, 1), np.uint8)
        edges = np.zeros((max(ne, 1), 6), np.uint32)
        lib().orc_compact_export(h, p(seqs), p(offs), cv.ctypes.data_as(C.POINTER(C.c_float)), p(circ), p(edges.reshape(-1)))
    finally:
        lib().orc_compact_free(h)
    out = [seqs[offs[i]:offs[i + 1]].tobytes() for i in range(n)]
    return out, cv[:n], circ[:n].astype(bool), edges[:ne]


def edge_counts(n: int, edges: np.ndarray):
    """Edges per unitig side (edges_fwd.len(), edges_rev.len()) from the export layout."""
    e = np.asarray(edges).reshape(-1, 6)
    fwd = np.bincount(e[e[:, 1] == 0, 0].astype(np.int64), minlength=n)[:n].astype(np.uint32)
    rev = np.bincount(e[e[:, 1] == 1, 0].astype(np.int64), minlength=n)[:n].astype(np.uint32)
    return fwd, rev


def filter_active_reads(bank, seqs: list, circular, edges, graph_k: int):
    """Oracle of local_multik.rs:259-333: keep byte per read (merged, pe_fwd, pe_rev)."""
    n = len(seqs)
    useq = np.frombuffer(b"".join(seqs), np.uint8).copy() if seqs else np.zeros(1, np.uint8)
    uoff = np.zeros(n + 1, np.uint64)
    uoff[1:] = np.cumsum([len(x) for x in seqs]) if n else []
    circ = np.ascontiguousarray(np.asarray(circular, np.uint8)) if n else np.zeros(1, np.uint8)
    fwd, rev = edge_counts(n, edges)
    ar = arenas3(bank)
    total = sum(len(a) for a in bank.arenas)
    keep = np.zeros(max(total, 1), np.uint8)
    lib().orc_filter_active_reads(ar, p(useq), p(uoff), p(circ), p(np.ascontiguousarray(fwd)), p(np.ascontiguousarray(rev)),
                                  n, graph_k, p(keep))
    return keep[:total]


def index_terminal_kmers(seqs: list, k: int, key_bits: int):
    """Oracle of mapper.rs:89-136: (keys u64, unitig u32, is_rc u8, pos u32) sorted by key."""
    n = len(seqs)
    useq = np.frombuffer(b"".join(seqs), np.uint8).copy() if n else np.zeros(1, np.uint8)
    uoff = np.zeros(n + 1, np.uint64)
    if n:
        uoff[1:] = np.cumsum([len(x) for x in seqs])
    cap = sum(max(0, len(x) - k + 1) for x in seqs) + 1
    keys, uni = np.zeros(cap, np.uint64), np.zeros(cap, np.uint32)
    rc, pos = np.zeros(cap, np.uint8), np.zeros(cap, np.uint32)
    m = lib().orc_index_terminal_kmers(key_bits, k, p(useq), p(uoff), n, p(keys), p(uni), p(rc), p(pos), cap)
    return keys[:m], uni[:m], rc[:m], pos[:m]


# ---------------------------------------------------------------------------
# read ingest (trim_merge.rs:17-238, 307-417)
# ---------------------------------------------------------------------------
def _u8(b: bytes) -> np.ndarray:
    return np.frombuffer(b, np.uint8).copy() if b else np.zeros(1, np.uint8)


def trim_adapter(seq: bytes) -> int:
    """Kept length after 3' adapter clipping."""
    return int(lib().orc_trim_adapter(p(_u8(seq)), len(seq)))


def trim_quality(qual: bytes, min_qual: int, min_len: int):
    """Kept length after the 4-base window trim, or None."""
    n = lib().orc_trim_quality(p(_u8(qual)), len(qual), min_qual, min_len)
    return None if n < 0 else int(n)


def merge_read_pair(r1: bytes, q1: bytes, r2: bytes, q2: bytes, min_overlap: int = 15, ratio: float = 0.10):
    """(merged sequence, overlap, mismatches), or None when the pair stays unmerged."""
    out = np.zeros(len(r1) + len(r2) + 1, np.uint8)
    ov, mm = C.c_uint64(), C.c_uint64()
    n = lib().orc_merge_read_pair(p(_u8(r1)), p(_u8(q1)), len(r1), p(_u8(r2)), p(_u8(q2)), len(r2), min_overlap, ratio,
                                  p(out), C.byref(ov), C.byref(mm))
    return None if n < 0 else (out[:n].tobytes(), ov.value, mm.value)


INGEST_STATS = ("input_read_pairs", "retained_read_pairs", "bases_before_trim", "bases_after_trim", "merged_pairs_count",
                "merged_bases", "unmerged_pairs_count")


def ingest_fastq(r1: str, r2: str, subsample_factor: float = 1.0, min_len: int = 30, min_qual: int = 20,
                 enable_trim: bool = True, enable_merge: bool = True, seed: int = 0):
    """ingest_reads_ext_with_seed: ([3 arenas as (data, offsets, lengths, pair_idx)], stats dict).
    Raises RuntimeError with the reference's message on failure."""
    err = C.create_string_buffer(1024)
    h = lib().orc_ingest_fastq(str(r1).encode(), str(r2).encode(), subsample_factor, min_len, min_qual, int(enable_trim),
                               int(enable_merge), seed, err, len(err))
    if not h:
        raise RuntimeError(err.value.decode(errors="replace"))
    try:
        arenas = []
        for a in range(3):
            nw, ns = C.c_uint64(), C.c_uint64()
            lib().orc_ingest_sizes(h, a, C.byref(nw), C.byref(ns))
            d = np.zeros(max(nw.value, 1), np.uint64)
            o = np.zeros(max(ns.value, 1), np.uint64)
            L = np.zeros(max(ns.value, 1), np.uint32)
            pi = np.zeros(max(ns.value, 1), np.uint32)
            lib().orc_ingest_export(h, a, p(d), p(o), p(L), p(pi))
            arenas.append((d[:nw.value], o[:ns.value], L[:ns.value], pi[:ns.value]))
        st = np.zeros(7, np.uint64)
        lib().orc_ingest_stats(h, p(st))
        return arenas, dict(zip(INGEST_STATS, (int(x) for x in st)))
    finally:
        lib().orc_ingest_free(h)
