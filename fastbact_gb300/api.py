"""Python mirror of the reference's hot-path interface, backed by libfbk.so.

Names, argument meaning and error behaviour follow the Rust entry points of
fastBact (paths inside its repository):

* ``ReadBank`` / ``BitSeqArena``          — src/common/bitseq.rs:145-399
* ``CountMinSketch``                       — src/common/sketch.rs:121-253
* ``HyperLogLog``                          — src/common/sketch.rs:24-115
* ``count_fastx_exact``, ``estimate_genome``, ``compute_dynamic_kmers``
                                           — src/ingest/estimator.rs:104-440
* ``ingest_reads_ext_with_seed``           — src/ingest/trim_merge.rs:307-417
* ``build_cdbg*``                          — src/graph/build.rs:37-328 (front end:
  passes 1-2 and the SolidKmerNode conversion; the returned ``SolidTable`` is the
  table the unitig compaction walks)

Every computation on k-mers runs in the device kernels; this module only moves
buffers and parameters across the C ABI.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from ._native import check, ptr

CONFIDENCE = {0: "HIGH", 1: "LOW_COVERAGE_WARNING", 2: "UNRELIABLE"}


def key_bits_for_k(k: int) -> int:
    """KmerInt width the reference dispatches to (src/main.rs:350-364)."""
    if k <= 31:
        return 64
    if k <= 63:
        return 128
    if k <= 127:
        return 256
    raise ValueError(f"k={k} exceeds 127")


def splitmix64(z: int) -> int:
    z &= (1 << 64) - 1
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & ((1 << 64) - 1)
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & ((1 << 64) - 1)
    return z ^ (z >> 31)


# ---------------------------------------------------------------------------
# context
# ---------------------------------------------------------------------------
class Context:
    """One device, one stream, one (optional) memory pool.

    Device objects created on a context register with it; closing the context
    releases them first, so no object outlives the context it points into."""

    def __init__(self, device: int = 0, pool_bytes: int = 0):
        self._h = C.c_void_p()
        self._children = weakref.WeakSet()
        st = N.lib().fbk_ctx_create(device, pool_bytes, C.byref(self._h))
        if st != N.FBK_OK:
            raise N.FbkError(st, f"fbk_ctx_create(device={device})")
        self.device = device

    @property
    def handle(self):
        return self._h

    @property
    def alive(self) -> bool:
        return bool(self._h)

    def adopt(self, obj) -> None:
        self._children.add(obj)

    def close(self):
        if self._h:
            for child in list(self._children):
                child.release()
            N.lib().fbk_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(N.lib().fbk_ctx_sync(self._h), self._h)

    def set_timing(self, on: bool):
        check(N.lib().fbk_ctx_set_timing(self._h, 1 if on else 0), self._h)

    def timing(self, prefix: str = "") -> tuple[float, int]:
        ms, n = C.c_double(), C.c_uint64()
        check(N.lib().fbk_ctx_timing(self._h, prefix.encode(), C.byref(ms), C.byref(n)), self._h)
        return ms.value, n.value

    def timing_reset(self):
        check(N.lib().fbk_ctx_timing_reset(self._h), self._h)

    def set_tuning(self, **kw) -> None:
        for name, v in kw.items():
            check(N.lib().fbk_ctx_set_tuning(self._h, name.encode(), float(v)), self._h, "set_tuning")

    def get_tuning(self, name: str) -> float:
        v = C.c_double()
        check(N.lib().fbk_ctx_get_tuning(self._h, name.encode(), C.byref(v)), self._h, "get_tuning")
        return v.value

    def record(self, slot: int) -> None:
        check(N.lib().fbk_ctx_event_record(self._h, slot), self._h)

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_double()
        check(N.lib().fbk_ctx_event_elapsed(self._h, a, b, C.byref(ms)), self._h)
        return ms.value

    def launch_count(self) -> int:
        n = C.c_uint64()
        check(N.lib().fbk_ctx_launch_count(self._h, C.byref(n)), self._h)
        return n.value

    def mem_info(self) -> tuple[int, int]:
        u, s = C.c_uint64(), C.c_uint64()
        check(N.lib().fbk_ctx_mem_info(self._h, C.byref(u), C.byref(s)), self._h)
        return u.value, s.value


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---------------------------------------------------------------------------
# read bank (host side)
# ---------------------------------------------------------------------------
_A2B = np.zeros(256, dtype=np.uint8)
for _c, _v in ((b"C", 1), (b"c", 1), (b"G", 2), (b"g", 2), (b"T", 3), (b"t", 3)):
    _A2B[_c[0]] = _v


@dataclass
class BitSeqArena:
    """BitSeqArena: base i at bits 2*(i%32) of data[i/32] (bitseq.rs:145-222)."""
    data: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))
    offsets: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))
    lengths: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))
    pair_idx: np.ndarray | None = None

    @staticmethod
    def from_seqs(seqs: list[bytes], pair_idx: list[int] | None = None) -> "BitSeqArena":
        lengths = np.array([len(s) for s in seqs], dtype=np.uint32)
        offsets = np.zeros(len(seqs), dtype=np.uint64)
        if len(seqs):
            offsets[1:] = np.cumsum(lengths[:-1], dtype=np.uint64)
        total = int(lengths.sum(dtype=np.uint64))
        codes = _A2B[np.frombuffer(b"".join(seqs), dtype=np.uint8)] if total else np.zeros(0, np.uint8)
        return BitSeqArena(pack_codes(codes), offsets, lengths,
                           None if pair_idx is None else np.asarray(pair_idx, dtype=np.uint32))

    def __len__(self):
        return int(self.offsets.size)

    def total_bases(self) -> int:
        return int(self.lengths.sum(dtype=np.uint64))

    def extract_ascii(self, i: int) -> bytes:
        o, n = int(self.offsets[i]), int(self.lengths[i])
        g = np.arange(o, o + n, dtype=np.uint64)
        codes = (self.data[g >> np.uint64(5)] >> ((g & np.uint64(31)) << np.uint64(1))) & np.uint64(3)
        return np.frombuffer(b"ACGT", dtype=np.uint8)[codes.astype(np.intp)].tobytes()

    def view(self) -> N.ArenaView:
        return N.arena_view(self.data, self.offsets, self.lengths, self.pair_idx)


def pack_codes(codes: np.ndarray) -> np.ndarray:
    """Packs 2-bit codes LSB-first, 32 per u64 word."""
    n = codes.size
    nw = (n + 31) // 32
    padded = np.zeros(nw * 32, dtype=np.uint64)
    padded[:n] = codes
    shifts = (np.arange(32, dtype=np.uint64) * np.uint64(2))
    return np.bitwise_or.reduce(padded.reshape(nw, 32) << shifts, axis=1).astype(np.uint64) if nw else np.zeros(0, np.uint64)


@dataclass
class IngestStats:
    input_read_pairs: int = 0
    retained_read_pairs: int = 0
    merged_pairs_count: int = 0
    unmerged_pairs_count: int = 0
    bases_before_trim: int = 0
    bases_after_trim: int = 0


@dataclass
class ReadBank:
    """ReadBank (bitseq.rs:350-399): merged reads, then unmerged R1, then R2."""
    merged_reads: BitSeqArena = field(default_factory=BitSeqArena)
    pe_forward: BitSeqArena = field(default_factory=BitSeqArena)
    pe_reverse: BitSeqArena = field(default_factory=BitSeqArena)

    @property
    def arenas(self):
        return [self.merged_reads, self.pe_forward, self.pe_reverse]

    def total_reads(self) -> int:
        return sum(len(a) for a in self.arenas)

    def total_bases(self) -> int:
        return sum(a.total_bases() for a in self.arenas)

    def views(self):
        arr = (N.ArenaView * 3)()
        for i, a in enumerate(self.arenas):
            arr[i] = a.view()
        return arr


def _arena_from_view(v: N.ArenaView) -> BitSeqArena:
    def cp(p, n, dt):
        if n == 0 or not p:
            return np.zeros(0, dt)
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)

    return BitSeqArena(cp(v.data, v.n_words, np.uint64), cp(v.offsets, v.n_seqs, np.uint64),
                       cp(v.lengths, v.n_seqs, np.uint32), cp(v.pair_idx, v.n_seqs, np.uint32))


def _bank_from_hbank(h, L=None) -> tuple[ReadBank, IngestStats]:
    """Copies a host bank out; L is the library that made it (libfbk or libfbk_synth)."""
    L = L or N.lib()
    arenas = []
    for i in range(3):
        v = N.ArenaView()
        check(L.fbk_hbank_arena(h, i, C.byref(v)))
        arenas.append(_arena_from_view(v))
    vals = [C.c_uint64() for _ in range(6)]
    check(L.fbk_hbank_stats(h, *[C.byref(x) for x in vals]))
    st = IngestStats(vals[0].value, vals[1].value, vals[2].value, vals[3].value, vals[4].value, vals[5].value)
    return ReadBank(*arenas), st


def ingest_reads_ext_with_seed(r1: str, r2: str, subsample_factor: float, min_len: int, min_qual: int,
                               enable_trim: bool = True, enable_merge: bool = True, seed: int = 0):
    """trim_merge.rs:307-417 (host-side CPU ingest producing the bank)."""
    h = C.c_void_p()
    err = C.create_string_buffer(1024)
    st = N.lib().fbk_ingest_fastq(str(r1).encode(), str(r2).encode(), subsample_factor, min_len, min_qual,
                                  int(enable_trim), int(enable_merge), seed, C.byref(h), err, len(err))
    if st != N.FBK_OK:
        raise N.FbkError(st, err.value.decode(errors="replace"))
    try:
        return _bank_from_hbank(h)
    finally:
        N.lib().fbk_hbank_free(h)


# ---------------------------------------------------------------------------
# estimator
# ---------------------------------------------------------------------------
@dataclass
class ExactCountStats:
    exact_read_pairs: int
    total_bases_r1: int
    total_bases_r2: int
    total_bases: int
    min_read_len: int
    max_read_len: int
    mean_read_len: float
    median_read_len: int

    @staticmethod
    def from_c(s: N.CountStats) -> "ExactCountStats":
        return ExactCountStats(s.exact_read_pairs, s.total_bases_r1, s.total_bases_r2, s.total_bases,
                               s.min_read_len, s.max_read_len, s.mean_read_len, s.median_read_len)

    def to_c(self) -> N.CountStats:
        s = N.CountStats()
        for f in ("exact_read_pairs", "total_bases_r1", "total_bases_r2", "total_bases", "min_read_len",
                  "max_read_len", "mean_read_len", "median_read_len"):
            setattr(s, f, getattr(self, f))
        return s


@dataclass
class GenomeEstimate:
    genome_size: int
    exact_read_pairs: int
    total_bases: int
    median_read_len: int
    max_read_len: int
    estimated_cov: float
    subsample_factor: float
    kmers: list
    confidence: str
    u_ge_1: int
    u_ge_2: int
    sample_kmer_depth: float
    pairs_sampled: int = 0
    m_sample: int = 0

    @staticmethod
    def from_c(e: N.GenomeEstimate) -> "GenomeEstimate":
        return GenomeEstimate(e.genome_size, e.exact_read_pairs, e.total_bases, e.median_read_len, e.max_read_len,
                              e.estimated_cov, e.subsample_factor, [e.kmers[i] for i in range(e.n_kmers)],
                              CONFIDENCE[e.confidence], e.u_ge_1, e.u_ge_2, e.sample_kmer_depth, e.pairs_sampled,
                              e.m_sample)

    def to_c(self) -> N.GenomeEstimate:
        e = N.GenomeEstimate()
        for f in ("genome_size", "exact_read_pairs", "total_bases", "median_read_len", "max_read_len", "estimated_cov",
                  "subsample_factor", "u_ge_1", "u_ge_2", "sample_kmer_depth", "pairs_sampled", "m_sample"):
            setattr(e, f, getattr(self, f))
        for i, k in enumerate(self.kmers[:8]):
            e.kmers[i] = k
        e.n_kmers = min(8, len(self.kmers))
        e.confidence = {v: c for c, v in CONFIDENCE.items()}[self.confidence]
        return e


def count_fastx_exact(r1: str, r2: str) -> ExactCountStats:
    s = N.CountStats()
    err = C.create_string_buffer(2048)
    st = N.lib().fbk_count_fastx_exact(str(r1).encode(), str(r2).encode(), C.byref(s), err, len(err))
    if st != N.FBK_OK:
        raise N.FbkError(st, err.value.decode(errors="replace"))
    return ExactCountStats.from_c(s)


def compute_dynamic_kmers(median_len: int, target_max_k: int | None = None) -> list[int]:
    out = (C.c_uint64 * 16)()
    n = N.lib().fbk_compute_dynamic_kmers(median_len, -1 if target_max_k is None else target_max_k, out, 16)
    return [out[i] for i in range(n)]


def estimator_params(**kw) -> N.EstimatorParams:
    p = N.EstimatorParams()
    N.lib().fbk_estimator_defaults(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def estimate_genome(r1: str, r2: str, max_pairs: int, target_cov: float, ctx: Context | None = None) -> GenomeEstimate:
    """estimator.rs:286-440: FASTQ scan on the host, sample loop on the device."""
    ctx = ctx or default_context()
    e = N.GenomeEstimate()
    check(N.lib().fbk_estimate_genome(ctx.handle, str(r1).encode(), str(r2).encode(), max_pairs, target_cov,
                                      C.byref(e)), ctx.handle, "estimate_genome")
    return GenomeEstimate.from_c(e)


def estimate_sample(ctx: Context, sample: BitSeqArena, n_pairs: int, stats: ExactCountStats, **params):
    """Device sample loop over packed raw reads (R1,R2 interleaved per pair).
    Returns (GenomeEstimate, regs_total, regs_solid)."""
    p = estimator_params(**params)
    m = 1 << p.hll_p
    rt = np.zeros(m, np.uint8)
    rs = np.zeros(m, np.uint8)
    v = sample.view()
    cs = stats.to_c()
    e = N.GenomeEstimate()
    check(N.lib().fbk_estimate_sample(ctx.handle, C.byref(v), n_pairs, C.byref(cs), C.byref(p), C.byref(e), ptr(rt),
                                      ptr(rs)), ctx.handle, "estimate_sample")
    return GenomeEstimate.from_c(e), rt, rs


def estimate_bank(ctx: Context, sample_bank: "DeviceBank", lengths: np.ndarray, n_pairs: int, stats: ExactCountStats,
                  want_registers: bool = False, **params):
    """estimate_sample on an already uploaded sample (R1,R2 interleaved)."""
    p = estimator_params(**params)
    m = 1 << p.hll_p
    rt = np.zeros(m, np.uint8) if want_registers else None
    rs = np.zeros(m, np.uint8) if want_registers else None
    cs = stats.to_c()
    e = N.GenomeEstimate()
    check(N.lib().fbk_estimate_bank(ctx.handle, sample_bank.handle, ptr(lengths), n_pairs, C.byref(cs), C.byref(p),
                                    C.byref(e), ptr(rt), ptr(rs)), ctx.handle, "estimate_bank")
    return GenomeEstimate.from_c(e), rt, rs


def est_shard_plan(lengths: np.ndarray, n_pairs: int, stats: ExactCountStats, **params) -> tuple[int, int]:
    """(n_use, n_segs) of the sharded estimator: the pairs the sample loop can read and
    its checkpoint segments (host only)."""
    p = estimator_params(**params)
    lengths = np.ascontiguousarray(lengths, np.uint32)
    cs = stats.to_c()
    n_use, n_segs = C.c_uint64(), C.c_uint32()
    check(N.lib().fbk_est_shard_plan(ptr(lengths), n_pairs, C.byref(cs), C.byref(p), C.byref(n_use), C.byref(n_segs)),
          None, "est_shard_plan")
    return n_use.value, n_segs.value


def est_shard_firstpos(ctx: Context, sample_bank: "DeviceBank", lengths: np.ndarray, n_use: int, pair_begin: int,
                       pair_end: int, **params) -> np.ndarray:
    """Stage 1 of the sharded estimator on this rank's pairs: the first occurrence
    index touching each sketch counter (uint32[4 << cms_log2_width])."""
    p = estimator_params(**params)
    lengths = np.ascontiguousarray(lengths, np.uint32)
    first = np.zeros(4 << p.cms_log2_width, np.uint32)
    check(N.lib().fbk_est_shard_firstpos(ctx.handle, sample_bank.handle, ptr(lengths), n_use, pair_begin, pair_end,
                                         C.byref(p), ptr(first)), ctx.handle, "est_shard_firstpos")
    return first


def est_shard_segments(ctx: Context, sample_bank: "DeviceBank", lengths: np.ndarray, n_use: int, pair_begin: int,
                       pair_end: int, first: np.ndarray, **params) -> np.ndarray:
    """Stage 2 on this rank's pairs with the merged first-touch array: HLL register
    maxima per checkpoint segment, uint8[2 * n_segs << hll_p] (total, then solid)."""
    p = estimator_params(**params)
    lengths = np.ascontiguousarray(lengths, np.uint32)
    n_segs = 1 if n_use <= 6000 else 1 + (n_use - 6000 + 1999) // 2000
    regs = np.zeros(2 * n_segs << p.hll_p, np.uint8)
    first = np.ascontiguousarray(first, np.uint32)
    check(N.lib().fbk_est_shard_segments(ctx.handle, sample_bank.handle, ptr(lengths), n_use, pair_begin, pair_end,
                                         C.byref(p), ptr(first), ptr(regs)), ctx.handle, "est_shard_segments")
    return regs


def est_shard_finish(lengths: np.ndarray, n_use: int, stats: ExactCountStats, regs: np.ndarray, **params):
    """Checkpoints and post-math from the merged segment registers (host only).
    Returns (GenomeEstimate, regs_total, regs_solid)."""
    p = estimator_params(**params)
    lengths = np.ascontiguousarray(lengths, np.uint32)
    regs = np.ascontiguousarray(regs, np.uint8)
    m = 1 << p.hll_p
    rt, rs = np.zeros(m, np.uint8), np.zeros(m, np.uint8)
    cs = stats.to_c()
    e = N.GenomeEstimate()
    check(N.lib().fbk_est_shard_finish(ptr(lengths), n_use, C.byref(cs), C.byref(p), ptr(regs), C.byref(e), ptr(rt),
                                       ptr(rs)), None, "est_shard_finish")
    return GenomeEstimate.from_c(e), rt, rs


# ---------------------------------------------------------------------------
# device objects
# ---------------------------------------------------------------------------
class DeviceBank:
    """A ReadBank uploaded to device memory."""

    def __init__(self, ctx: Context, bank: ReadBank | BitSeqArena, async_upload: bool = False):
        """async_upload: when every array is page-locked, return once the copies are
        queued (fbk_bank_upload_async); the bank keeps its host arrays alive, and every
        call that reads it waits for the copies on the device."""
        self.ctx = ctx
        if isinstance(bank, BitSeqArena):
            bank = ReadBank(merged_reads=bank)
        self._views = bank.views()
        self._host = bank if async_upload else None
        self._h = C.c_void_p()
        fn = N.lib().fbk_bank_upload_async if async_upload else N.lib().fbk_bank_upload
        check(fn(ctx.handle, self._views, C.byref(self._h)), ctx.handle, "bank upload")
        ctx.adopt(self)
        nr, nb = C.c_uint64(), C.c_uint64()  # the totals the upload's scan computed
        check(N.lib().fbk_bank_info(self._h, C.byref(nr), C.byref(nb)))
        self.n_reads, self.n_bases = nr.value, nb.value

    @classmethod
    def from_handle(cls, ctx: Context, h) -> "DeviceBank":
        """Wraps a bank made on the device (e.g. by ingest_fastq_device)."""
        self = cls.__new__(cls)
        self.ctx, self._h, self._views = ctx, h, None
        ctx.adopt(self)
        nr, nb = C.c_uint64(), C.c_uint64()
        check(N.lib().fbk_bank_info(h, C.byref(nr), C.byref(nb)))
        self.n_reads, self.n_bases = nr.value, nb.value
        return self

    def export(self):
        """(words, bank-global offsets, lengths, pair indices, reads per arena)."""
        nw = C.c_uint64()
        check(N.lib().fbk_bank_words(self._h, C.byref(nw)))
        words = np.zeros(max(nw.value, 1), np.uint64)
        offs = np.zeros(max(self.n_reads, 1), np.uint64)
        lens = np.zeros(max(self.n_reads, 1), np.uint32)
        pidx = np.zeros(max(self.n_reads, 1), np.uint32)
        check(N.lib().fbk_bank_export(self._h, ptr(words), ptr(offs), ptr(lens), ptr(pidx)), self.ctx.handle, "bank export")
        counts = np.zeros(3, np.uint64)
        check(N.lib().fbk_bank_arena_counts(self._h, ptr(counts)))
        n = self.n_reads
        return words[:nw.value], offs[:n], lens[:n], pidx[:n], [int(c) for c in counts]

    @property
    def handle(self):
        return self._h

    def release(self):
        if self._h and self.ctx.alive:
            N.lib().fbk_bank_release(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def _subsample(ss):
    if ss is None:
        return None
    factor, seed = ss
    s = N.Subsample()
    s.factor = factor
    s.seed = seed
    return C.byref(s)


class CountMinSketch:
    """4-row Count-Min Sketch on the device (sketch.rs:121-253).  counter_bits=4 is
    the reference nibble layout; 16 gives u16 counters."""

    def __init__(self, width: int, ctx: Context | None = None, counter_bits: int = 4):
        self.ctx = ctx or default_context()
        if width & (width - 1):
            width = 1 << (width - 1).bit_length()  # sketch.rs:141-143
        self.width = width
        self.counter_bits = counter_bits
        self._h = C.c_void_p()
        check(N.lib().fbk_cms_create(self.ctx.handle, width.bit_length() - 1, counter_bits, C.byref(self._h)),
              self.ctx.handle, "cms create")
        self.ctx.adopt(self)

    @classmethod
    def build(cls, ctx: Context, bank: "DeviceBank", k: int, log2_width: int, counter_bits: int = 4,
              key_bits: int | None = None) -> "CountMinSketch":
        """Pass 1 in one call (fbk_cms_build): a new sketch holding every k-mer of the bank."""
        self = cls.__new__(cls)
        self.ctx, self.width, self.counter_bits = ctx, 1 << log2_width, counter_bits
        self._h = C.c_void_p()
        check(N.lib().fbk_cms_build(ctx.handle, bank.handle, k, key_bits or key_bits_for_k(k), log2_width, counter_bits,
                                    C.byref(self._h)), ctx.handle, "cms build")
        ctx.adopt(self)
        return self

    @staticmethod
    def width_for_genome_size(g: int) -> int:
        return N.lib().fbk_cms_width_for_genome_size(g)

    @classmethod
    def for_genome_size(cls, g: int, ctx: Context | None = None, counter_bits: int = 4):
        return cls(cls.width_for_genome_size(g), ctx, counter_bits)

    def add(self, keys) -> None:
        k = np.ascontiguousarray(np.atleast_1d(np.asarray(keys, dtype=np.uint64)))
        check(N.lib().fbk_cms_add_keys(self._h, ptr(k), k.size), self.ctx.handle, "cms add")

    def estimate(self, keys) -> np.ndarray:
        k = np.ascontiguousarray(np.atleast_1d(np.asarray(keys, dtype=np.uint64)))
        out = np.zeros(k.size, np.uint32)
        check(N.lib().fbk_cms_estimate_keys(self._h, ptr(k), k.size, ptr(out)), self.ctx.handle, "cms estimate")
        return out

    def add_bank(self, bank: DeviceBank, k: int, key_bits: int | None = None, subsample=None) -> None:
        check(N.lib().fbk_cms_add_bank(self._h, bank.handle, k, key_bits or key_bits_for_k(k), _subsample(subsample)),
              self.ctx.handle, "cms pass 1")

    def add_contigs(self, contigs: list[bytes], k: int, key_bits: int | None = None) -> None:
        ascii, offs = _contig_buffers(contigs)
        check(N.lib().fbk_cms_add_contigs(self._h, ptr(ascii), ptr(offs), len(contigs), k, key_bits or key_bits_for_k(k)),
              self.ctx.handle, "cms contigs")

    def export(self) -> np.ndarray:
        n = C.c_uint64()
        check(N.lib().fbk_cms_nbytes(self._h, C.byref(n)))
        out = np.zeros(n.value, np.uint8)
        check(N.lib().fbk_cms_export(self._h, ptr(out), n.value), self.ctx.handle, "cms export")
        return out

    def load(self, raw: np.ndarray) -> None:
        """Replaces the counters with bytes in the export layout."""
        raw = np.ascontiguousarray(raw, dtype=np.uint8)
        check(N.lib().fbk_cms_import(self._h, ptr(raw), raw.size), self.ctx.handle, "cms import")

    def counts_tensor(self):
        """The device counters (4 rows of 2^log2w u32, each <= 65535 between calls) as
        an int32 CUDA tensor that aliases them (no copy): a collective can reduce the
        sketches of several ranks in place.  Call clamp_counts() afterwards."""
        import torch

        ptr_, n = C.c_void_p(), C.c_uint64()
        check(N.lib().fbk_cms_counts_device(self._h, C.byref(ptr_), C.byref(n)), self.ctx.handle, "cms counters")
        return torch.as_tensor(_CudaArray(ptr_.value, (n.value,), "<i4"), device="cuda")

    def clamp_counts(self) -> None:
        check(N.lib().fbk_cms_clamp_counts(self._h), self.ctx.handle, "cms clamp")

    def merge(self, other: "CountMinSketch") -> None:
        check(N.lib().fbk_cms_merge(self._h, other._h), self.ctx.handle, "cms merge")

    def clear(self) -> None:
        check(N.lib().fbk_cms_clear(self._h), self.ctx.handle)

    def release(self):
        if self._h and self.ctx.alive:
            N.lib().fbk_cms_release(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class HyperLogLog:
    """HyperLogLog on the device (sketch.rs:24-115); p = 14 in the reference."""

    def __init__(self, p: int = 14, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.p = p
        self._h = C.c_void_p()
        check(N.lib().fbk_hll_create(self.ctx.handle, p, C.byref(self._h)), self.ctx.handle, "hll create")
        self.ctx.adopt(self)

    def add_hash(self, h) -> None:
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(h, dtype=np.uint64)))
        check(N.lib().fbk_hll_add_hashes(self._h, ptr(a), a.size), self.ctx.handle)

    def add_canonical_hash(self, h) -> None:
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(h, dtype=np.uint64)))
        check(N.lib().fbk_hll_add_canonical_hashes(self._h, ptr(a), a.size), self.ctx.handle)

    def merge(self, other: "HyperLogLog") -> None:
        check(N.lib().fbk_hll_merge(self._h, other._h), self.ctx.handle)

    def registers(self) -> np.ndarray:
        r = np.zeros(1 << self.p, np.uint8)
        check(N.lib().fbk_hll_export(self._h, ptr(r), r.size), self.ctx.handle)
        return r

    def estimate(self) -> float:
        d = C.c_double()
        check(N.lib().fbk_hll_estimate(self._h, C.byref(d)), self.ctx.handle)
        return d.value

    def release(self):
        if self._h and self.ctx.alive:
            N.lib().fbk_hll_release(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class SolidTable:
    """Device-resident solid k-mer table (SolidKmerNode rows, build.rs:295-328)."""

    def __init__(self, ctx: Context, handle, k: int, key_bits: int):
        self.ctx, self._h, self.k, self.key_bits = ctx, handle, k, key_bits
        self.nw = key_bits // 64
        self._pending = None
        ctx.adopt(self)

    @property
    def handle(self):
        return self._h

    def info(self) -> tuple[int, int, int]:
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(N.lib().fbk_table_info(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def __len__(self):
        return self.info()[1]

    def _out_rows(self, n_solid: int, out):
        if out is not None and len(out[1]) >= n_solid and len(out[2]) >= n_solid and len(out[0]) >= n_solid:
            keys, cov, mask = out[0][:n_solid], out[1][:n_solid], out[2][:n_solid]
            if keys.dtype != np.uint64 or keys.shape[1:] != (self.nw,) or not keys.flags.c_contiguous \
                    or cov.dtype != np.uint16 or mask.dtype != np.uint8:
                raise ValueError("export: out must be (uint64[n, nw], uint16[n], uint8[n]) C-contiguous arrays")
            return keys, cov, mask
        return np.zeros((n_solid, self.nw), np.uint64), np.zeros(n_solid, np.uint16), np.zeros(n_solid, np.uint8)

    def export(self, sort: bool = False, out=None):
        """(keys[n, nw] big-endian words, cov u16, mask u8).  `out` = (keys, cov, mask)
        arrays with room for at least n rows (e.g. reused pinned buffers) receive the
        rows; the returned arrays are views of their first n rows."""
        n_solid = self.info()[1]
        keys, cov, mask = self._out_rows(n_solid, out)
        n = C.c_uint64()
        check(N.lib().fbk_table_export(self._h, ptr(keys.reshape(-1)), ptr(cov), ptr(mask), n_solid, C.byref(n)),
              self.ctx.handle, "table export")
        return sort_rows(keys, cov, mask) if sort else (keys, cov, mask)

    def export_async(self, out):
        """Queues the copy of the rows into `out` = (keys, cov, mask) page-locked arrays
        with room for every row and returns at once; export_wait() returns the rows
        (views of out) once they have arrived.  The next build may run meanwhile."""
        n_solid = self.info()[1]
        keys, cov, mask = self._out_rows(n_solid, out)
        n = C.c_uint64()
        check(N.lib().fbk_table_export_async(self._h, ptr(keys.reshape(-1)), ptr(cov), ptr(mask), n_solid, C.byref(n)),
              self.ctx.handle, "table export_async")
        self._pending = (keys, cov, mask)

    def export_wait(self):
        check(N.lib().fbk_table_export_wait(self._h), self.ctx.handle, "table export_wait")
        rows, self._pending = self._pending, None
        return rows

    def export_acc(self, sort: bool = True):
        """Every accumulated key: (keys[n, nw], cov u16, edge_counts[n, 8] u16)."""
        n_keys = self.info()[0]
        keys = np.zeros((n_keys, self.nw), np.uint64)
        cov = np.zeros(n_keys, np.uint16)
        edges = np.zeros((n_keys, 8), np.uint16)
        n = C.c_uint64()
        check(N.lib().fbk_table_export_acc(self._h, ptr(keys.reshape(-1)), ptr(cov), ptr(edges.reshape(-1)), n_keys,
                                           C.byref(n)), self.ctx.handle, "table export_acc")
        return sort_rows(keys, cov, edges) if sort else (keys, cov, edges)

    def filtered(self) -> bool:
        """True when the accumulator holds only keys that may become SolidKmerNodes
        (keys seen in fewer than min_trans_cov windows were kept out of the table)."""
        f = C.c_uint32()
        check(N.lib().fbk_table_flags(self._h, C.byref(f)))
        return bool(f.value & 1)

    def pushes(self) -> int:
        n = C.c_uint64()
        check(N.lib().fbk_table_pushes(self._h, C.byref(n)))
        return n.value

    def export_acc_owned(self, world: int):
        """Every accumulated key with its 8 edge counts, grouped by owner rank
        (splitmix64(fold(key)) mod world), as an int64 CUDA tensor of
        (n, key_bits/64 + 2) rows (key words, then the edge counts packed as u16
        fields), and the rows per owner."""
        import torch

        n = self.info()[0]
        rows = torch.empty((max(n, 1), self.nw + 2), dtype=torch.int64, device="cuda")
        counts = np.zeros(world, np.uint64)
        torch.cuda.synchronize()
        check(N.lib().fbk_table_export_acc_owned(self._h, world, C.c_void_p(rows.data_ptr()), n, ptr(counts)),
              self.ctx.handle, "owner rows")
        return rows[:n], [int(c) for c in counts]

    def acc_digest(self) -> tuple[int, int]:
        """(order-free digest of every accumulated key with its KmerAcc, n_keys)."""
        d, n = C.c_uint64(), C.c_uint64()
        check(N.lib().fbk_table_acc_digest(self._h, C.byref(d), C.byref(n)), self.ctx.handle, "accumulator digest")
        return d.value, n.value

    def digest(self) -> tuple[int, int]:
        d, n = C.c_uint64(), C.c_uint64()
        check(N.lib().fbk_table_digest(self._h, C.byref(d), C.byref(n)))
        return d.value, n.value

    def release(self):
        if self._h and self.ctx.alive:
            N.lib().fbk_table_release(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def compact(table: "SolidTable"):
    """Unitig compaction of a solid table (build.rs:330-594): returns (sequences
    list[bytes], cov f32[n], circular bool[n], edges u32[m, 6] = from unitig, from side,
    to unitig, to reverse, overlap, support)."""
    h = C.c_void_p()
    check(N.lib().fbk_compact(table.handle, C.byref(h)), table.ctx.handle, "compact")
    try:
        n, nb, ne = C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(N.lib().fbk_unitigs_info(h, C.byref(n), C.byref(nb), C.byref(ne)))
        seqs = np.zeros(max(nb.value, 1), np.uint8)
        offs = np.zeros(n.value + 1, np.uint64)
        cov = np.zeros(max(n.value, 1), np.float32)
        circ = np.zeros(max(n.value, 1), np.uint8)
        check(N.lib().fbk_unitigs_export(h, ptr(seqs), ptr(offs), cov.ctypes.data_as(C.POINTER(C.c_float)), ptr(circ)))
        edges = np.zeros((max(ne.value, 1), 6), np.uint32)
        m = C.c_uint64()
        check(N.lib().fbk_unitigs_edges(h, ptr(edges.reshape(-1)), ne.value, C.byref(m)))
    finally:
        N.lib().fbk_unitigs_release(h)
    out = [seqs[offs[i]:offs[i + 1]].tobytes() for i in range(n.value)]
    return out, cov[:n.value], circ[:n.value].astype(bool), edges[:ne.value]


def filter_active_reads(ctx: Context, bank, seqs: list, circular, edges, graph_k: int):
    """filter_active_reads (local_multik.rs:259-333) on the device: the keep byte of every
    read in bank order (merged, pe_forward, pe_reverse) and the kept count.  seqs,
    circular and edges are compact()'s unitigs."""
    dbank = bank if isinstance(bank, DeviceBank) else DeviceBank(ctx, bank)
    n = len(seqs)
    useq = np.frombuffer(b"".join(seqs), np.uint8).copy() if n else np.zeros(1, np.uint8)
    uoff = np.zeros(n + 1, np.uint64)
    if n:
        uoff[1:] = np.cumsum([len(x) for x in seqs])
    circ = np.ascontiguousarray(np.asarray(circular, np.uint8)) if n else np.zeros(1, np.uint8)
    e = np.asarray(edges).reshape(-1, 6)
    fwd = np.bincount(e[e[:, 1] == 0, 0].astype(np.int64), minlength=n)[:n].astype(np.uint32)
    rev = np.bincount(e[e[:, 1] == 1, 0].astype(np.int64), minlength=n)[:n].astype(np.uint32)
    if not n:
        fwd = rev = np.zeros(1, np.uint32)
    total = int(sum(dbank_reads for dbank_reads in _bank_reads(bank)))
    keep = np.zeros(max(total, 1), np.uint8)
    kept = C.c_uint64()
    check(N.lib().fbk_filter_active_reads(ctx.handle, dbank.handle, ptr(useq), ptr(uoff), ptr(circ), ptr(fwd), ptr(rev), n,
                                          graph_k, ptr(keep), C.byref(kept)), ctx.handle, "filter_active_reads")
    return keep[:total], kept.value


def index_terminal_kmers(ctx: Context, seqs: list, k: int, key_bits: int | None = None):
    """index_terminal_kmers (mapper.rs:89-136) on the device: unique canonical terminal
    k-mers (folded to u64) of the unitigs with (unitig, is_rc, position), sorted by key."""
    key_bits = key_bits or key_bits_for_k(k)
    n = len(seqs)
    useq = np.frombuffer(b"".join(seqs), np.uint8).copy() if n else np.zeros(1, np.uint8)
    uoff = np.zeros(n + 1, np.uint64)
    if n:
        uoff[1:] = np.cumsum([len(x) for x in seqs])
    m = C.c_uint64()
    check(N.lib().fbk_index_terminal_kmers(ctx.handle, ptr(useq), ptr(uoff), n, k, key_bits, None, None, None, None, 0,
                                           C.byref(m)), ctx.handle, "index_terminal_kmers")
    cap = m.value
    keys, uni = np.zeros(max(cap, 1), np.uint64), np.zeros(max(cap, 1), np.uint32)
    rc, pos = np.zeros(max(cap, 1), np.uint8), np.zeros(max(cap, 1), np.uint32)
    check(N.lib().fbk_index_terminal_kmers(ctx.handle, ptr(useq), ptr(uoff), n, k, key_bits, ptr(keys), ptr(uni), ptr(rc),
                                           ptr(pos), cap, C.byref(m)), ctx.handle, "index_terminal_kmers")
    return keys[:cap], uni[:cap], rc[:cap], pos[:cap]


def ingest_fastq_device(ctx: Context, r1: str, r2: str, subsample_factor: float = 1.0, min_len: int = 30, min_qual: int = 20,
                        enable_trim: bool = True, enable_merge: bool = True, seed: int = 0):
    """ingest_reads_ext_with_seed (trim_merge.rs:307-417) on the device: reads the two
    files, uploads their bytes and returns (DeviceBank, IngestStats, merged_bases)."""
    a = np.fromfile(str(r1), dtype=np.uint8)
    b = np.fromfile(str(r2), dtype=np.uint8)
    h = C.c_void_p()
    st = N.IngestStatsC()
    check(N.lib().fbk_ingest_fastq_device(ctx.handle, ptr(a) if a.size else None, a.size, ptr(b) if b.size else None, b.size,
                                          subsample_factor, min_len, min_qual, int(enable_trim), int(enable_merge), seed,
                                          C.byref(h), C.byref(st)), ctx.handle, "device ingest")
    stats = IngestStats(st.input_read_pairs, st.retained_read_pairs, st.merged_pairs_count, st.unmerged_pairs_count,
                        st.bases_before_trim, st.bases_after_trim)
    return DeviceBank.from_handle(ctx, h), stats, st.merged_bases


def _bank_reads(bank):
    if isinstance(bank, DeviceBank):
        return [bank.n_reads]
    return [len(a) for a in bank.arenas]


def select_reads(bank: "ReadBank", keep: np.ndarray) -> "ReadBank":
    """The ReadBank of the reads whose keep byte is set (packed words shared)."""
    out, pos = [], 0
    for a in bank.arenas:
        m = keep[pos:pos + len(a)].astype(bool)
        pos += len(a)
        out.append(BitSeqArena(a.data, np.ascontiguousarray(a.offsets[m]), np.ascontiguousarray(a.lengths[m]),
                               np.ascontiguousarray(a.pair_idx[m]) if a.pair_idx is not None else None))
    return ReadBank(*out)


def sort_rows(keys: np.ndarray, *cols):
    """Sorts rows by key (big-endian word order = KmerInt's Ord)."""
    if keys.shape[0] == 0:
        return (keys, *cols)
    order = np.lexsort(tuple(keys[:, j] for j in reversed(range(keys.shape[1]))))
    return (keys[order], *[c[order] for c in cols])


def _contig_buffers(contigs: list[bytes]):
    ascii = np.frombuffer(b"".join(contigs), dtype=np.uint8).copy() if contigs else np.zeros(1, np.uint8)
    offs = np.zeros(len(contigs) + 1, np.uint64)
    if contigs:
        offs[1:] = np.cumsum([len(c) for c in contigs], dtype=np.uint64)
    return ascii, offs


def build_params(k: int, target_solid_cov: int | None = None, genome_size: int | None = None, key_bits: int | None = None,
                 counter_bits: int = 4, cms_log2_width: int = 0, table_log2_cap: int = 0) -> N.BuildParams:
    p = N.BuildParams()
    p.k = k
    p.key_bits = key_bits or key_bits_for_k(k)
    p.cms_log2_width = cms_log2_width
    p.counter_bits = counter_bits
    p.t_solid = 2 if target_solid_cov is None else target_solid_cov          # build.rs:141
    p.min_trans_cov = 3 if target_solid_cov is None else target_solid_cov    # build.rs:302
    p.table_log2_cap = table_log2_cap
    p.genome_size = genome_size or 0
    return p


def build_cdbg_with_contigs_ext(bank, contigs: list[bytes], k: int, target_solid_cov: int | None = None,
                                genome_size: int | None = None, *, ctx: Context | None = None, key_bits: int | None = None,
                                counter_bits: int = 4, cms_log2_width: int = 0, subsample=None, keep_cms: bool = False):
    """Front end of build_cdbg_with_contigs_ext (build.rs:67-328): CMS pass 1, the
    CMS-gated transition pass 2 and the SolidKmerNode conversion, on the device.
    Returns the SolidTable (and the pass-1 CountMinSketch when keep_cms)."""
    ctx = ctx or default_context()
    dbank = bank if isinstance(bank, DeviceBank) else DeviceBank(ctx, bank)
    p = build_params(k, target_solid_cov, genome_size, key_bits, counter_bits, cms_log2_width)
    ascii, offs = _contig_buffers(contigs)
    t, c = C.c_void_p(), C.c_void_p()
    check(N.lib().fbk_build_front(ctx.handle, dbank.handle, C.byref(p), _subsample(subsample), ptr(ascii), ptr(offs),
                                  len(contigs), C.byref(t), C.byref(c) if keep_cms else None), ctx.handle, "build front")
    table = SolidTable(ctx, t, k, p.key_bits)
    if keep_cms:
        cms = CountMinSketch.__new__(CountMinSketch)
        cms.ctx, cms._h, cms.counter_bits = ctx, c, counter_bits
        ctx.adopt(cms)
        cms.width = 1 << p.cms_log2_width if p.cms_log2_width else None
        return table, cms
    return table


def build_cdbg(bank, k: int, target_solid_cov: int | None = None, **kw):
    return build_cdbg_with_contigs_ext(bank, [], k, target_solid_cov, None, **kw)


def build_cdbg_ext(bank, k: int, target_solid_cov: int | None = None, genome_size: int | None = None, **kw):
    return build_cdbg_with_contigs_ext(bank, [], k, target_solid_cov, genome_size, **kw)


def build_cdbg_with_contigs(bank, contigs: list[bytes], k: int, target_solid_cov: int | None = None, **kw):
    return build_cdbg_with_contigs_ext(bank, contigs, k, target_solid_cov, None, **kw)


def solid_build(ctx: Context, bank: DeviceBank, cms: CountMinSketch, k: int, target_solid_cov: int | None = None,
                key_bits: int | None = None, contigs: list[bytes] | None = None, subsample=None,
                table_log2_cap: int = 0) -> SolidTable:
    """Pass 2 + conversion against an existing pass-1 sketch."""
    p = build_params(k, target_solid_cov, None, key_bits, cms.counter_bits, 0, table_log2_cap)
    contigs = contigs or []
    ascii, offs = _contig_buffers(contigs)
    t = C.c_void_p()
    check(N.lib().fbk_solid_build(ctx.handle, bank.handle, cms._h, C.byref(p), _subsample(subsample), ptr(ascii), ptr(offs),
                                  len(contigs), C.byref(t)), ctx.handle, "solid build")
    return SolidTable(ctx, t, k, p.key_bits)


def table_from_acc_rows(ctx: Context, k: int, key_bits: int, min_trans_cov: int, rows) -> SolidTable:
    """An owner's table from the accumulated rows it received from every rank (a
    contiguous int64 CUDA tensor of (n, key_bits/64 + 2) rows, as export_acc_owned
    writes them): equal keys add up, then the SolidKmerNode conversion."""
    import torch

    rows = rows.contiguous()
    t = C.c_void_p()
    torch.cuda.synchronize()
    check(N.lib().fbk_table_from_acc_rows(ctx.handle, k, key_bits, min_trans_cov, C.c_void_p(rows.data_ptr() if len(rows) else 0),
                                          len(rows), C.byref(t)), ctx.handle, "table from rows")
    return SolidTable(ctx, t, k, key_bits)


class _CudaArray:
    """A device buffer owned by the library, described for torch.as_tensor."""

    def __init__(self, ptr_: int, shape: tuple, typestr: str):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr_, False), "version": 2,
                                         "strides": None}


def subsample_mask(ctx: Context, n_pairs: int, factor: float, seed: int) -> np.ndarray:
    out = np.zeros((n_pairs + 63) // 64, np.uint64)
    s = N.Subsample()
    s.factor, s.seed = factor, seed
    check(N.lib().fbk_subsample_mask(ctx.handle, n_pairs, C.byref(s), ptr(out)), ctx.handle, "subsample")
    return out


def nthash_arena(ctx: Context, arena: BitSeqArena, k: int) -> np.ndarray:
    total = int(np.maximum(arena.lengths.astype(np.int64) - k + 1, 0).sum())
    out = np.zeros(max(total, 1), np.uint64)
    n = C.c_uint64()
    v = arena.view()
    check(N.lib().fbk_nthash_arena(ctx.handle, C.byref(v), k, ptr(out), out.size, C.byref(n)), ctx.handle)
    return out[:n.value]


def canonical_kmers_arena(ctx: Context, arena: BitSeqArena, k: int, key_bits: int | None = None):
    kb = key_bits or key_bits_for_k(k)
    nw = kb // 64
    total = int(np.maximum(arena.lengths.astype(np.int64) - k + 1, 0).sum())
    out = np.zeros((max(total, 1), nw), np.uint64)
    rc = np.zeros(max(total, 1), np.uint8)
    n = C.c_uint64()
    v = arena.view()
    check(N.lib().fbk_canonical_kmers_arena(ctx.handle, C.byref(v), k, kb, ptr(out.reshape(-1)), ptr(rc), total,
                                            C.byref(n)), ctx.handle)
    return out[:n.value], rc[:n.value]


# ---------------------------------------------------------------------------
# subsampling policy and batches
# ---------------------------------------------------------------------------
SUBSAMPLE_REASONS = [
    "EXPLICIT_NO_SUBSAMPLE_FLAG", "EXPLICIT_GENOME_SIZE_ZERO_INVALID", "AUTO_SUBSAMPLE_EXPLICIT_GENOME_SIZE",
    "AUTO_SUBSAMPLE_EXPLICIT_GENOME_SIZE_WITHIN_TARGET", "AUTO_SUBSAMPLE_HIGH_CONFIDENCE",
    "AUTO_SUBSAMPLE_HIGH_CONFIDENCE_WITHIN_TARGET", "AUTO_SUBSAMPLE_INTERCEPTED_LOW_COVERAGE_WARNING",
    "AUTO_SUBSAMPLE_INTERCEPTED_UNRELIABLE", "GENOME_SIZE_PRIOR_PROVIDED_SUBSAMPLING_NOT_ENABLED",
    "DISABLED_BY_DEFAULT_SAFE_FALLBACK",
]


def subsample_policy(no_subsample: bool = False, enable_auto_subsample: bool = False, genome_size: int | None = None,
                     depth: float = 120.0, threshold_ratio: float = 1.5) -> N.SubsamplePolicy:
    """The pipeline driver's subsampling options (src/main.rs:76-180, cli.rs:30-72)."""
    p = N.SubsamplePolicy()
    N.lib().fbk_subsample_policy_defaults(C.byref(p))
    p.no_subsample = int(no_subsample)
    p.enable_auto_subsample = int(enable_auto_subsample)
    p.has_genome_size = int(genome_size is not None)
    p.genome_size = genome_size or 0
    p.depth = depth
    p.threshold_ratio = threshold_ratio
    return p


def subsample_decide(policy: N.SubsamplePolicy, estimate: GenomeEstimate) -> tuple[float, str]:
    """(subsample factor, reason) for an estimate, as main.rs:84-180 decides them."""
    e = estimate.to_c()
    f, r = C.c_double(), C.c_int32()
    check(N.lib().fbk_subsample_decide(C.byref(policy), C.byref(e), C.byref(f), C.byref(r)), None, "subsample_decide")
    return f.value, SUBSAMPLE_REASONS[r.value]


def batch_params(policy: N.SubsamplePolicy | None = None, **kw) -> N.BatchParams:
    p = N.BatchParams()
    N.lib().fbk_batch_defaults(C.byref(p))
    if policy is not None:
        p.policy = policy
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Batch:
    """Many isolates counted together (fbk_batch_*): per isolate the estimate, the
    subsampling decision and the build front end at one k, each phase one launch
    over every isolate of a wave."""

    def __init__(self, ctx: Context, params: N.BatchParams | None = None, **kw):
        self.ctx = ctx
        self.params = params if params is not None else batch_params(**kw)
        self.key_bits = self.params.key_bits
        self._h = C.c_void_p()
        check(N.lib().fbk_batch_create(ctx.handle, C.byref(self.params), C.byref(self._h)), ctx.handle, "batch create")
        ctx.adopt(self)

    def submit(self, bank: ReadBank, sample: BitSeqArena, sample_pairs: int, stats: ExactCountStats) -> int:
        views = bank.views()
        sv = sample.view()
        cs = stats.to_c()
        i = C.c_uint64()
        check(N.lib().fbk_batch_submit(self._h, views, C.byref(sv), sample_pairs, C.byref(cs), C.byref(i)),
              self.ctx.handle, "batch submit")
        return i.value

    def run(self) -> None:
        check(N.lib().fbk_batch_run(self._h), self.ctx.handle, "batch run")

    def result(self, i: int) -> N.BatchResult:
        r = N.BatchResult()
        check(N.lib().fbk_batch_get_result(self._h, i, C.byref(r)), self.ctx.handle, "batch result")
        return r

    def take_table(self, i: int) -> SolidTable:
        h = C.c_void_p()
        check(N.lib().fbk_batch_take_table(self._h, i, C.byref(h)), self.ctx.handle, "batch take table")
        return SolidTable(self.ctx, h, self.params.k, self.key_bits)

    def drop(self, i: int) -> None:
        check(N.lib().fbk_batch_drop(self._h, i), self.ctx.handle, "batch drop")

    def stats(self) -> N.BatchStats:
        s = N.BatchStats()
        check(N.lib().fbk_batch_get_stats(self._h, C.byref(s)), self.ctx.handle, "batch stats")
        return s

    def release(self):
        if self._h and self.ctx.alive:
            N.lib().fbk_batch_release(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


REQUEST_STATES = {0: "queued", 1: "admitted", 2: "estimated", 3: "counted", 4: "done", 5: "drained", -1: "failed"}


def server_params(policy: N.SubsamplePolicy | None = None, workers: int = 2, budget_bytes: int = 0, **batch_kw) -> N.ServerParams:
    p = N.ServerParams()
    N.lib().fbk_server_defaults(C.byref(p))
    if policy is not None:
        p.batch.policy = policy
    for k, v in batch_kw.items():
        setattr(p.batch, k, v)
    p.workers = workers
    p.budget_bytes = budget_bytes
    return p


class Server:
    """Request loop with continuous batching (fbk_server_*).  submit() queues an
    isolate and returns its id; the host arrays passed in are kept referenced until
    the request has been uploaded."""

    def __init__(self, ctx: Context, params: N.ServerParams | None = None, **kw):
        self.ctx = ctx
        self.params = params if params is not None else server_params(**kw)
        self._h = C.c_void_p()
        self._pending: dict[int, tuple] = {}
        check(N.lib().fbk_server_create(ctx.handle, C.byref(self.params), C.byref(self._h)), ctx.handle, "server create")
        ctx.adopt(self)

    def submit(self, bank: ReadBank, sample: BitSeqArena, sample_pairs: int, stats: ExactCountStats) -> int:
        views = bank.views()
        sv = sample.view()
        cs = stats.to_c()
        i = C.c_uint64()
        check(N.lib().fbk_server_submit(self._h, views, C.byref(sv), sample_pairs, C.byref(cs), C.byref(i)),
              self.ctx.handle, "server submit")
        self._pending[i.value] = (bank, sample, views, sv)   # alive until uploaded
        return i.value

    def _settle(self, i: int, info: N.RequestInfo) -> None:
        if info.state >= 2 or info.state < 0:
            self._pending.pop(i, None)

    def poll(self, i: int) -> N.RequestInfo:
        info = N.RequestInfo()
        check(N.lib().fbk_server_poll(self._h, i, C.byref(info)), self.ctx.handle, "server poll")
        self._settle(i, info)
        return info

    def wait(self, i: int, timeout_ms: float = 600_000.0) -> N.RequestInfo:
        info = N.RequestInfo()
        st = N.lib().fbk_server_wait(self._h, i, timeout_ms, C.byref(info))
        self._settle(i, info)
        check(st, self.ctx.handle, f"server wait (request {i})")
        return info

    def take_table(self, i: int) -> SolidTable:
        h = C.c_void_p()
        check(N.lib().fbk_server_take_table(self._h, i, C.byref(h)), self.ctx.handle, "server take table")
        return SolidTable(self.ctx, h, self.params.batch.k, self.params.batch.key_bits)

    def release_request(self, i: int) -> None:
        check(N.lib().fbk_server_release_request(self._h, i), self.ctx.handle, "server release request")

    def stats(self) -> N.ServerStats:
        s = N.ServerStats()
        check(N.lib().fbk_server_get_stats(self._h, C.byref(s)), self.ctx.handle, "server stats")
        return s

    def release(self):
        if self._h and self.ctx.alive:
            N.lib().fbk_server_destroy(self._h)
        self._h = C.c_void_p()
        self._pending.clear()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# synthetic isolates
# ---------------------------------------------------------------------------
def synth_params(**kw) -> N.SynthParams:
    p = N.SynthParams()
    N.synth_lib().fbk_synth_defaults(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def synth_isolate(params: N.SynthParams, threads: int = 0, min_len: int = 30, min_qual: int = 20, enable_trim: bool = True,
                  enable_merge: bool = True, sample_pairs: int = 150000):
    """Generates an isolate and ingests it (trim/merge on the host).  Returns
    (ReadBank with pair indices, IngestStats, raw estimator sample arena, n sample
    pairs, ExactCountStats)."""
    hb, hs = C.c_void_p(), C.c_void_p()
    cs = N.CountStats()
    check(N.synth_lib().fbk_synth_isolate(C.byref(params), threads, min_len, min_qual, int(enable_trim), int(enable_merge),
                                    C.byref(hb), sample_pairs, C.byref(hs) if sample_pairs else None, C.byref(cs)),
          None, "synth isolate")
    try:
        bank, st = _bank_from_hbank(hb, N.synth_lib())
        sample = None
        if sample_pairs:
            sbank, _ = _bank_from_hbank(hs, N.synth_lib())
            sample = sbank.merged_reads
    finally:
        N.synth_lib().fbk_hbank_free(hb)
        if sample_pairs:
            N.synth_lib().fbk_hbank_free(hs)
    n_sample = len(sample) // 2 if sample is not None else 0
    return bank, st, sample, n_sample, ExactCountStats.from_c(cs)


def synth_write_fastq(params: N.SynthParams, r1: str, r2: str) -> None:
    check(N.synth_lib().fbk_synth_write_fastq(C.byref(params), str(r1).encode(), str(r2).encode()), None, "synth fastq")


def synth_genome(params: N.SynthParams) -> bytes:
    g = np.zeros(params.genome_len, np.uint8)
    check(N.synth_lib().fbk_synth_genome(C.byref(params), ptr(g)))
    return g.tobytes()


def synth_pairs(params: N.SynthParams, genome: bytes, first: int, n: int):
    L = params.read_len
    bufs = [np.zeros(n * L, np.uint8) for _ in range(4)]
    g = np.frombuffer(genome, np.uint8).copy()
    check(N.synth_lib().fbk_synth_pairs(C.byref(params), ptr(g), first, n, *[ptr(b) for b in bufs]))
    return [b.reshape(n, L) for b in bufs]


# single-pair ingest helpers (their known-answer tests mirror trim_merge.rs:423-508)
def trim_adapter(seq: bytes) -> bytes:
    a = np.frombuffer(seq, np.uint8).copy()
    return seq[:N.lib().fbk_trim_adapter(ptr(a), a.size)]


def trim_quality(seq: bytes, qual: bytes, min_qual: int, min_len: int):
    a = np.frombuffer(seq, np.uint8).copy()
    q = np.frombuffer(qual, np.uint8).copy()
    n = N.lib().fbk_trim_quality(ptr(a), ptr(q), a.size, min_qual, min_len)
    return None if n < 0 else (seq[:n], qual[:n])


def merge_read_pair(r1: bytes, q1: bytes, r2: bytes, q2: bytes, min_overlap: int = 15, max_mismatch_ratio: float = 0.10):
    """Returns (merged_seq, overlap_len, mismatches) or None when unmerged."""
    a, qa = np.frombuffer(r1, np.uint8).copy(), np.frombuffer(q1, np.uint8).copy()
    b, qb = np.frombuffer(r2, np.uint8).copy(), np.frombuffer(q2, np.uint8).copy()
    out = np.zeros(len(r1) + len(r2) + 1, np.uint8)
    ov, mm = C.c_uint64(), C.c_uint64()
    n = N.lib().fbk_merge_read_pair(ptr(a), ptr(qa), a.size, ptr(b), ptr(qb), b.size, min_overlap, max_mismatch_ratio,
                                    ptr(out), C.byref(ov), C.byref(mm))
    if n < 0:
        return None
    return out[:n].tobytes(), ov.value, mm.value
