"""Parity of the device kernels (through the C ABI) with the oracle on the same
seeded inputs.  Integer results must be bit-identical; the estimator's f64 outputs
too (same operation order, same libm on the same host).  Tolerance: exact (0)."""
import ctypes as C

import numpy as np
import pytest

from fastbact_gb300 import api
from oracle import orc

pytestmark = pytest.mark.gpu
M64 = (1 << 64) - 1


def splitmix_py(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def rand_seqs(seed, n, lo, hi, alphabet=b"ACGT"):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.integers(lo, hi + 1))
        out.append(bytes(np.frombuffer(alphabet, np.uint8)[rng.integers(0, len(alphabet), L)]))
    return out


def oracle_rolling(seq: bytes, k: int, kb: int):
    nw = kb // 64
    n = len(seq) - k + 1
    if n <= 0:
        return np.zeros((0, nw), np.uint64), np.zeros(0, np.uint8)
    out = np.zeros(n * nw, np.uint64)
    rc = np.zeros(n, np.uint8)
    a = np.frombuffer(seq, np.uint8).copy()
    assert orc.lib().orc_rolling_canonicals(kb, orc.p(a), len(seq), k, orc.p(out), orc.p(rc)) == n
    return out.reshape(n, nw), rc


@pytest.fixture(scope="module")
def small_isolate():
    p = api.synth_params(seed=101, genome_len=60_000, coverage=30.0, gc=0.5)
    return api.synth_isolate(p, threads=0, sample_pairs=150_000)


@pytest.fixture(scope="module")
def repeat_isolate():
    # repeats + tandem array + indels + 1% errors: stresses the saturating counters
    p = api.synth_params(seed=202, genome_len=50_000, coverage=60.0, gc=0.66, n_repeats=4, repeat_len=2000,
                         tandem_copies=60, tandem_unit=60, sub_rate=0.01, indel_rate=0.0005)
    return api.synth_isolate(p, threads=0, sample_pairs=150_000)


# ---------------------------------------------------------------------------
# k-mer extraction and ntHash
# ---------------------------------------------------------------------------
KS = [(1, 64), (5, 64), (21, 64), (31, 64), (21, 128), (33, 128), (55, 128), (63, 128), (31, 256), (45, 256),
      (65, 256), (77, 256), (96, 256), (97, 256), (99, 256), (127, 256)]


@pytest.mark.parametrize("k,kb", KS)
def test_canonical_kmers_match_rolling(ctx, k, kb):
    seqs = rand_seqs(k * 7 + kb, 60, 1, 400) + [b"A" * 200, b"ACGT" * 60, b"T" * (k + 1), b"G" * k]
    arena = api.BitSeqArena.from_seqs(seqs)
    got, got_rc = api.canonical_kmers_arena(ctx, arena, k, kb)
    exp = [oracle_rolling(s, k, kb) for s in seqs]
    exp_k = np.concatenate([e[0] for e in exp])
    exp_rc = np.concatenate([e[1] for e in exp])
    assert got.shape == exp_k.shape
    assert np.array_equal(got, exp_k)
    assert np.array_equal(got_rc, exp_rc)


@pytest.mark.parametrize("k", [1, 15, 21, 31, 64, 65, 127])
def test_nthash_matches_rolling(ctx, k):
    seqs = rand_seqs(k, 80, 1, 300) + [b"N" * 50 + b"ACGT" * 20]
    # N maps to A in the hash (ASCII_TO_2BIT); the packed arena stores it as A too
    arena = api.BitSeqArena.from_seqs(seqs)
    got = api.nthash_arena(ctx, arena, k)
    exp = []
    for s in seqs:
        if len(s) < k:
            continue
        o = np.zeros(len(s) - k + 1, np.uint64)
        a = np.frombuffer(s, np.uint8).copy()
        orc.lib().orc_nthash_rolling_all(orc.p(a), len(s), k, orc.p(o))
        exp.append(o)
    assert np.array_equal(got, np.concatenate(exp))


# ---------------------------------------------------------------------------
# sketches
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("cb", [4, 16])
def test_cms_keys_and_saturation(ctx, cb):
    rng = np.random.default_rng(cb)
    keys = rng.integers(0, 1 << 63, 20000, dtype=np.uint64)
    hot = np.repeat(keys[:40], 40)  # counters beyond 15
    allk = np.concatenate([keys, hot])
    cms = api.CountMinSketch(1 << 12, ctx, counter_bits=cb)
    cms.add(allk)
    ref = orc.Cms(1 << 12, cb)
    ref.add(allk)
    assert np.array_equal(cms.export(), ref.export())
    est = cms.estimate(keys[:3000])
    assert [int(x) for x in est] == [ref.estimate(int(x)) for x in keys[:3000]]
    c2 = api.CountMinSketch(1024, ctx, counter_bits=cb)  # sketch.rs:305-319
    assert int(c2.estimate([42])[0]) == 0
    c2.add([42] * 5)
    assert int(c2.estimate([42])[0]) == 5
    c2.add([42] * 20)
    assert int(c2.estimate([42])[0]) == (15 if cb == 4 else 25)


@pytest.mark.parametrize("cb", [4, 16])
def test_cms_merge_equals_union(ctx, cb):
    rng = np.random.default_rng(5)
    a = rng.integers(0, 1 << 20, 30000, dtype=np.uint64)
    b = rng.integers(0, 1 << 20, 30000, dtype=np.uint64)
    ca, cbm, cu = (api.CountMinSketch(1 << 10, ctx, cb) for _ in range(3))
    ca.add(a)
    cbm.add(b)
    cu.add(np.concatenate([a, b]))
    ca.merge(cbm)
    assert np.array_equal(ca.export(), cu.export())


@pytest.mark.parametrize("p", [14, 16])
def test_hll_registers_and_estimate(ctx, p):
    n = 300_000
    xs = np.array([splitmix_py(i) for i in range(n)], np.uint64)
    h = api.HyperLogLog(p, ctx)
    h.add_hash(xs)
    r = orc.Hll(p)
    r.add_hash(xs)
    assert np.array_equal(h.registers(), r.registers())
    assert h.estimate() == r.estimate()
    h2, r2 = api.HyperLogLog(p, ctx), orc.Hll(p)
    h2.add_canonical_hash(xs[:1000])
    r2.add_canonical_hash(xs[:1000])
    h.merge(h2)
    r.merge(r2)
    assert np.array_equal(h.registers(), r.registers())


# ---------------------------------------------------------------------------
# build front end
# ---------------------------------------------------------------------------
def row_view(keys: np.ndarray) -> np.ndarray:
    keys = np.ascontiguousarray(keys)
    return keys.view(np.dtype((np.void, keys.shape[1] * 8))).ravel()


def assert_acc_matches(table, o_tab, mtc):
    """The accumulated keys (KmerAcc rows) equal the oracle's; for a table built with
    the record filter they are a subset of the oracle's rows, identical where present,
    that holds every key with an edge count >= min_trans_cov."""
    gk, gc, ge = table.export_acc(sort=True)
    ok, oc, oe = api.sort_rows(*o_tab.export_acc())
    if not table.filtered():
        assert gk.shape == ok.shape, (gk.shape, ok.shape)
        assert np.array_equal(gk, ok) and np.array_equal(gc, oc) and np.array_equal(ge, oe)
        return
    gv, ov = row_view(gk), row_view(ok)
    common, gi, oi = np.intersect1d(gv, ov, return_indices=True)
    assert len(common) == len(gv), "a kept key is not an accumulated key of the oracle"
    assert np.array_equal(gc[gi], oc[oi]) and np.array_equal(ge[gi], oe[oi])
    need = (oe.astype(np.int64) >= mtc).any(axis=1)
    assert np.isin(ov[need], gv).all(), "a key with an edge count >= min_trans_cov was filtered out"


def compare_build(ctx, bank, k, kb, cb, tsc, log2w, contigs=None, subsample=None, keep_mask=None):
    dbank = api.DeviceBank(ctx, bank)
    table, cms = api.build_cdbg_with_contigs_ext(dbank, contigs or [], k, tsc, None, ctx=ctx, key_bits=kb,
                                                 counter_bits=cb, cms_log2_width=log2w, subsample=subsample,
                                                 keep_cms=True)
    o_cms, o_tab, t_solid, mtc = orc.build_front(bank, k, kb, log2w, cb, tsc, threads=4, keep_mask=keep_mask,
                                                 contigs=contigs)
    assert np.array_equal(cms.export(), o_cms.export()), "pass-1 CMS bytes differ"
    assert_acc_matches(table, o_tab, mtc)
    sk, sc, sm = table.export(sort=True)
    xk, xc, xm = api.sort_rows(*o_tab.export_solid(mtc))
    assert np.array_equal(sk, xk) and np.array_equal(sc, xc) and np.array_equal(sm, xm)
    assert table.digest() == o_tab.digest(mtc)
    return table, len(sk)


def compare_gate_only(ctx, bank, k, kb, cb, tsc, log2w, subsample=None, keep_mask=None):
    """A build that does not return its sketch (pass 1 keeps only the gate, as a
    threshold ladder when 1 <= t_solid <= 8) against the oracle's full build."""
    table = api.build_cdbg_with_contigs_ext(bank, [], k, tsc, None, ctx=ctx, key_bits=kb, counter_bits=cb,
                                            cms_log2_width=log2w, subsample=subsample)
    _, o_tab, _, mtc = orc.build_front(bank, k, kb, log2w, cb, tsc, threads=4, keep_mask=keep_mask)
    assert_acc_matches(table, o_tab, mtc)
    sk, sc, sm = table.export(sort=True)
    xk, xc, xm = api.sort_rows(*o_tab.export_solid(mtc))
    assert np.array_equal(sk, xk) and np.array_equal(sc, xc) and np.array_equal(sm, xm)
    assert table.digest() == o_tab.digest(mtc)
    return len(sk)


@pytest.mark.parametrize("k,kb", [(21, 64), (31, 64), (33, 128), (55, 128), (77, 256), (127, 256)])
@pytest.mark.parametrize("cb", [4, 16])
def test_gate_only_build_matches_oracle(ctx, small_isolate, k, kb, cb):
    assert compare_gate_only(ctx, small_isolate[0], k, kb, cb, None, 16) > 1000


@pytest.mark.parametrize("tsc", [None, 1, 3, 5, 8, 9, 15])
def test_gate_only_thresholds_and_saturation(ctx, repeat_isolate, tsc):
    # t <= 8: ladder levels; 9 and 15: the exact sketch; 2^12 columns: heavy collisions
    for cb in (4, 16):
        for log2w in (12, 16):
            compare_gate_only(ctx, repeat_isolate[0], 31, 64, cb, tsc, log2w)
    compare_gate_only(ctx, repeat_isolate[0], 45, 128, 16, tsc, 14)
    compare_gate_only(ctx, repeat_isolate[0], 99, 256, 4, tsc, 14)


def test_gate_only_with_subsampling(ctx, repeat_isolate):
    bank = repeat_isolate[0]
    n_pairs = int(max(int(a.pair_idx.max()) for a in bank.arenas if len(a))) + 1
    keep = api.subsample_mask(ctx, n_pairs, 0.35, 1234)
    compare_gate_only(ctx, bank, 31, 64, 16, None, 16, subsample=(0.35, 1234), keep_mask=keep)


@pytest.mark.parametrize("lookahead", [1, 2, 3, 4])
def test_emit_variants_with_subsampling_and_256_bit_keys(repeat_isolate, lookahead):
    """Every record-emit form (gate one or two chunks ahead, read by read or over the
    flattened window stream) with skipped reads and keys of every width, including
    256-bit keys whose slot tag lives in the key (k <= 96) or apart (k > 96)."""
    bank = repeat_isolate[0]
    c = api.Context(0)
    try:
        c.set_tuning(emit_lookahead=lookahead)
        n_pairs = int(max(int(a.pair_idx.max()) for a in bank.arenas if len(a))) + 1
        keep = api.subsample_mask(c, n_pairs, 0.5, 77)
        for k, kb in [(21, 64), (33, 128), (77, 256), (101, 256)]:
            compare_gate_only(c, bank, k, kb, 16, None, 14, subsample=(0.5, 77), keep_mask=keep)
        compare_gate_only(c, bank, 77, 256, 16, None, 16)
    finally:
        c.close()


@pytest.mark.parametrize("k,kb", [(21, 64), (45, 128), (77, 256), (101, 256)])
def test_record_filter_keeps_the_solid_rows(repeat_isolate, k, kb):
    """With the record filter (default) the table holds fewer keys, and the
    SolidKmerNode rows, digest and push count equal the unfiltered build's."""
    bank = repeat_isolate[0]
    c = api.Context(0)
    try:
        out = {}
        for f in (2, 0):
            c.set_tuning(acc_filter=f)
            for tsc in (None, 2, 5):
                t = api.build_cdbg_with_contigs_ext(bank, [], k, tsc, None, ctx=c, key_bits=kb, counter_bits=16,
                                                    cms_log2_width=14)
                out[f, tsc] = (t.filtered(), t.info()[0], t.export(sort=True), t.digest(), t.pushes())
                t.release()
        for tsc in (None, 2, 5):
            on, off = out[2, tsc], out[0, tsc]
            assert on[0] and not off[0]
            assert on[1] < off[1]
            assert all(np.array_equal(a, b) for a, b in zip(on[2], off[2]))
            assert on[3] == off[3] and on[4] == off[4]
        # min_trans_cov = 1 cannot filter anything; the default filters 256-bit keys only
        c.set_tuning(acc_filter=2)
        t = api.build_cdbg_with_contigs_ext(bank, [], k, 1, None, ctx=c, key_bits=kb, counter_bits=16, cms_log2_width=14)
        assert not t.filtered()
        t.release()
        c.set_tuning(acc_filter=1)
        t = api.build_cdbg_with_contigs_ext(bank, [], k, None, None, ctx=c, key_bits=kb, counter_bits=16,
                                            cms_log2_width=14)
        if kb == 256:
            assert t.filtered()
        assert t.digest() == out[0, None][3]
        t.release()
    finally:
        c.close()


def test_sketch_mode_off_matches(repeat_isolate):
    c = api.Context(0)
    try:
        c.set_tuning(sketch_mode=0)
        assert c.get_tuning("sketch_mode") == 0
        compare_gate_only(c, repeat_isolate[0], 31, 64, 16, None, 14)
    finally:
        c.close()


@pytest.mark.parametrize("k,kb", [(21, 64), (31, 64), (33, 128), (55, 128), (77, 256), (127, 256)])
@pytest.mark.parametrize("cb", [4, 16])
def test_build_front_matches_oracle(ctx, small_isolate, k, kb, cb):
    bank = small_isolate[0]
    _, n_solid = compare_build(ctx, bank, k, kb, cb, None, 16)
    assert n_solid > 1000


@pytest.mark.parametrize("tsc", [None, 1, 5, 15, 20])
def test_build_thresholds(ctx, repeat_isolate, tsc):
    # tsc = 20 is above the nibble cap: the reference's capped estimate never reaches it
    compare_build(ctx, repeat_isolate[0], 31, 64, 4, tsc, 14)
    compare_build(ctx, repeat_isolate[0], 31, 64, 16, tsc, 14)


def test_build_saturation_and_repeats(ctx, repeat_isolate):
    # small CMS (many collisions, saturated nibbles) + repeat-rich bank, both widths
    for k, kb in [(21, 64), (45, 128), (99, 256)]:
        compare_build(ctx, repeat_isolate[0], k, kb, 4, None, 10)
        compare_build(ctx, repeat_isolate[0], k, kb, 16, None, 10)


def test_build_with_subsampling(ctx, repeat_isolate):
    bank = repeat_isolate[0]
    n_pairs = int(max(int(a.pair_idx.max()) for a in bank.arenas if len(a))) + 1
    keep = api.subsample_mask(ctx, n_pairs, 0.35, 1234)
    thr = int(0.35 * 2.0 ** 64)
    exp = np.zeros_like(keep)
    for q in range(n_pairs):
        if splitmix_py((q + 1) ^ 1234) <= thr:
            exp[q >> 6] |= np.uint64(1 << (q & 63))
    assert np.array_equal(keep, exp)
    compare_build(ctx, bank, 31, 64, 4, None, 16, subsample=(0.35, 1234), keep_mask=keep)


def test_build_with_prior_contigs(ctx, small_isolate):
    bank = small_isolate[0]
    contigs = rand_seqs(9, 30, 20, 3000) + [b"ACGT" * 100]
    compare_build(ctx, bank, 31, 64, 4, None, 16, contigs=contigs)
    compare_build(ctx, bank, 33, 128, 16, 4, 16, contigs=contigs)
    compare_build(ctx, bank, 79, 256, 4, 4, 16, contigs=contigs)


def test_build_edge_cases(ctx):
    k = 31
    seqs = [b"", b"A", b"ACGT" * 7, b"C" * 31, b"G" * 32, b"T" * 1000, b"ACGTTGCA" * 600] + rand_seqs(3, 50, 1, 70)
    bank = api.ReadBank(api.BitSeqArena.from_seqs(seqs[:4]), api.BitSeqArena.from_seqs(seqs[4:30]),
                        api.BitSeqArena.from_seqs(seqs[30:]))
    compare_build(ctx, bank, k, 64, 4, None, 12)
    compare_build(ctx, bank, k, 64, 4, 1, 12)
    compare_build(ctx, bank, 127, 256, 16, 1, 12)
    empty = api.ReadBank()
    t = api.build_cdbg_ext(empty, 31, None, 100000, ctx=ctx)
    assert t.info()[:2] == (0, 0)


EDGE_SEQS = [b"", b"A", b"ACGT" * 7, b"C" * 31, b"G" * 32, b"T" * 1000, b"ACGTTGCA" * 600] + rand_seqs(3, 50, 1, 70)


@pytest.mark.parametrize("k,kb", [(1, 64), (5, 64), (21, 64), (28, 64), (29, 64), (31, 64), (33, 128), (55, 128), (60, 128),
                                  (61, 128), (63, 128), (65, 256), (77, 256), (92, 256), (93, 256), (96, 256), (97, 256),
                                  (124, 256), (125, 256), (127, 256)])
@pytest.mark.parametrize("rolled", [0, 1, 2])
def test_gate_only_every_record_layout(repeat_isolate, k, kb, rolled):
    """Every pass-2 record layout (records of ceil((2k + 8) / 64) words, the info byte
    packed into the key's free top bits or in a word of its own: the boundaries are
    k = 28/29, 60/61, 92/93, 124/125), with the per-window kernels and with the rolled
    one-lane-per-read kernels (pass 1 rolling one or two windows per step); an
    edge-case bank whose runs include reads too long to stage (the global-memory path),
    empty and shorter-than-k reads, and reads of odd and even window counts."""
    c = api.Context(0)
    try:
        if rolled:
            c.set_tuning(ladder_ilp=4 if rolled == 1 else 5, emit_lookahead=4)
        compare_gate_only(c, repeat_isolate[0], k, kb, 16, None, 14)
        edge = api.ReadBank(api.BitSeqArena.from_seqs(EDGE_SEQS[:4]), api.BitSeqArena.from_seqs(EDGE_SEQS[4:30]),
                            api.BitSeqArena.from_seqs(EDGE_SEQS[30:]))
        compare_gate_only(c, edge, k, kb, 4, 1, 12)
    finally:
        c.close()


def test_build_rc_bank_invariance(ctx, small_isolate):
    """Size-independent property: the bank of reverse-complemented reads yields the
    same CMS and the same solid table."""
    bank = small_isolate[0]
    seqs = [bank.pe_forward.extract_ascii(i) for i in range(min(3000, len(bank.pe_forward)))]
    rcs = [s[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA")) for s in seqs]
    b1 = api.ReadBank(pe_forward=api.BitSeqArena.from_seqs(seqs))
    b2 = api.ReadBank(pe_forward=api.BitSeqArena.from_seqs(rcs))
    t1, c1 = api.build_cdbg_ext(b1, 31, None, None, ctx=ctx, cms_log2_width=16, keep_cms=True)
    t2, c2 = api.build_cdbg_ext(b2, 31, None, None, ctx=ctx, cms_log2_width=16, keep_cms=True)
    assert np.array_equal(c1.export(), c2.export())
    assert t1.digest() == t2.digest()


# ---------------------------------------------------------------------------
# estimator
# ---------------------------------------------------------------------------
def sample_reads(sample: api.BitSeqArena, n_pairs: int):
    return [sample.extract_ascii(i) for i in range(2 * n_pairs)]


@pytest.mark.parametrize("max_pairs", [3000, 6000, 9000, 250000])
def test_estimator_matches_oracle(ctx, small_isolate, max_pairs):
    bank, st, sample, n_sample, cs = small_isolate
    reads = sample_reads(sample, n_sample)
    ost = orc.count_stats(**cs.__dict__)
    rc, oe, ort, ors = orc.estimate_from_reads(reads, ost, max_pairs, 110.0)
    assert rc == 0
    ge, rt, rs = api.estimate_sample(ctx, sample, n_sample, cs, max_pairs=max_pairs, target_cov=110.0)
    assert np.array_equal(rt, ort) and np.array_equal(rs, ors)
    for f in ("genome_size", "exact_read_pairs", "total_bases", "median_read_len", "max_read_len", "estimated_cov",
              "subsample_factor", "u_ge_1", "u_ge_2", "sample_kmer_depth", "pairs_sampled", "m_sample"):
        assert getattr(ge, f) == getattr(oe, f), f
    assert ge.kmers == [oe.kmers[i] for i in range(oe.n_kmers)]
    assert {"HIGH": 0, "LOW_COVERAGE_WARNING": 1, "UNRELIABLE": 2}[ge.confidence] == oe.confidence


def test_estimator_early_stop_and_p16(ctx, repeat_isolate):
    bank, st, sample, n_sample, cs = repeat_isolate
    reads = sample_reads(sample, n_sample)
    ost = orc.count_stats(**cs.__dict__)
    for p in (14, 16):
        rc, oe, ort, ors = orc.estimate_from_reads(reads, ost, 250000, 0.0, hll_p=p)
        ge, rt, rs = api.estimate_sample(ctx, sample, n_sample, cs, max_pairs=250000, hll_p=p)
        assert np.array_equal(rt, ort) and np.array_equal(rs, ors)
        assert (ge.genome_size, ge.u_ge_1, ge.u_ge_2, ge.pairs_sampled) == (oe.genome_size, oe.u_ge_1, oe.u_ge_2,
                                                                            oe.pairs_sampled)
        assert ge.sample_kmer_depth == oe.sample_kmer_depth


def test_estimate_genome_from_fastq(ctx, tmp_path):
    p = api.synth_params(seed=303, genome_len=80_000, coverage=40.0)
    r1, r2 = tmp_path / "e_1.fq", tmp_path / "e_2.fq"
    api.synth_write_fastq(p, r1, r2)
    ge = api.estimate_genome(r1, r2, 250000, 30.0, ctx=ctx)
    oe = orc.OrcEstimate()
    err = C.create_string_buffer(256)
    assert orc.lib().orc_estimate_genome(str(r1).encode(), str(r2).encode(), 250000, 30.0, C.byref(oe), None, None, err,
                                         256) == 0
    assert (ge.genome_size, ge.u_ge_1, ge.u_ge_2, ge.estimated_cov, ge.subsample_factor) == \
           (oe.genome_size, oe.u_ge_1, oe.u_ge_2, oe.estimated_cov, oe.subsample_factor)
    assert ge.confidence in ("HIGH", "LOW_COVERAGE_WARNING", "UNRELIABLE")
    assert 0.7 * 80_000 < ge.genome_size < 1.3 * 80_000


def test_estimator_reads_with_n_and_short(ctx):
    seqs = []
    for i in range(7000):
        a, b = rand_seqs(i, 2, 10, 150, alphabet=b"ACGTN")
        seqs += [a, b]
    arena = api.BitSeqArena.from_seqs(seqs)
    stats = api.ExactCountStats(7000, 1, 1, sum(map(len, seqs)), 10, 150, sum(map(len, seqs)) / 14000, 80)
    ge, rt, rs = api.estimate_sample(ctx, arena, 7000, stats, max_pairs=250000)
    rc, oe, ort, ors = orc.estimate_from_reads([s.replace(b"N", b"A") for s in seqs], orc.count_stats(**stats.__dict__),
                                               250000, 0.0)
    assert np.array_equal(rt, ort) and np.array_equal(rs, ors)
    assert (ge.genome_size, ge.u_ge_2, ge.pairs_sampled) == (oe.genome_size, oe.u_ge_2, oe.pairs_sampled)


@pytest.mark.parametrize("world,max_pairs,hll_p", [(1, 250000, 14), (3, 250000, 14), (4, 9000, 16), (2, 5000, 14)])
def test_sharded_estimator_stages_on_device(ctx, repeat_isolate, world, max_pairs, hll_p):
    """The device stages of the sharded estimator, run per pair range and merged (MIN,
    then MAX) as the ranks' all-reduces would, give the one-process device estimate
    and the oracle's sequential sample loop."""
    from fastbact_gb300 import shard

    bank, st, sample, n_sample, cs = repeat_isolate
    params = dict(max_pairs=max_pairs, hll_p=hll_p, target_cov=110.0)
    lengths = np.ascontiguousarray(sample.lengths[:2 * n_sample])
    eng = shard.DeviceEstimatorEngine(ctx, sample, lengths, **params)
    try:
        n_use, n_segs = api.est_shard_plan(lengths, n_sample, cs, **params)
        ranges = [shard.pair_range(n_use, r, world) for r in range(world)]
        first = np.minimum.reduce([eng.firstpos(n_use, lo, hi) for lo, hi in ranges])
        regs = np.maximum.reduce([eng.segments(n_use, lo, hi, first) for lo, hi in ranges])
        ge, rt, rs = api.est_shard_finish(lengths, n_use, cs, regs, **params)
        one, ort1, ors1 = api.estimate_bank(ctx, eng.bank, lengths, n_sample, cs, want_registers=True, **params)
    finally:
        eng.release()
    assert ge == one
    assert np.array_equal(rt, ort1) and np.array_equal(rs, ors1)
    rc, oe, ort, ors = orc.estimate_from_reads(sample_reads(sample, n_sample), orc.count_stats(**cs.__dict__), max_pairs,
                                               110.0, hll_p=hll_p)
    assert (ge.genome_size, ge.u_ge_1, ge.u_ge_2, ge.pairs_sampled, ge.m_sample) == \
        (oe.genome_size, oe.u_ge_1, oe.u_ge_2, oe.pairs_sampled, oe.m_sample)
    assert np.array_equal(rt, ort) and np.array_equal(rs, ors)


# ---------------------------------------------------------------------------
# launch / sizing variants must not change any result
# ---------------------------------------------------------------------------
TUNINGS = [
    dict(pass2_mode=0),                                   # direct sweep
    dict(sweep_bytes=1 << 20, bucket_bytes=1 << 20),      # many column slices, 64 buckets
    dict(sweep_bytes=1 << 31, bucket_bytes=1 << 30),      # one sweep over all rows, one bucket
    dict(stripes=1, record_factor=0.05),                  # stripes overflow -> direct fallback
    dict(load_factor=0.85, block_pass1=128, block_pass2=64, grid_pass1=37, grid_pass2=91),
    dict(ladder_ilp=2, block_pass1=128),                 # two windows per lane in the ladder pass 1
    dict(ladder_ilp=3),                                   # ladder pass 1 pipelined over chunks
    dict(emit_lookahead=1),                               # gate loads one chunk ahead of the emit
    dict(emit_lookahead=2),                               # emit read by read, gate loads two chunks ahead
    dict(emit_lookahead=3),                               # emit over the flattened window stream
    dict(emit_lookahead=5),                               # rolled emit at two blocks per SM for every width
    dict(ladder_ilp=4, emit_lookahead=4),                 # one lane per read, k-mers rolled, runs staged in smem
    dict(ladder_ilp=5),                                   # the same pass 1 rolling two windows per step
    dict(acc_filter=0),                                   # every accumulated key kept
    dict(acc_filter=2),                                   # keys that cannot be solid dropped at every width
    dict(acc_filter=2, block_pass2=96),                   # the filter's survivors queued per warp, 3 warps per block
    dict(acc_filter=2, upsert_queue=2),                   # the same at six blocks per SM
    dict(acc_filter=2, upsert_queue=0),                   # the filter tested inline
    dict(filter_sizing=0, load_factor=0.9, acc_filter=2),  # long probe runs in the queued upsert
    dict(upsert_all=1, acc_filter=0),                     # persistent upsert, probes run to the end lane by lane
    dict(upsert_all=2, acc_filter=0, load_factor=0.9),    # ... with long probe runs
    dict(filter_sizing=0, acc_filter=2),                  # filtered tables sized from the distinct k-mers
    dict(filter_sizing=1, filter_load=0.62, acc_filter=2),  # ... from the first bucket's survivors at a high load
    dict(filter_sizing=1, filter_load=0.9, acc_filter=2, bucket_bytes=1 << 16),  # ... from a small first bucket
    dict(upsert_all=0, acc_filter=0),                     # one upsert launch per bucket
    dict(block_emit=256),                                 # record emit in blocks of 256
]


@pytest.mark.parametrize("tune", TUNINGS)
def test_build_tuning_variants(repeat_isolate, tune):
    c = api.Context(0)
    try:
        c.set_tuning(**tune)
        for k, kb, cb in [(31, 64, 4), (45, 128, 16), (99, 256, 4)]:
            compare_build(c, repeat_isolate[0], k, kb, cb, None, 14)
            compare_gate_only(c, repeat_isolate[0], k, kb, cb, None, 14)
    finally:
        c.close()


# ---------------------------------------------------------------------------
# unitig compaction (build.rs:330-594)
# ---------------------------------------------------------------------------
def _canon_cycle(s: bytes) -> bytes:
    """Rotation- and strand-independent form of a circular sequence."""
    rc = s[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA"))
    return min(min(x[i:] + x[:i] for i in range(len(x))) for x in (s, rc))


def _cov_choices(seq: bytes, rows: dict, k: int, kb: int):
    """Both coverages a linear unitig can get (walked from either end): mean node
    coverage of its k-mers without the last one of the walk."""
    nw = kb // 64
    covs = []
    for i in range(len(seq) - k + 1):
        w = seq[i:i + k]
        key = np.zeros(nw, np.uint64)
        assert orc.lib().orc_kmer_from_ascii(kb, orc.p(np.frombuffer(w, np.uint8).copy()), k, orc.p(key)) == 0
        rk = np.zeros(nw, np.uint64)
        orc.lib().orc_kmer_rev_comp(kb, orc.p(key), k, orc.p(rk))
        can = min(tuple(int(x) for x in key), tuple(int(x) for x in rk))
        covs.append(rows.get(can, 0))
    a = np.float32(max(1.0, np.float32(sum(covs[:-1])) / np.float32(len(covs) - 1))) if len(covs) > 1 else None
    b = np.float32(max(1.0, np.float32(sum(covs[1:])) / np.float32(len(covs) - 1))) if len(covs) > 1 else None
    return {a, b}


def compare_compaction(ctx, bank, k, kb, cb, tsc, log2w):
    table = api.build_cdbg_with_contigs_ext(bank, [], k, tsc, None, ctx=ctx, key_bits=kb, counter_bits=cb,
                                            cms_log2_width=log2w)
    keys, cov, mask = table.export()
    gseq, gcov, gcirc, gedges = api.compact(table)
    oseq, ocov, ocirc, oedges = orc.compact(keys, cov, mask, k, kb)
    # linear unitigs: the same canonical sequences; circular ones up to rotation
    assert sorted(s for s, c in zip(gseq, gcirc) if not c) == sorted(s for s, c in zip(oseq, ocirc) if not c)
    assert sorted(_canon_cycle(s) for s, c in zip(gseq, gcirc) if c) == sorted(_canon_cycle(s) for s, c in zip(oseq, ocirc) if c)
    # coverage: one of the two ends' values, as the reference's map order picks one
    rows = {tuple(int(x) for x in kk): int(c) for kk, c in zip(keys.reshape(len(cov), -1), cov)}
    for s, c, circ in zip(gseq, gcov, gcirc):
        if not circ:
            assert np.float32(c) in _cov_choices(s, rows, k, kb), s[:40]
    # edges between linear unitigs: same (from seq, side, to seq, strand, overlap, support) multiset
    def edge_set(seqs, circ, edges):
        out = []
        for f, side, t, trc, ov, sup in edges:
            if circ[f] or circ[t]:
                continue
            out.append((seqs[f], int(side), seqs[t], int(trc), int(ov), int(sup)))
        return sorted(out)
    assert edge_set(gseq, gcirc, gedges) == edge_set(oseq, ocirc, oedges)
    return gseq, gcirc


@pytest.mark.parametrize("k,kb", [(21, 64), (31, 64), (45, 128), (77, 256)])
def test_compaction_matches_oracle(ctx, repeat_isolate, k, kb):
    seqs, circ = compare_compaction(ctx, repeat_isolate[0], k, kb, 16, None, 16)
    assert len(seqs) > 10


def test_compaction_three_unitig_gate(ctx):
    # build.rs:604-687: 10 kb circular genome with a 200 bp repeat, 1% errors, solidity 5
    from test_compact_oracle import gate_reads, gate_width
    reads = gate_reads()
    bank = api.ReadBank(merged_reads=api.BitSeqArena.from_seqs(reads))
    log2w = gate_width(sum(map(len, reads))).bit_length() - 1
    table = api.build_cdbg(bank, 31, 5, ctx=ctx, key_bits=64, counter_bits=4, cms_log2_width=log2w)
    seqs, cov, circ, edges = api.compact(table)
    assert len(seqs) == 3 and not circ.any()
    compare_compaction(ctx, bank, 31, 64, 4, 5, log2w)


def test_compaction_circular_plasmid(ctx):
    # an error-free circular sequence with no repeat compacts to one circular unitig
    rng = np.random.default_rng(5)
    plasmid = bytes(np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 3000)])
    ring = plasmid + plasmid[:200]
    reads = [ring[i:i + 150] for i in range(0, 3000, 7)] * 8
    bank = api.ReadBank(merged_reads=api.BitSeqArena.from_seqs(reads))
    seqs, circ = compare_compaction(ctx, bank, 31, 64, 16, None, 16)
    assert list(circ) == [True] and len(seqs[0]) == 3000
    assert _canon_cycle(seqs[0]) == _canon_cycle(plasmid)


# ---------------------------------------------------------------------------
# multi-k input filter (local_multik.rs:259-333)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("k,graph_k", [(31, 31), (45, 45), (21, 21)])
def test_filter_active_reads_matches_oracle(ctx, repeat_isolate, k, graph_k):
    bank = repeat_isolate[0]
    kb = api.key_bits_for_k(k)
    table = api.build_cdbg_ext(bank, k, None, ctx=ctx, key_bits=kb, counter_bits=16, cms_log2_width=16)
    seqs, cov, circ, edges = api.compact(table)
    keep, kept = api.filter_active_reads(ctx, bank, seqs, circ, edges, graph_k)
    okeep = orc.filter_active_reads(bank, seqs, circ, edges, graph_k)
    assert np.array_equal(keep, okeep)
    assert kept == int(okeep.sum()) and 0 < kept <= len(keep)
    if k == 31:
        # long unitigs exist, so only reads near their ends and junctions stay
        assert any(len(s) >= 2000 for s in seqs) and kept < len(keep)
    sub = api.select_reads(bank, keep)
    assert sub.total_reads() == kept


# ---------------------------------------------------------------------------
# PE mapper terminal k-mer index (mapper.rs:89-136)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("k,kb", [(31, 64), (45, 128), (77, 256)])
def test_terminal_kmer_index_matches_oracle(ctx, repeat_isolate, k, kb):
    table = api.build_cdbg_ext(repeat_isolate[0], k, None, ctx=ctx, key_bits=kb, counter_bits=16, cms_log2_width=16)
    seqs, cov, circ, edges = api.compact(table)
    got = api.index_terminal_kmers(ctx, seqs, k, kb)
    exp = orc.index_terminal_kmers(seqs, k, kb)
    for a, b in zip(got, exp):
        assert np.array_equal(a, b)
    assert len(got[0]) > 1000
    # a repeat k-mer shared by two unitig ends is not unique and is dropped
    total = sum(min(len(s) - k + 1, 2000) for s in seqs if len(s) >= k)
    assert len(got[0]) <= total


# ---------------------------------------------------------------------------
# ingest on the device (trim_merge.rs:307-417) equals the oracle's restatement
# ---------------------------------------------------------------------------
def _oracle_bank_concat(arenas):
    """The device bank layout of the oracle's three arenas: words back to back, offsets
    rebased by the preceding arenas' words."""
    words, offs, lens, pidx, wbase = [], [], [], [], 0
    for d, o, L, pi in arenas:
        words.append(d)
        offs.append(o.astype(np.uint64) + np.uint64(wbase * 32))
        lens.append(L)
        pidx.append(pi)
        wbase += len(d)
    return np.concatenate(words), np.concatenate(offs), np.concatenate(lens), np.concatenate(pidx)


def _check_device_ingest(ctx, r1, r2, kw):
    o_arenas, o_st = orc.ingest_fastq(r1, r2, **kw)
    dbank, dst, merged_bases = api.ingest_fastq_device(ctx, r1, r2, **kw)
    for f in ("input_read_pairs", "retained_read_pairs", "bases_before_trim", "bases_after_trim", "merged_pairs_count",
              "unmerged_pairs_count"):
        assert getattr(dst, f) == o_st[f], f
    assert merged_bases == o_st["merged_bases"]
    words, offs, lens, pidx, counts = dbank.export()
    ow, oo, ol, op = _oracle_bank_concat(o_arenas)
    assert counts == [len(a[2]) for a in o_arenas]
    assert np.array_equal(lens, ol) and np.array_equal(offs, oo) and np.array_equal(pidx, op)
    assert np.array_equal(words[: ow.size], ow) and not words[ow.size:].any()
    return dbank, o_st


@pytest.mark.parametrize("opts", [dict(), dict(subsample_factor=0.4, seed=11), dict(enable_merge=False),
                                  dict(enable_trim=False, min_len=100), dict(min_qual=35, min_len=60)])
def test_device_ingest_matches_oracle(ctx, tmp_path, opts):
    p = api.synth_params(seed=303, genome_len=30_000, coverage=20.0, gc=0.45, sub_rate=0.01)
    r1, r2 = tmp_path / "d_1.fq", tmp_path / "d_2.fq"
    api.synth_write_fastq(p, r1, r2)
    kw = dict(subsample_factor=1.0, min_len=30, min_qual=20, enable_trim=True, enable_merge=True, seed=0)
    kw.update(opts)
    dbank, o_st = _check_device_ingest(ctx, r1, r2, kw)
    if not opts:
        assert o_st["merged_pairs_count"] > 0  # the default settings merge overlapping pairs
    # the device bank counts like the uploaded host bank
    hbank, _ = api.ingest_reads_ext_with_seed(r1, r2, kw["subsample_factor"], kw["min_len"], kw["min_qual"], kw["enable_trim"],
                                              kw["enable_merge"], kw["seed"])
    t1 = api.build_cdbg_ext(dbank, 31, None, ctx=ctx, key_bits=64, counter_bits=16, cms_log2_width=16)
    t2 = api.build_cdbg_ext(hbank, 31, None, ctx=ctx, key_bits=64, counter_bits=16, cms_log2_width=16)
    assert t1.digest() == t2.digest()


def test_device_ingest_matches_oracle_on_odd_reads(ctx, tmp_path):
    """Lowercase, N, planted adapters, short reads and pairs over 512 bases (whose
    reverse complement turns a non-ACGT base into 'T', not 'A')."""
    from _ingest_cases import OPTS, odd_pairs_fastq

    r1, r2 = tmp_path / "o_1.fq", tmp_path / "o_2.fq"
    odd_pairs_fastq(r1, r2, 78, 400)
    for opts in OPTS:
        kw = dict(subsample_factor=1.0, min_len=30, min_qual=20, enable_trim=True, enable_merge=True, seed=0)
        kw.update(opts)
        _check_device_ingest(ctx, r1, r2, kw)


def test_device_ingest_rejects_bad_records(ctx, tmp_path):
    r1, r2 = tmp_path / "b_1.fq", tmp_path / "b_2.fq"
    r1.write_text("@a/1\nACGT\n+\nIIII\n@b/1\nACGT\n+\nIII\n")
    r2.write_text("@a/2\nACGT\n+\nIIII\n@b/2\nACGT\n+\nIIII\n")
    with pytest.raises(Exception):
        api.ingest_fastq_device(ctx, r1, r2)
    r1.write_text("@a/1\nACGT\n+\nIIII\n")
    with pytest.raises(Exception):
        api.ingest_fastq_device(ctx, r1, r2)


def test_bank_upload_checks_every_sequence(ctx):
    """The upload scans all reads (in blocks, on several threads): a bad sequence in
    any block is refused, and the bank's totals match the host arenas."""
    from fastbact_gb300 import _native as N

    rng = np.random.default_rng(8)
    n = 300_000  # several scan blocks
    lengths = rng.integers(0, 300, n).astype(np.uint32)
    offsets = np.zeros(n, np.uint64)
    offsets[1:] = np.cumsum(lengths[:-1], dtype=np.uint64)
    words = rng.integers(0, 2**63, (int(lengths.sum()) + 31) // 32 + 1, dtype=np.uint64)
    good = api.BitSeqArena(words, offsets, lengths)
    db = api.DeviceBank(ctx, good)
    assert (db.n_reads, db.n_bases) == (n, int(lengths.sum()))
    db.release()
    for bad_at in (0, 70_000, n - 1):  # first, middle and last scan block
        offs = offsets.copy()
        lens = lengths.copy()
        lens[bad_at] = 100
        offs[bad_at] = len(words) * 32 - 50
        with pytest.raises(N.FbkError, match="extends past"):
            api.DeviceBank(ctx, api.BitSeqArena(words, offs, lens))


@pytest.mark.parametrize("k,kb,cb", [(31, 64, 4), (45, 128, 16), (77, 256, 4)])
def test_cms_build_one_call(ctx, small_isolate, k, kb, cb):
    """fbk_cms_build (create + pass 1) gives the oracle's pass-1 sketch bytes."""
    bank = small_isolate[0]
    db = api.DeviceBank(ctx, bank)
    cms = api.CountMinSketch.build(ctx, db, k, 14, cb, key_bits=kb)
    assert np.array_equal(cms.export(), orc.build_front(bank, k, kb, 14, cb, None, threads=4)[0].export())
    cms.release()
    db.release()


@pytest.mark.parametrize("cb,log2w", [(16, 22), (4, 24)])
def test_large_sketch_export_import_round_trip(ctx, small_isolate, cb, log2w):
    """Sketches of 32 MB go through the pinned staging slots both ways (several
    16 MB chunks); the bytes equal the oracle's pass-1 sketch."""
    bank = small_isolate[0]
    t, cms = api.build_cdbg_ext(bank, 31, None, ctx=ctx, key_bits=64, counter_bits=cb, cms_log2_width=log2w,
                                keep_cms=True)
    t.release()
    raw = cms.export()
    assert raw.nbytes == 32 << 20
    o_cms = orc.build_front(bank, 31, 64, log2w, cb, None, threads=4)[0]
    assert np.array_equal(raw, o_cms.export())
    other = api.CountMinSketch(1 << log2w, ctx, counter_bits=cb)
    other.load(raw)
    assert np.array_equal(other.export(), raw)
    # a page-locked destination takes the direct path and gives the same bytes
    import torch

    from fastbact_gb300 import _native as N

    pinned = torch.empty(raw.nbytes, dtype=torch.uint8, pin_memory=True).numpy()
    assert N.lib().fbk_cms_export(other._h, N.ptr(pinned), raw.nbytes) == 0
    assert np.array_equal(pinned, raw)


def test_u16_sketch_saturates_like_the_reference(ctx):
    # 2^10 columns and ~80 M k-mer occurrences: most u16 counters pass 65535 and must
    # stop there (sketch.rs:199-221), in the exported sketch and in the gate
    p = api.synth_params(seed=404, genome_len=400_000, coverage=220.0, gc=0.66, n_repeats=3, repeat_len=3000,
                         tandem_copies=50, tandem_unit=60, sub_rate=0.01, indel_rate=0.0005)
    bank = api.synth_isolate(p, threads=0, sample_pairs=0)[0]
    table, n_solid = compare_build(ctx, bank, 31, 64, 16, None, 10)
    cms = api.build_cdbg_ext(bank, 31, None, ctx=ctx, key_bits=64, counter_bits=16, cms_log2_width=10, keep_cms=True)[1]
    vals = cms.export().view(np.uint16)
    assert (vals == 65535).mean() > 0.5
    compare_gate_only(ctx, bank, 127, 256, 16, None, 10)
