"""Pins the oracle (CPU restatement) against every known-answer and statistical test
the reference's own test modules hold for the hot path, plus published SplitMix64
vectors.  No GPU needed."""
import ctypes as C

import numpy as np
import pytest

from oracle import orc

L = orc.lib()
M64 = (1 << 64) - 1


def lcg_bases(seed, n):
    """The tests' LCG (bitseq.rs:479-484, kmer.rs:629-633) over ACGT."""
    out, s = [], seed
    for _ in range(n):
        s = (s * 6364136223846793005 + 1442695040888963407) & M64
        out.append(b"ACGT"[s % 4])
    return bytes(out)


def splitmix_py(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def buf(b: bytes):
    a = np.frombuffer(b, np.uint8).copy()
    return a, orc.p(a)


def test_splitmix64_published_vectors():
    # SplitMix64 generator (state += 0x9e3779b97f4a7c15) from seed 0: published outputs.
    expect = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F, 0xF88BB8A8724C81EC, 0x1B39896A51A8749B]
    s = 0
    for e in expect:
        s = (s + 0x9E3779B97F4A7C15) & M64
        assert L.orc_splitmix64(s) == e
    for z in [0, 1, 42, M64, 0x123456789ABCDEF]:
        assert L.orc_splitmix64(z) == splitmix_py(z)


def test_rev_comp_word_kat():  # bitseq.rs:433-446
    assert L.orc_rev_comp_word(0b00_01_10, 3) == 0b01_10_11
    assert L.orc_rev_comp_word(0b00_01_10_11, 4) == 0b00_01_10_11
    assert L.orc_rev_comp_word(0x123, 0) == 0


def rc_ascii(s: bytes) -> bytes:
    return s[::-1].translate(bytes.maketrans(b"ACGTacgt", b"TGCAtgca"))


@pytest.mark.parametrize("kb,seq", [(64, b"ACGTACGTACGTACGTACGTACGT"),
                                    (128, b"ACGT" * 14),
                                    (256, b"ACGT" * 24)])
def test_kmer_basic_roundtrip_and_rc(kb, seq):  # kmer.rs:543-577
    nw = kb // 64
    k = len(seq)
    a, pa = buf(seq)
    w = np.zeros(4, np.uint64)
    L.orc_kmer_from_ascii(kb, pa, k, orc.p(w))
    # MSB-first: decode the words back to ASCII
    bits = 0
    for i in range(nw):
        bits = (bits << 64) | int(w[i])
    dec = bytes(b"ACGT"[(bits >> (2 * (k - 1 - i))) & 3] for i in range(k))
    assert dec == seq
    rcw = np.zeros(4, np.uint64)
    L.orc_kmer_rev_comp(kb, orc.p(w), k, orc.p(rcw))
    r, pr = buf(rc_ascii(seq))
    w2 = np.zeros(4, np.uint64)
    L.orc_kmer_from_ascii(kb, pr, k, orc.p(w2))
    assert (rcw[:nw] == w2[:nw]).all()


@pytest.mark.parametrize("k,kb", [(21, 64), (55, 128), (99, 256), (127, 256)])
def test_rolling_canonical_gate(k, kb):  # kmer.rs:580-651
    seq = lcg_bases(0xCAFEBABEDEADBEEF, 300)
    nw = kb // 64
    n = 300 - k + 1
    f = np.zeros(n * nw, np.uint64)
    r = np.zeros(n * nw, np.uint64)
    a, pa = buf(seq)
    b, pb = buf(rc_ascii(seq))
    assert L.orc_rolling_canonicals(kb, pa, 300, k, orc.p(f), None) == n
    assert L.orc_rolling_canonicals(kb, pb, 300, k, orc.p(r), None) == n
    assert (f.reshape(n, nw) == r.reshape(n, nw)[::-1]).all()


def test_nthash_rolling_matches_fresh():  # kmer.rs:654-664
    seq = b"ACGTACGTACGTTTGCAACCGGTTACGT"
    k = 15
    n = len(seq) - k + 1
    out = np.zeros(n, np.uint64)
    a, pa = buf(seq)
    assert L.orc_nthash_rolling_all(pa, len(seq), k, orc.p(out)) == n
    for i in range(n):
        w, pw = buf(seq[i:i + k])
        assert int(out[i]) == L.orc_nthash_canonical(pw, k)


def test_nthash_single_base_is_seed():
    # a 1-base window hashes to the seed itself (kmer.rs:385-404)
    seeds = {b"A": 0x3C8BFBB395C60474, b"C": 0x3193C18562A02B4C, b"G": 0x20323EE046061444, b"T": 0x295C504FAC61002E}
    for base, v in seeds.items():
        a, pa = buf(base)
        assert L.orc_nthash_fwd(pa, 1) == v
    a, pa = buf(b"N")
    assert L.orc_nthash_fwd(pa, 1) == seeds[b"A"]  # non-ACGT maps to A


def test_hll_cardinality_gate():  # sketch.rs:262-284
    h = orc.Hll(14)
    h.add_hash(np.array([splitmix_py(i) for i in range(100_000)], np.uint64))
    assert abs(h.estimate() - 100_000) / 100_000 < 0.03


def test_hll_merge():  # sketch.rs:287-302
    a, b = orc.Hll(14), orc.Hll(14)
    a.add_hash(np.array([splitmix_py(i) for i in range(50_000)], np.uint64))
    b.add_hash(np.array([splitmix_py(i) for i in range(50_000, 100_000)], np.uint64))
    a.merge(b)
    assert abs(a.estimate() - 100_000) / 100_000 < 0.03


def _raw_min(s1, s2, n):
    i = np.arange(n, dtype=np.uint64)
    f = np.array([splitmix_py(s1 ^ int(x)) for x in i], np.uint64)
    r = np.array([splitmix_py(s2 ^ int(x)) for x in i], np.uint64)
    return np.minimum(f, r)


def test_hll_raw_min_skew_vs_splitmix():  # sketch.rs:345-382
    n = 200_000
    raw = _raw_min(0x123456789ABCDEF0, 0xFEDCBA9876543210, n)
    a, b = orc.Hll(14), orc.Hll(14)
    a.add_hash(raw)
    b.add_canonical_hash(raw)
    assert (a.estimate() - n) / n < -0.50
    assert abs(b.estimate() - n) / n <= 0.025


@pytest.mark.parametrize("n", [50_000, 200_000, 1_000_000])
def test_hll_multi_scale(n):  # sketch.rs:385-407 (2.5M scale in the slow suite)
    raw = _raw_min(0xABCDEF0123456789, 0x9876543210FEDCBA, n)
    h = orc.Hll(14)
    h.add_canonical_hash(raw)
    assert abs(h.estimate() - n) / n <= 0.025


def test_cms_basic_saturation():  # sketch.rs:305-319
    c = orc.Cms(1024, 4)
    assert c.estimate(42) == 0
    c.add([42] * 5)
    assert c.estimate(42) == 5
    c.add([42] * 20)
    assert c.estimate(42) == 15


def test_cms_repeated_adds():  # sketch.rs:322-342 (4 threads x 3 adds == 12)
    c = orc.Cms(4096, 4)
    c.add([12345] * 12)
    assert c.estimate(12345) == 12


def test_cms_u16_relation():
    # nibble estimate == min(15, u16 estimate) for every key
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 1 << 63, 5000, dtype=np.uint64)
    keys = np.concatenate([keys, np.repeat(keys[:50], 30)])
    a, b = orc.Cms(1 << 10, 4), orc.Cms(1 << 10, 16)
    a.add(keys)
    b.add(keys)
    for key in keys[:500]:
        assert a.estimate(int(key)) == min(15, b.estimate(int(key)))


def test_cms_width_for_genome_size():  # sketch.rs:165-168
    assert L.orc_cms_width_for_genome_size(1) == 1 << 21
    assert L.orc_cms_width_for_genome_size(1_000_000) == 1 << 24
    assert L.orc_cms_width_for_genome_size(5_000_000) == 1 << 27
    assert L.orc_cms_width_for_genome_size(100_000_000) == 1 << 27


def kmers(median, target=None):
    out = (C.c_uint64 * 16)()
    n = L.orc_compute_dynamic_kmers(median, -1 if target is None else target, out, 16)
    return [out[i] for i in range(n)]


def test_compute_dynamic_kmers():  # estimator.rs:529-546
    k = kmers(150)
    assert k[0] == 31 and k[-1] == 127 and all(x % 2 == 1 and 31 <= x <= 127 for x in k)
    k = kmers(50)
    assert k[0] == 21 and all(x % 2 == 1 for x in k)


def test_subsample_keep_rule():  # trim_merge.rs:324-348
    assert L.orc_subsample_keep(5, 1.0, 0) == 1
    assert L.orc_subsample_keep(5, 0.9995, 7) == 1  # factor >= 0.999 keeps everything
    thr = int(0.3 * 2.0 ** 64)
    for i in range(1, 2000):
        assert L.orc_subsample_keep(i, 0.3, 99) == (1 if splitmix_py(i ^ 99) <= thr else 0)


def write_fastq(path, recs):
    with open(path, "w") as f:
        for name, seq, qual in recs:
            f.write(f"@{name}\n{seq}\n+\n{qual}\n")


def test_count_fastx_exact_oracle_kats(tmp_path):  # estimator.rs:463-526
    r1, r2 = tmp_path / "a_1.fq", tmp_path / "a_2.fq"
    write_fastq(r1, [(f"pair_{i}/1", "ACGTACGTACGT", "I" * 12) for i in range(1, 11)])
    write_fastq(r2, [(f"pair_{i}/2", "TGCATGCATGCA", "I" * 12) for i in range(1, 11)])
    s = orc.OrcCountStats()
    err = C.create_string_buffer(512)
    assert L.orc_count_fastx_exact(str(r1).encode(), str(r2).encode(), C.byref(s), err, 512) == 0
    assert (s.exact_read_pairs, s.total_bases_r1, s.total_bases_r2, s.total_bases) == (10, 120, 120, 240)
    assert (s.min_read_len, s.max_read_len, s.median_read_len) == (12, 12, 12)
    assert abs(s.mean_read_len - 12.0) < 1e-6
    write_fastq(r1, [(f"pair_{i}/1", "ACGT", "IIII") for i in range(1, 6)])
    write_fastq(r2, [(f"pair_{i}/2", "ACGT", "IIII") for i in range(1, 5)])
    assert L.orc_count_fastx_exact(str(r1).encode(), str(r2).encode(), C.byref(s), err, 512) != 0
    assert b"R1 has more reads than R2" in err.value
    write_fastq(r1, [("pair_A/1", "ACGT", "IIII")])
    write_fastq(r2, [("pair_B/2", "ACGT", "IIII")])
    assert L.orc_count_fastx_exact(str(r1).encode(), str(r2).encode(), C.byref(s), err, 512) != 0
    assert b"synchronization error" in err.value
