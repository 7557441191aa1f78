"""The oracle's restatement of read ingest (src/ingest/trim_merge.rs:17-238 and the
ingest loop :307-417), pinned by the reference's own trim/merge tests
(trim_merge.rs:423-508), and the library's host ingest checked against it: the single
pair helpers on many random inputs (lowercase, N, planted adapters, reads over 512
bases) and whole FASTQ files under every option the loop takes.  Results must be
identical: arena words, offsets, lengths, input pair of every read, IngestStats."""
import numpy as np
import pytest

from _ingest_cases import OPTS, odd_pairs_fastq, rand_read, rc
from fastbact_gb300 import api
from oracle import orc

M64 = (1 << 64) - 1


def splitmix_py(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


# ---- the reference's known answers, on the oracle ------------------------------------
def test_oracle_merges_230bp_fragment_with_errors():  # trim_merge.rs:424-471
    frag = bytes(b"ACGT"[splitmix_py(0x5EEDCAFE12345678 + i) % 4] for i in range(230))
    r1, q1 = bytearray(frag[:150]), bytearray(b"I" * 150)
    r1[130] = ord("C") if r1[130] == ord("A") else ord("A")
    q1[130] = ord("!")
    r2, q2 = bytearray(rc(frag[80:230])), bytearray(b"I" * 150)
    r2[129] = ord("T") if r2[129] == ord("A") else ord("A")
    q2[129] = ord("!")
    seq, ov, mm = orc.merge_read_pair(bytes(r1), bytes(q1), bytes(r2), bytes(q2), 15, 0.10)
    assert (len(seq), ov, mm) == (230, 70, 2) and seq == frag


def test_oracle_keeps_450bp_fragment_unmerged():  # trim_merge.rs:473-497
    frag = bytes(b"ACGT"[splitmix_py(0xABCDEF0123456789 + i) % 4] for i in range(450))
    assert orc.merge_read_pair(frag[:150], b"I" * 150, rc(frag[300:450]), b"I" * 150) is None


def test_oracle_trims_adapter():  # trim_merge.rs:499-507
    seq = b"ACGTACGTACGTACGT" + b"AGATCGGAAGAGCextra"
    assert orc.trim_adapter(seq) == 16


def test_oracle_quality_window():  # trim_merge.rs:79-115
    assert orc.trim_quality(b"I" * 40, 20, 30) == 40
    q = b"I" * 36 + b"####"  # a low tail: the window slides back until its mean is >= 20
    assert orc.trim_quality(q, 20, 30) == 38
    assert orc.trim_quality(b"I" * 20, 20, 30) is None  # shorter than min_len


# ---- the library's host ingest against the oracle --------------------------------------
def test_single_pair_helpers_match_oracle():
    rng = np.random.default_rng(2024)
    for it in range(600):
        n = int(rng.integers(1, 700 if it % 5 == 0 else 200))
        s = rand_read(rng, n)
        assert len(api.trim_adapter(s)) == orc.trim_adapter(s), s
        q = bytes(rng.integers(33, 75, n).astype(np.uint8))
        got = api.trim_quality(s, q, 20, 30)
        assert (None if got is None else len(got[0])) == orc.trim_quality(q, 20, 30)
    for it in range(400):
        # overlapping pairs from a random fragment, with errors, N and lowercase; reads
        # above 512 bases take the long-read complement rule
        frag_len = int(rng.integers(40, 1400 if it % 4 == 0 else 400))
        frag = rand_read(rng, frag_len)
        l1 = int(rng.integers(15, frag_len + 1))
        l2 = int(rng.integers(15, frag_len + 1))
        r1 = frag[:l1]
        r2 = rc(frag[frag_len - l2:].upper().replace(b"N", b"A"))
        r2 = bytes(c if rng.random() > 0.02 else ord("N") for c in r2)
        q1 = bytes(rng.integers(33, 75, l1).astype(np.uint8))
        q2 = bytes(rng.integers(33, 75, l2).astype(np.uint8))
        assert api.merge_read_pair(r1, q1, r2, q2, 15, 0.10) == orc.merge_read_pair(r1, q1, r2, q2, 15, 0.10)


def compare_ingest(r1, r2, **kw):
    o_arenas, o_stats = orc.ingest_fastq(r1, r2, **kw)
    bank, st = api.ingest_reads_ext_with_seed(r1, r2, kw.get("subsample_factor", 1.0), kw.get("min_len", 30),
                                              kw.get("min_qual", 20), kw.get("enable_trim", True),
                                              kw.get("enable_merge", True), kw.get("seed", 0))
    for a, (d, o, L, pi) in zip(bank.arenas, o_arenas):
        assert np.array_equal(a.lengths, L) and np.array_equal(a.offsets, o)
        assert np.array_equal(a.data[: d.size], d) and not a.data[d.size:].any()
        assert np.array_equal(a.pair_idx, pi)
    for f in ("input_read_pairs", "retained_read_pairs", "bases_before_trim", "bases_after_trim", "merged_pairs_count",
              "unmerged_pairs_count"):
        assert getattr(st, f) == o_stats[f], f
    assert bank.merged_reads.total_bases() == o_stats["merged_bases"]
    return o_stats


@pytest.mark.parametrize("opts", OPTS)
def test_host_ingest_matches_oracle(tmp_path, opts):
    p = api.synth_params(seed=303, genome_len=30_000, coverage=20.0, gc=0.45, sub_rate=0.01)
    r1, r2 = tmp_path / "s_1.fq", tmp_path / "s_2.fq"
    api.synth_write_fastq(p, r1, r2)
    st = compare_ingest(r1, r2, **opts)
    if not opts:
        assert st["merged_pairs_count"] > 0 and st["unmerged_pairs_count"] > 0


def test_host_ingest_matches_oracle_on_odd_reads(tmp_path):
    """Lowercase, N, planted adapters, short reads and pairs over 512 bases."""
    r1, r2 = tmp_path / "o_1.fq", tmp_path / "o_2.fq"
    odd_pairs_fastq(r1, r2, 77, 300)
    for opts in OPTS:
        compare_ingest(r1, r2, **opts)


def test_oracle_ingest_errors(tmp_path):
    r1, r2 = tmp_path / "e_1.fq", tmp_path / "e_2.fq"
    r1.write_text("@a/1\nACGTACGTACGT\n+\nIIIIIIIIIIII\n@b/1\nACGT\n+\nIIII\n")
    r2.write_text("@a/2\nACGTACGTACGT\n+\nIIIIIIIIIIII\n")
    with pytest.raises(RuntimeError, match="Mismatched paired-end FASTQ mate counts"):
        orc.ingest_fastq(r1, r2)
    r1.write_text("@a/1\nACGT\n+\nIIII\n")
    r2.write_text("@a/2\nACGT\n+\nIIII\n")
    with pytest.raises(RuntimeError, match="No valid reads survived trimming"):
        orc.ingest_fastq(r1, r2)
