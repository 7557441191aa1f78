"""The oracle and the host-side generator reproduce the committed golden fixtures."""
import numpy as np
import pytest

from _golden import GOLDEN, mg
from oracle import orc


def test_golden_vectors_oracle():
    seqs = mg.golden_sequences()
    assert [s.decode() for s in seqs] == GOLDEN["sequences"]
    assert [int(x) for x in mg.nthash_vectors(seqs, 21)[:40]] == GOLDEN["nthash_k21"]
    assert mg.sha(mg.nthash_vectors(seqs, 21)) == GOLDEN["nthash_k21_sha256"]
    assert mg.sha(mg.nthash_vectors(seqs, 15)) == GOLDEN["nthash_k15_sha256"]
    for k, kb in [(21, 64), (31, 64), (55, 128), (99, 256), (127, 256)]:
        ks, rcs = mg.canon_vectors(seqs, k, kb)
        assert mg.sha(ks) == GOLDEN[f"canon_k{k}_sha256"]
        assert mg.sha(rcs) == GOLDEN[f"canon_k{k}_rc_sha256"]


def test_golden_sketches_oracle():
    M64 = (1 << 64) - 1
    keys = np.array([(i * 0x9E3779B97F4A7C15) & M64 for i in range(20000)], np.uint64)
    keys = np.concatenate([keys, np.repeat(keys[:64], 24)])
    for cb in (4, 16):
        c = orc.Cms(1 << 12, cb)
        c.add(keys)
        assert mg.sha(c.export()) == GOLDEN[f"cms_{cb}_sha256"]
    h = orc.Hll(14)
    h.add_canonical_hash(keys)
    assert mg.sha(h.registers()) == GOLDEN["hll14_registers_sha256"]
    assert h.estimate() == GOLDEN["hll14_estimate"]


@pytest.fixture(scope="module")
def isolate():
    return mg.isolate()


def test_golden_isolate_generator(isolate):
    bank, st, sample, n_sample, stats = isolate
    gi = GOLDEN["isolate"]
    assert (bank.total_reads(), bank.total_bases(), n_sample) == (gi["reads"], gi["bases"], gi["n_sample"])
    assert [mg.sha(a.data) for a in bank.arenas] == gi["data_sha256"]
    assert [mg.sha(a.lengths) for a in bank.arenas] == gi["lengths_sha256"]
    assert mg.sha(sample.data) == gi["sample_sha256"]


def test_golden_estimate_and_builds_oracle(isolate):
    bank, st, sample, n_sample, stats = isolate
    reads = [sample.extract_ascii(i) for i in range(2 * n_sample)]
    rc, oe, rt, rs = orc.estimate_from_reads(reads, orc.count_stats(**stats.__dict__), 250_000, 110.0)
    ge = GOLDEN["estimate"]
    assert rc == 0
    for f in ("genome_size", "u_ge_1", "u_ge_2", "estimated_cov", "subsample_factor", "sample_kmer_depth", "confidence",
              "pairs_sampled", "m_sample"):
        assert getattr(oe, f) == ge[f], f
    assert mg.sha(rt) == ge["regs_total_sha256"] and mg.sha(rs) == ge["regs_solid_sha256"]
    from fastbact_gb300.api import sort_rows

    for name, exp in GOLDEN["builds"].items():
        k, kb, cb, tsc = name.split("_")
        k, kb, cb = int(k[1:]), int(kb[1:]), int(cb[1:])
        tsc = None if tsc == "tNone" else int(tsc[1:])
        cms, tab, ts, mtc = orc.build_front(bank, k, kb, 15, cb, tsc, threads=2)
        assert mg.sha(cms.export()) == exp["cms_sha256"], name
        keys, cov, edges = sort_rows(*tab.export_acc())
        assert (int(keys.shape[0]), mg.sha(keys), mg.sha(cov), mg.sha(edges)) == \
               (exp["n_keys"], exp["acc_keys_sha256"], exp["acc_cov_sha256"], exp["acc_edges_sha256"]), name
        assert tab.digest(mtc) == (exp["digest"], exp["n_solid"]), name
