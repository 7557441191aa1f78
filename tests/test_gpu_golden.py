"""The device kernels reproduce the committed golden fixtures (exact)."""
import numpy as np
import pytest

from _golden import GOLDEN, mg
from fastbact_gb300 import api

pytestmark = pytest.mark.gpu


def test_golden_nthash_and_canonical(ctx):
    seqs = mg.golden_sequences()
    arena = api.BitSeqArena.from_seqs(seqs)
    h21 = api.nthash_arena(ctx, arena, 21)
    assert [int(x) for x in h21[:40]] == GOLDEN["nthash_k21"]
    assert mg.sha(h21) == GOLDEN["nthash_k21_sha256"]
    assert mg.sha(api.nthash_arena(ctx, arena, 15)) == GOLDEN["nthash_k15_sha256"]
    for k, kb in [(21, 64), (31, 64), (55, 128), (99, 256), (127, 256)]:
        ks, rcs = api.canonical_kmers_arena(ctx, arena, k, kb)
        assert mg.sha(ks) == GOLDEN[f"canon_k{k}_sha256"]
        assert mg.sha(rcs) == GOLDEN[f"canon_k{k}_rc_sha256"]


def test_golden_sketches(ctx):
    M64 = (1 << 64) - 1
    keys = np.array([(i * 0x9E3779B97F4A7C15) & M64 for i in range(20000)], np.uint64)
    keys = np.concatenate([keys, np.repeat(keys[:64], 24)])
    for cb in (4, 16):
        c = api.CountMinSketch(1 << 12, ctx, counter_bits=cb)
        c.add(keys)
        assert mg.sha(c.export()) == GOLDEN[f"cms_{cb}_sha256"]
    h = api.HyperLogLog(14, ctx)
    h.add_canonical_hash(keys)
    assert mg.sha(h.registers()) == GOLDEN["hll14_registers_sha256"]
    assert h.estimate() == GOLDEN["hll14_estimate"]


def test_golden_isolate_estimate_and_builds(ctx):
    bank, st, sample, n_sample, stats = mg.isolate()
    assert [mg.sha(a.data) for a in bank.arenas] == GOLDEN["isolate"]["data_sha256"]
    e, rt, rs = api.estimate_sample(ctx, sample, n_sample, stats, max_pairs=250_000, target_cov=110.0)
    ge = GOLDEN["estimate"]
    conf = {"HIGH": 0, "LOW_COVERAGE_WARNING": 1, "UNRELIABLE": 2}[e.confidence]
    assert (e.genome_size, e.u_ge_1, e.u_ge_2, e.estimated_cov, e.subsample_factor, e.sample_kmer_depth, conf,
            e.pairs_sampled, e.m_sample) == (ge["genome_size"], ge["u_ge_1"], ge["u_ge_2"], ge["estimated_cov"],
                                            ge["subsample_factor"], ge["sample_kmer_depth"], ge["confidence"],
                                            ge["pairs_sampled"], ge["m_sample"])
    assert mg.sha(rt) == ge["regs_total_sha256"] and mg.sha(rs) == ge["regs_solid_sha256"]
    prev = ctx.get_tuning("acc_filter")
    try:
        for name, exp in GOLDEN["builds"].items():
            k, kb, cb, tsc = name.split("_")
            k, kb, cb = int(k[1:]), int(kb[1:]), int(cb[1:])
            tsc = None if tsc == "tNone" else int(tsc[1:])
            # every accumulated key (the fixtures hash the whole accumulator) ...
            ctx.set_tuning(acc_filter=0)
            t, cms = api.build_cdbg_with_contigs_ext(bank, [], k, tsc, None, ctx=ctx, key_bits=kb, counter_bits=cb,
                                                     cms_log2_width=15, keep_cms=True)
            assert mg.sha(cms.export()) == exp["cms_sha256"], name
            keys, cov, edges = t.export_acc(sort=True)
            assert (int(keys.shape[0]), mg.sha(keys), mg.sha(cov), mg.sha(edges)) == \
                   (exp["n_keys"], exp["acc_keys_sha256"], exp["acc_cov_sha256"], exp["acc_edges_sha256"]), name
            assert t.digest() == (exp["digest"], exp["n_solid"]), name
            t.release()
            # ... and a build with the record filter at every key width: same rows
            ctx.set_tuning(acc_filter=2)
            t = api.build_cdbg_with_contigs_ext(bank, [], k, tsc, None, ctx=ctx, key_bits=kb, counter_bits=cb,
                                                cms_log2_width=15)
            assert t.digest() == (exp["digest"], exp["n_solid"]), name
            t.release()
    finally:
        ctx.set_tuning(acc_filter=prev)
