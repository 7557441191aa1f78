"""Bit-exact parity at the full sizes of the named workloads: the device path through
the C ABI against the oracle on the same seeded inputs.

* plain 1 Mbp (GC 0.50, 50x, k = 31, CMS 4 x 2^22 u16, HLL p = 14);
* isolate scale, the benchmark's own workload (5 Mbp, 100x, k = 21/33/55/77, CMS
  4 x 2^24 u16) — the same builds the benchmark times;
* stress (12 Mbp GC 0.66, repeats and a tandem array, 300x with indels, k = 127,
  CMS 4 x 2^26 u16, HLL p = 16), on the full input and subsampled to 110x by the
  pipeline driver's policy.

Compared, exactly (tolerance 0): every GenomeEstimate field and both HLL register
arrays (estimator.rs:286-440); the sorted SolidKmerNode rows and their digest
(build.rs:295-328) of the default build (the one the benchmark times, with its
threshold-ladder gate and, where it applies, its record filter); the whole KmerAcc
accumulator of a build without the record filter (build.rs:141-289), through the
order-free accumulator digest (tens of millions of keys; both sides compute the same
sum) and the key count; and the counted sketch's bytes where the workload keeps it.
"""
import numpy as np
import pytest

from fastbact_gb300 import api, workloads
from oracle import orc

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def ascii_reads(arena: api.BitSeqArena, n: int) -> list[bytes]:
    """The first n reads of an arena as ASCII (vectorised decode)."""
    if n == 0:
        return []
    end = int(arena.offsets[n - 1]) + int(arena.lengths[n - 1])
    g = np.arange(end, dtype=np.uint64)
    codes = (arena.data[g >> np.uint64(5)] >> ((g & np.uint64(31)) << np.uint64(1))) & np.uint64(3)
    s = np.frombuffer(b"ACGT", np.uint8)[codes.astype(np.intp)].tobytes()
    return [s[int(o):int(o) + int(L)] for o, L in zip(arena.offsets[:n], arena.lengths[:n])]


def keep_bits(n_pairs: int, factor: float, seed: int) -> np.ndarray:
    """The subsampler's keep rule (trim_merge.rs:324-348) for pairs 1..n_pairs, as a
    little-endian bitmap over 0-based pairs; spot-checked against the oracle's own
    keep test."""
    i = np.arange(1, n_pairs + 1, dtype=np.uint64)
    z = i ^ np.uint64(seed)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    keep = np.ones(n_pairs, bool) if factor >= 0.999 else z <= np.uint64(int(factor * 2.0 ** 64))
    for j in range(0, n_pairs, max(1, n_pairs // 997)):
        assert bool(keep[j]) == bool(orc.lib().orc_subsample_keep(j + 1, factor, seed))
    b = np.packbits(keep, bitorder="little")
    b = np.concatenate([b, np.zeros((-b.size) % 8, np.uint8)])
    return b.view(np.uint64)


EST_FIELDS = ("genome_size", "exact_read_pairs", "total_bases", "median_read_len", "max_read_len", "estimated_cov",
              "subsample_factor", "kmers", "n_kmers", "confidence", "u_ge_1", "u_ge_2", "sample_kmer_depth",
              "pairs_sampled", "m_sample")


def check_estimator(ctx, sample, n_sample, stats, hll_p):
    ge, rt, rs = api.estimate_sample(ctx, sample, n_sample, stats, max_pairs=workloads.EST_MAX_PAIRS,
                                     target_cov=workloads.EST_TARGET_COV, hll_p=hll_p)
    reads = ascii_reads(sample, 2 * n_sample)
    rc, oe, ort, ors = orc.estimate_from_reads(reads, orc.count_stats(**stats.__dict__), workloads.EST_MAX_PAIRS,
                                               workloads.EST_TARGET_COV, hll_p=hll_p)
    assert rc == 0
    gc = ge.to_c()
    for f in EST_FIELDS:
        g, o = getattr(gc, f), getattr(oe, f)
        if f == "kmers":
            g, o = list(g), list(o)
        assert g == o, (f, g, o)
    assert np.array_equal(rt, ort), "total HyperLogLog registers differ"
    assert np.array_equal(rs, ors), "solid HyperLogLog registers differ"
    return ge


def oracle_build(bank, k, log2w, keep_mask=None):
    """The oracle's full build at k (u16 counters, t_solid 2, min_trans_cov 3)."""
    kb = api.key_bits_for_k(k)
    o_cms, o_tab, _, mtc = orc.build_front(bank, k, kb, log2w, 16, None, threads=0, keep_mask=keep_mask)
    rows = api.sort_rows(*o_tab.export_solid(mtc))
    out = dict(rows=rows, digest=o_tab.digest(mtc), acc=o_tab.acc_digest(), cms=o_cms)
    del o_tab
    return out


def check_rows(table, ref):
    sk, sc, sm = table.export(sort=True)
    xk, xc, xm = ref["rows"]
    assert sk.shape == xk.shape, (sk.shape, xk.shape)
    assert np.array_equal(sk, xk) and np.array_equal(sc, xc) and np.array_equal(sm, xm)
    assert table.digest() == ref["digest"]


def device_builds(ctx, dbank, k, log2w, ref, subsample=None, keep_cms=False):
    """Default build (rows), then a build without the record filter (the whole
    accumulator), then optionally the counted sketch (bytes + rows)."""
    t = api.build_cdbg_ext(dbank, k, None, ctx=ctx, counter_bits=16, cms_log2_width=log2w, subsample=subsample)
    check_rows(t, ref)
    t.release()
    old = ctx.get_tuning("acc_filter")
    ctx.set_tuning(acc_filter=0)
    try:
        t = api.build_cdbg_ext(dbank, k, None, ctx=ctx, counter_bits=16, cms_log2_width=log2w, subsample=subsample)
        assert not t.filtered()
        assert t.acc_digest() == ref["acc"], "accumulator (every KmerAcc) differs"
        check_rows(t, ref)
        t.release()
    finally:
        ctx.set_tuning(acc_filter=old)
    if keep_cms:
        t, cms = api.build_cdbg_ext(dbank, k, None, ctx=ctx, counter_bits=16, cms_log2_width=log2w, subsample=subsample,
                                    keep_cms=True)
        assert np.array_equal(cms.export(), ref["cms"].export()), "pass-1 sketch bytes differ"
        check_rows(t, ref)
        t.release()
        cms.release()


def test_plain_1mbp_bit_exact(ctx):
    wl = workloads.PLAIN_1MBP
    _, bank, _, sample, n_sample, stats = workloads.generate(wl)
    check_estimator(ctx, sample, n_sample, stats, wl["hll_p"])
    dbank = api.DeviceBank(ctx, bank)
    for k in wl["ks"]:
        ref = oracle_build(bank, k, wl["cms_log2w"])
        device_builds(ctx, dbank, k, wl["cms_log2w"], ref, keep_cms=True)
    dbank.release()


def test_isolate_5mbp_bit_exact(ctx):
    """The benchmark's workload and builds (the same default tuning it times)."""
    wl = workloads.ISOLATE_5MBP
    _, bank, _, sample, n_sample, stats = workloads.generate(wl)
    check_estimator(ctx, sample, n_sample, stats, wl["hll_p"])
    dbank = api.DeviceBank(ctx, bank)
    for k in wl["ks"]:
        ref = oracle_build(bank, k, wl["cms_log2w"])
        device_builds(ctx, dbank, k, wl["cms_log2w"], ref, keep_cms=(k == 77))
        del ref
    dbank.release()


def test_stress_12mbp_bit_exact(ctx):
    wl = workloads.STRESS_12MBP
    _, bank, _, sample, n_sample, stats = workloads.generate(wl)
    ge = check_estimator(ctx, sample, n_sample, stats, wl["hll_p"])
    dbank = api.DeviceBank(ctx, bank)
    k, log2w = wl["ks"][0], wl["cms_log2w"]
    ref = oracle_build(bank, k, log2w)
    device_builds(ctx, dbank, k, log2w, ref, keep_cms=True)
    del ref
    # subsampled to 110x by the pipeline driver's policy, from the estimate
    f, why = api.subsample_decide(api.subsample_policy(**workloads.SUBSAMPLE_110X), ge)
    assert f < 0.999, (f, why)
    ref = oracle_build(bank, k, log2w, keep_mask=keep_bits(int(stats.exact_read_pairs), f, 0))
    device_builds(ctx, dbank, k, log2w, ref, subsample=(f, 0))
    dbank.release()
