"""The allocation-free estimator entry point (fbk_estimate_sample_noalloc) agrees
exactly with fbk_estimate_sample on the same sample, on two calls in a row.

It exists for callers that cannot call cudaMalloc — hosts whose device memory belongs
to another runtime's allocator, or loops that must not take allocator locks — so it is
called here through the C ABI with host buffers only.  Requests beyond its fixed
scratch (pairs, bases, sketch width, HLL precision) are refused before any copy.  This
file is collected last so that a failure here does not stop the rest of the suite."""
import ctypes as C

import numpy as np
import pytest

from fastbact_gb300 import _native as N
from fastbact_gb300 import api

pytestmark = pytest.mark.gpu


def _sample(seed, genome_len, coverage, pairs):
    p = api.synth_params(seed=seed, genome_len=genome_len, coverage=coverage)
    bank, st, sample, n_sample, stats = api.synth_isolate(p, threads=0, sample_pairs=pairs)
    return sample, n_sample, stats


def _noalloc(sample, n_pairs, stats, **params):
    prm = api.estimator_params(**params)
    m = 1 << prm.hll_p
    rt, rs = np.zeros(m, np.uint8), np.zeros(m, np.uint8)
    e = N.GenomeEstimate()
    err = C.create_string_buffer(256)
    v = sample.view()
    cs = stats.to_c()
    st = N.lib().fbk_estimate_sample_noalloc(0, None, C.byref(v), n_pairs, C.byref(cs), C.byref(prm), C.byref(e),
                                            N.ptr(rt), N.ptr(rs), err, len(err))
    return st, api.GenomeEstimate.from_c(e), rt, rs, err.value.decode()


FIELDS = ("genome_size", "exact_read_pairs", "total_bases", "median_read_len", "max_read_len", "estimated_cov",
          "subsample_factor", "kmers", "confidence", "u_ge_1", "u_ge_2", "sample_kmer_depth", "pairs_sampled",
          "m_sample")


@pytest.mark.parametrize("seed,genome_len,coverage,pairs", [(5, 40_000, 150.0, 20_000), (6, 120_000, 30.0, 9_000)])
def test_noalloc_matches_estimate_sample_twice(seed, genome_len, coverage, pairs):
    sample, n_pairs, stats = _sample(seed, genome_len, coverage, pairs)
    params = dict(cms_log2_width=18, hll_p=14, max_pairs=250_000, target_cov=50.0)
    ctx = api.Context(0)
    try:
        ref, rt_ref, rs_ref = api.estimate_sample(ctx, sample, n_pairs, stats, **params)
    finally:
        ctx.close()
    for _ in range(2):  # the second call must not see the first call's scratch contents
        st, got, rt, rs, msg = _noalloc(sample, n_pairs, stats, **params)
        assert st == 0, msg
        for f in FIELDS:
            assert getattr(got, f) == getattr(ref, f), f
        assert np.array_equal(rt, rt_ref) and np.array_equal(rs, rs_ref)


def test_noalloc_rejects_oversized_requests():
    sample, n_pairs, stats = _sample(7, 30_000, 20.0, 2_000)
    st, _, _, _, msg = _noalloc(sample, n_pairs, stats, cms_log2_width=19)
    assert st == 1 and "cms_log2_width" in msg
    st, _, _, _, msg = _noalloc(sample, n_pairs, stats, hll_p=16)
    assert st == 1 and "hll_p" in msg


def test_noalloc_rejects_too_many_pairs():
    # 30000 pairs at 150x of a 60 kb genome: 25000 sampled pairs exceed the 20000 limit
    sample, n_pairs, stats = _sample(8, 60_000, 150.0, 25_000)
    assert n_pairs > 20_000
    st, _, _, _, msg = _noalloc(sample, n_pairs, stats, cms_log2_width=18, hll_p=14, max_pairs=250_000)
    assert st == 1 and "20000 sampled pairs" in msg


def test_noalloc_rejects_too_many_bases():
    # two pairs whose last read ends past base 2^23 (the sample's extent, not its
    # length, sizes the packed copy)
    n_words = ((1 << 23) + 256) // 32 + 1
    data = np.zeros(n_words, np.uint64)
    offsets = np.array([0, 100, 200, (1 << 23) + 10], np.uint64)
    lengths = np.array([100, 100, 100, 100], np.uint32)
    sample = api.BitSeqArena(data, offsets, lengths)
    stats = api.ExactCountStats(2, 200, 200, 400, 100, 100, 100.0, 100)
    st, _, _, _, msg = _noalloc(sample, 2, stats, cms_log2_width=18, hll_p=14, max_pairs=250_000)
    assert st == 1 and "2^23 sample bases" in msg
