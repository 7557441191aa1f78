"""Batches: every isolate of a multi-isolate batch gets exactly the results of the
single-isolate calls — the same GenomeEstimate, the same subsampling decision
(src/main.rs:84-180 with --enable-auto-subsample --depth 110 and a 150x trigger)
and the same SolidKmerNode table — whatever the wave sizes, with or without CUDA
graphs and the autotuner.  One isolate is also checked against the oracle."""
import numpy as np
import pytest

from fastbact_gb300 import api
from oracle import orc

pytestmark = pytest.mark.gpu

# seed, genome length, depth, GC: two isolates above 150x (subsampled to 110x), one
# at low coverage, the rest in between; genome sizes differ so waves are uneven.
SPECS = [
    (1000, 40_000, 30.0, 0.35),
    (1001, 80_000, 200.0, 0.62),
    (1002, 25_000, 90.0, 0.50),
    (1003, 60_000, 170.0, 0.45),
    (1004, 30_000, 12.0, 0.55),
]
POLICY = dict(enable_auto_subsample=True, depth=110.0, threshold_ratio=150.0 / 110.0)
K, LOG2W = 31, 18


@pytest.fixture(scope="module")
def isolates():
    out = []
    for seed, g, cov, gc in SPECS:
        p = api.synth_params(seed=seed, genome_len=g, coverage=cov, gc=gc)
        out.append(api.synth_isolate(p, threads=0, sample_pairs=150_000))
    return out


def single(ctx, iso):
    bank, _, sample, n_sample, cs = iso
    est, _, _ = api.estimate_sample(ctx, sample, n_sample, cs, max_pairs=250_000, target_cov=110.0)
    f, why = api.subsample_decide(api.subsample_policy(**POLICY), est)
    t = api.build_cdbg_ext(bank, K, None, ctx=ctx, key_bits=64, counter_bits=16, cms_log2_width=LOG2W, subsample=(f, 0))
    out = dict(est=est, factor=f, why=why, digest=t.digest(), info=t.info()[:2], rows=t.export(sort=True),
               filtered=t.filtered())
    t.release()
    return out


@pytest.fixture(scope="module")
def expected(ctx, isolates):
    return [single(ctx, iso) for iso in isolates]


def run_batch(ctx, isolates, **kw):
    b = api.Batch(ctx, api.batch_params(policy=api.subsample_policy(**POLICY), cms_log2_width=LOG2W, **kw))
    ids = [b.submit(bank, sample, n, cs) for bank, _, sample, n, cs in isolates]
    b.run()
    got = []
    for i in ids:
        r = b.result(i)
        t = b.take_table(i)
        got.append(dict(res=r, digest=t.digest(), info=t.info()[:2], rows=t.export(sort=True), filtered=t.filtered()))
        t.release()
    stats = b.stats()
    b.release()
    return got, stats


def check_same(got, expected):
    assert len(got) == len(expected)
    for g, e in zip(got, expected):
        r = g["res"]
        assert r.state == 3
        est = api.GenomeEstimate.from_c(r.estimate)
        assert est == e["est"]
        assert r.subsample_factor == e["factor"]
        assert api.SUBSAMPLE_REASONS[r.subsample_reason] == e["why"]
        assert g["digest"] == e["digest"]
        # SolidKmerNode rows are exact; the number of accumulated keys is exact too
        # unless a record filter kept some keys out (which ones depends on how the
        # path groups records into buckets)
        assert g["info"][1] == e["info"][1] and r.n_solid == e["info"][1]
        if not (g["filtered"] or e["filtered"]):
            assert g["info"] == e["info"] and r.n_keys == e["info"][0]
        for a, b in zip(g["rows"], e["rows"]):
            assert np.array_equal(a, b)


def test_policy_subsamples_the_deep_isolates(expected):
    why = [e["why"] for e in expected]
    assert why[1] == why[3] == "AUTO_SUBSAMPLE_HIGH_CONFIDENCE"
    assert expected[1]["factor"] < 0.7 and expected[3]["factor"] < 0.8
    assert expected[0]["factor"] == expected[2]["factor"] == 1.0


def test_batch_graphs_autotuned_matches_single(ctx, isolates, expected):
    got, st = run_batch(ctx, isolates, use_graphs=1, autotune=1)
    check_same(got, expected)
    assert st.isolates_done == len(isolates) and st.tuned == 1 and st.graph_launches >= 2


def test_batch_streams_small_waves_matches_single(ctx, isolates, expected):
    got, st = run_batch(ctx, isolates, use_graphs=0, autotune=0, max_wave=2)
    check_same(got, expected)
    assert st.waves == 3 and st.graph_launches == 0


def test_batch_memory_limited_waves_match_single(ctx, isolates, expected):
    # a 1 MB wave budget: one isolate per phase-A wave and per phase-B sub-wave
    got, st = run_batch(ctx, isolates, use_graphs=1, autotune=0, max_wave_bytes=1 << 20)
    check_same(got, expected)
    assert st.waves == len(isolates)


def test_batch_isolate_matches_oracle(ctx, isolates, expected):
    bank, _, _, _, _ = isolates[3]
    f = expected[3]["factor"]
    n_pairs = int(max(int(a.pair_idx.max()) for a in bank.arenas if len(a)) + 1)
    keep = api.subsample_mask(ctx, n_pairs, f, 0)
    _, o_tab, _, mtc = orc.build_front(bank, K, 64, LOG2W, 16, None, threads=4, keep_mask=keep)
    okeys, ocov, omask = api.sort_rows(*o_tab.export_solid(mtc))
    keys, cov, mask = expected[3]["rows"]
    assert np.array_equal(keys, okeys) and np.array_equal(cov, ocov) and np.array_equal(mask, omask)
    got, _ = run_batch(ctx, [isolates[3]], use_graphs=1, autotune=0)
    assert got[0]["digest"][0] == o_tab.digest(mtc)[0]
